/*
 * bp_oracle_impl.h -- type-generic body of the CPU oracle (included by bp_oracle.c
 * once per element type).  TEST INFRASTRUCTURE ONLY: nothing in the product path
 * links, imports or executes this code; it exists to check the GPU library.
 *
 * Before inclusion the includer defines
 *   T          element type (double, float, double _Complex)
 *   SUF        function-name suffix (f64, f32, c128)
 *   CONJ(x)    complex conjugate (identity for real types)
 *   ABS2(x)    |x|^2 as double
 *   REALP(x)   real part as double
 *   IMAGP(x)   imaginary part as double
 *   IS_COMPLEX 0/1
 *
 * Every routine restates one reference routine; the citation is on each function.
 */

#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SUF)

/* ---- elementary contractions ------------------------------------------------------ */

/* Two-layer absorption of message m (D x D, row-major [bra][ket]) into the ket leg w
 * of T viewed as [outer][D][inner]:  out[o][b][i] = sum_k in[o][k][i] * m[b][k].
 * This is the pairwise contraction ITensorBase performs when contract_network
 * (contract_network.jl:32-37) multiplies an incoming message into the factor
 * lazy(A) * lazy(conj(B)) (normnetwork.jl:49-54). */
static void FN(absorb2)(const T *in, T *out, int64_t outer, int64_t D, int64_t inner,
                        const T *m) {
  for (int64_t o = 0; o < outer; ++o) {
    for (int64_t b = 0; b < D; ++b) {
      T *dst = out + (o * D + b) * inner;
      for (int64_t i = 0; i < inner; ++i) dst[i] = 0;
      for (int64_t k = 0; k < D; ++k) {
        const T mk = m[b * D + k];
        const T *src = in + (o * D + k) * inner;
        for (int64_t i = 0; i < inner; ++i) dst[i] += src[i] * mk;
      }
    }
  }
}

/* Single-layer absorption of a vector message: out[o][i] = sum_k in[o][k][i] * m[k]. */
static void FN(absorb1)(const T *in, T *out, int64_t outer, int64_t D, int64_t inner,
                        const T *m) {
  for (int64_t o = 0; o < outer; ++o) {
    T *dst = out + o * inner;
    for (int64_t i = 0; i < inner; ++i) dst[i] = 0;
    for (int64_t k = 0; k < D; ++k) {
      const T mk = m[k];
      const T *src = in + (o * D + k) * inner;
      for (int64_t i = 0; i < inner; ++i) dst[i] += src[i] * mk;
    }
  }
}

/* ---- one message update (beliefpropagation.jl:242-257) ------------------------------ */

/* Computes the message on directed slot `slot` (u -> nbr) from the incoming messages
 * of u other than the reverse one (incoming_messages, messagecache.jl:128-131),
 * contracted with the factor of u, then divides by sum(entries) when it is non-zero
 * (beliefpropagation.jl:248-253).  msg_in is read, out receives the message.
 * buf0/buf1 hold at least toff[u+1]-toff[u] elements each. */
static int FN(update_one)(const orc_graph *g, const T *tens, const T *msg_in, T *out,
                          int64_t slot, int normalize, T *buf0, T *buf1) {
  /* locate u and the leg of this slot */
  int64_t lo = 0, hi = g->nv;
  while (hi - lo > 1) {
    int64_t mid = (lo + hi) / 2;
    if (g->off[mid] <= slot) lo = mid; else hi = mid;
  }
  const int64_t u = lo;
  const int64_t z = g->off[u + 1] - g->off[u];
  const int64_t v = slot - g->off[u];
  const T *A = tens + g->toff[u];
  int64_t dims[ORC_MAX_LEGS];
  for (int64_t l = 0; l < z; ++l) dims[l] = g->bond[g->off[u] + l];
  const int64_t d = g->phys[u];
  int64_t n = d;
  for (int64_t l = 0; l < z; ++l) n *= dims[l];
  if (g->layers == 2) {
    memcpy(buf0, A, (size_t)n * sizeof(T));
    T *cur = buf0, *nxt = buf1;
    for (int64_t w = 0; w < z; ++w) {
      if (w == v) continue;
      int64_t inner = 1, outer = d;
      for (int64_t l = w + 1; l < z; ++l) inner *= dims[l];
      for (int64_t l = 0; l < w; ++l) outer *= dims[l];
      const T *m = msg_in + g->moff[g->rev[g->off[u] + w]];
      FN(absorb2)(cur, nxt, outer, dims[w], inner, m);
      T *t = cur; cur = nxt; nxt = t;
    }
    /* out[b][k] = sum_{o,i} cur[o][k][i] * conj(A[o][b][i])  (leg v open on both layers) */
    int64_t inner = 1, outer = d;
    for (int64_t l = v + 1; l < z; ++l) inner *= dims[l];
    for (int64_t l = 0; l < v; ++l) outer *= dims[l];
    const int64_t Dv = dims[v];
    for (int64_t b = 0; b < Dv; ++b)
      for (int64_t k = 0; k < Dv; ++k) {
        T acc = 0;
        for (int64_t o = 0; o < outer; ++o) {
          const T *tc = cur + (o * Dv + k) * inner;
          const T *ac = A + (o * Dv + b) * inner;
          for (int64_t i = 0; i < inner; ++i) acc += tc[i] * CONJ(ac[i]);
        }
        out[b * Dv + k] = acc;
      }
    if (normalize) {
      T s = 0;
      for (int64_t j = 0; j < Dv * Dv; ++j) s += out[j];
      if (s != 0)
        for (int64_t j = 0; j < Dv * Dv; ++j) out[j] /= s;
    }
  } else {
    if (d != 1) return ORC_ERR_ARG;
    memcpy(buf0, A, (size_t)n * sizeof(T));
    T *cur = buf0, *nxt = buf1;
    int64_t cdims[ORC_MAX_LEGS];
    int64_t cz = z, vpos = v;
    for (int64_t l = 0; l < z; ++l) cdims[l] = dims[l];
    int64_t orig[ORC_MAX_LEGS];
    for (int64_t l = 0; l < z; ++l) orig[l] = l;
    /* absorb every leg except v; the tensor shrinks by one leg per absorption */
    for (int64_t w = 0; w < z; ++w) {
      if (w == v) continue;
      int64_t pos = -1;
      for (int64_t l = 0; l < cz; ++l) if (orig[l] == w) pos = l;
      int64_t inner = 1, outer = 1;
      for (int64_t l = pos + 1; l < cz; ++l) inner *= cdims[l];
      for (int64_t l = 0; l < pos; ++l) outer *= cdims[l];
      const T *m = msg_in + g->moff[g->rev[g->off[u] + w]];
      FN(absorb1)(cur, nxt, outer, cdims[pos], inner, m);
      for (int64_t l = pos; l + 1 < cz; ++l) { cdims[l] = cdims[l + 1]; orig[l] = orig[l + 1]; }
      --cz;
      T *t = cur; cur = nxt; nxt = t;
    }
    (void)vpos;
    const int64_t Dv = dims[v];
    for (int64_t k = 0; k < Dv; ++k) out[k] = cur[k];
    if (normalize) {
      T s = 0;
      for (int64_t k = 0; k < Dv; ++k) s += out[k];
      if (s != 0)
        for (int64_t k = 0; k < Dv; ++k) out[k] /= s;
    }
  }
  return ORC_OK;
}

static int64_t FN(max_tensor)(const orc_graph *g) {
  int64_t mx = 1;
  for (int64_t u = 0; u < g->nv; ++u) {
    int64_t n = g->toff[u + 1] - g->toff[u];
    if (n > mx) mx = n;
  }
  return mx;
}

static int FN(check_graph)(const orc_graph *g) {
  if (g->layers != 1 && g->layers != 2) return ORC_ERR_ARG;
  for (int64_t u = 0; u < g->nv; ++u)
    if (g->off[u + 1] - g->off[u] > ORC_MAX_LEGS) return ORC_ERR_ARG;
  return ORC_OK;
}

/* Reference message_update!(alg, cache, factors, edge): one in-place update. */
int FN(orc_message_update)(const orc_graph *g, const T *tens, T *msgs, int64_t slot,
                           int normalize) {
  if (FN(check_graph)(g)) return ORC_ERR_ARG;
  const int64_t nslots = g->off[g->nv];
  if (slot < 0 || slot >= nslots) return ORC_ERR_ARG;
  const int64_t mx = FN(max_tensor)(g);
  T *b0 = (T *)malloc((size_t)mx * sizeof(T));
  T *b1 = (T *)malloc((size_t)mx * sizeof(T));
  T *out = (T *)malloc((size_t)(g->moff[slot + 1] - g->moff[slot]) * sizeof(T));
  int st = FN(update_one)(g, tens, msgs, out, slot, normalize, b0, b1);
  if (!st)
    memcpy(msgs + g->moff[slot], out, (size_t)(g->moff[slot + 1] - g->moff[slot]) * sizeof(T));
  free(b0); free(b1); free(out);
  return st;
}

/* AIE.iterate_diff for MessageCache (beliefpropagation.jl:261-267):
 * max over directed edges of 1 - |<m1/|m1|, m2/|m2|>|^2.  NaN propagates. */
double FN(orc_iterate_diff)(int64_t nslots, const int64_t *moff, const T *m1, const T *m2) {
  double mx = -INFINITY;
  int saw_nan = 0;
  for (int64_t s = 0; s < nslots; ++s) {
    double n1 = 0, n2 = 0;
    double dre = 0, dim = 0;
    for (int64_t j = moff[s]; j < moff[s + 1]; ++j) {
      n1 += ABS2(m1[j]);
      n2 += ABS2(m2[j]);
      T p = CONJ(m1[j]) * m2[j];
      dre += REALP(p);
      dim += IMAGP(p);
    }
    double val = 1.0 - (dre * dre + dim * dim) / (n1 * n2);
    if (val != val) saw_nan = 1;
    else if (val > mx) mx = val;
  }
  return saw_nan ? NAN : mx;
}

/* One parallel (Jacobi) sweep: every directed slot recomputed from msg_in into msg_out.
 * The reference only has the sequential sweep (beliefpropagation.jl:200-210); the
 * Jacobi sweep applies the same update (beliefpropagation.jl:242-257) to all edges
 * against the previous iterate. */
static int FN(sweep_parallel)(const orc_graph *g, const T *tens, const T *msg_in, T *msg_out,
                              int normalize, int nthreads) {
  const int64_t nslots = g->off[g->nv];
  const int64_t mx = FN(max_tensor)(g);
  int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
#endif
  {
    T *b0 = (T *)malloc((size_t)mx * sizeof(T));
    T *b1 = (T *)malloc((size_t)mx * sizeof(T));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
    for (int64_t s = 0; s < nslots; ++s) {
      int st = FN(update_one)(g, tens, msg_in, msg_out + g->moff[s], s, normalize, b0, b1);
      if (st) err = st;
    }
    free(b0); free(b1);
  }
  (void)nthreads;
  return err;
}

/* Sequential (Gauss-Seidel) sweep over `edges` in order, updating in place
 * (BeliefPropagationSweep, beliefpropagation.jl:200-210). */
static int FN(sweep_sequential)(const orc_graph *g, const T *tens, T *msgs, const int64_t *edges,
                                int64_t n_edges, int normalize) {
  const int64_t mx = FN(max_tensor)(g);
  T *b0 = (T *)malloc((size_t)mx * sizeof(T));
  T *b1 = (T *)malloc((size_t)mx * sizeof(T));
  int64_t mmax = 1;
  for (int64_t s = 0; s < g->off[g->nv]; ++s)
    if (g->moff[s + 1] - g->moff[s] > mmax) mmax = g->moff[s + 1] - g->moff[s];
  T *out = (T *)malloc((size_t)mmax * sizeof(T));
  int err = 0;
  for (int64_t e = 0; e < n_edges && !err; ++e) {
    const int64_t s = edges[e];
    err = FN(update_one)(g, tens, msgs, out, s, normalize, b0, b1);
    if (!err) memcpy(msgs + g->moff[s], out, (size_t)(g->moff[s + 1] - g->moff[s]) * sizeof(T));
  }
  free(b0); free(b1); free(out);
  return err;
}

/* beliefpropagation(factors, messages; edges, stopping_criterion) (beliefpropagation.jl:69-92)
 * with the outer loop of AI.solve and StopAfterIteration(maxiter) | StopWhenConverged(tol)
 * (beliefpropagation.jl:27-55; AlgorithmsInterfaceExtensions.jl:73-118):
 *   before every outer step the criterion is evaluated; StopWhenConverged computes
 *   iterate_diff against the previous iterate, stores a copy, skips iteration 0 and
 *   fires when delta < tol.  maxiter < 0 means "not given"; tol < 0 means "not given".
 * msgs is updated in place.  schedule 0 = parallel (Jacobi), 1 = sequential over edges. */
int FN(orc_bp_run)(const orc_graph *g, const T *tens, T *msgs, int schedule,
                   const int64_t *edges, int64_t n_edges, int maxiter, double tol,
                   int normalize, int nthreads, int *out_iters, double *out_delta,
                   int *out_at_iter) {
  if (FN(check_graph)(g)) return ORC_ERR_ARG;
  if (maxiter < 0 && !(tol >= 0)) return ORC_ERR_ARG;
  const int64_t nslots = g->off[g->nv];
  const int64_t mtot = g->moff[nslots];
  T *prev = (T *)malloc((size_t)(mtot > 0 ? mtot : 1) * sizeof(T));
  T *tmp = (T *)malloc((size_t)(mtot > 0 ? mtot : 1) * sizeof(T));
  const int use_tol = tol >= 0;
  memcpy(prev, msgs, (size_t)mtot * sizeof(T));
  int iter = 0, at_iter = -1, err = 0;
  double delta = INFINITY;
  for (;;) {
    if (maxiter >= 0 && iter >= maxiter) break;
    if (use_tol) {
      double dl = FN(orc_iterate_diff)(nslots, g->moff, msgs, prev);
      memcpy(prev, msgs, (size_t)mtot * sizeof(T));
      if (iter > 0) {
        delta = dl;
        if (dl < tol) { at_iter = iter; break; }
      }
    }
    ++iter;
    if (schedule == 0) {
      err = FN(sweep_parallel)(g, tens, msgs, tmp, normalize, nthreads);
      memcpy(msgs, tmp, (size_t)mtot * sizeof(T));
    } else {
      err = FN(sweep_sequential)(g, tens, msgs, edges, n_edges, normalize);
    }
    if (err) break;
  }
  free(prev); free(tmp);
  if (out_iters) *out_iters = iter;
  if (out_delta) *out_delta = delta;
  if (out_at_iter) *out_at_iter = at_iter;
  return err;
}

/* Fixed number of parallel sweeps without the convergence test (the timed CPU
 * baseline workload). */
int FN(orc_bp_sweeps)(const orc_graph *g, const T *tens, T *msgs, int nsweeps, int normalize,
                      int nthreads) {
  if (FN(check_graph)(g)) return ORC_ERR_ARG;
  const int64_t mtot = g->moff[g->off[g->nv]];
  T *tmp = (T *)malloc((size_t)(mtot > 0 ? mtot : 1) * sizeof(T));
  int err = 0;
  for (int it = 0; it < nsweeps && !err; ++it) {
    err = FN(sweep_parallel)(g, tens, msgs, tmp, normalize, nthreads);
    memcpy(msgs, tmp, (size_t)mtot * sizeof(T));
  }
  free(tmp);
  return err;
}

/* log of a scalar as (re, im); real types promote like `complex.(x)` does in
 * bethe_free_energy (messagecache.jl:189-194): log(-x) = log(x) + i*pi. */
static void FN(clog2)(T zv, double *re, double *im) {
#if IS_COMPLEX
  double a = REALP(zv), b = IMAGP(zv);
  *re = 0.5 * log(a * a + b * b);
  *im = atan2(b, a);
#else
  double a = (double)zv;
  if (a < 0) { *re = log(-a); *im = M_PI; }
  else { *re = log(a); *im = 0.0; }
#endif
}

/* vertex_scalar (messagecache.jl:139-143): full contraction of the factor of u with all
 * of its incoming messages (incoming_edge_data, messagecache.jl:134-137). */
static T FN(vertex_scalar_one)(const orc_graph *g, const T *tens, const T *msgs, int64_t u,
                               T *buf0, T *buf1) {
  const int64_t z = g->off[u + 1] - g->off[u];
  const T *A = tens + g->toff[u];
  int64_t dims[ORC_MAX_LEGS];
  for (int64_t l = 0; l < z; ++l) dims[l] = g->bond[g->off[u] + l];
  const int64_t d = g->phys[u];
  int64_t n = d;
  for (int64_t l = 0; l < z; ++l) n *= dims[l];
  memcpy(buf0, A, (size_t)n * sizeof(T));
  T *cur = buf0, *nxt = buf1;
  if (g->layers == 2) {
    for (int64_t w = 0; w < z; ++w) {
      int64_t inner = 1, outer = d;
      for (int64_t l = w + 1; l < z; ++l) inner *= dims[l];
      for (int64_t l = 0; l < w; ++l) outer *= dims[l];
      FN(absorb2)(cur, nxt, outer, dims[w], inner, msgs + g->moff[g->rev[g->off[u] + w]]);
      T *t = cur; cur = nxt; nxt = t;
    }
    T acc = 0;
    for (int64_t j = 0; j < n; ++j) acc += cur[j] * CONJ(A[j]);
    return acc;
  } else {
    int64_t cz = z;
    int64_t cdims[ORC_MAX_LEGS];
    for (int64_t l = 0; l < z; ++l) cdims[l] = dims[l];
    /* absorb the last remaining leg each time (leg w = cz-1 keeps the CSR order) */
    for (int64_t w = z - 1; w >= 0; --w) {
      int64_t outer = 1;
      for (int64_t l = 0; l < w; ++l) outer *= cdims[l];
      FN(absorb1)(cur, nxt, outer * d, cdims[w], 1, msgs + g->moff[g->rev[g->off[u] + w]]);
      --cz;
      T *t = cur; cur = nxt; nxt = t;
    }
    T acc = 0;
    for (int64_t j = 0; j < d; ++j) acc += cur[j];
    return acc;
  }
}

/* edge_scalar (messagecache.jl:153-157): contract m(u->v) with m(v->u) over both
 * names, no conjugation. */
static T FN(edge_scalar_one)(const orc_graph *g, const T *msgs, int64_t slot) {
  const T *a = msgs + g->moff[slot];
  const T *b = msgs + g->moff[g->rev[slot]];
  T acc = 0;
  for (int64_t j = 0; j < g->moff[slot + 1] - g->moff[slot]; ++j) acc += a[j] * b[j];
  return acc;
}

/* vertex_scalars / edge_scalars / bethe_free_energy (messagecache.jl:145-201).
 * zv_out: nv raw scalars (as T), ze_out: one per undirected edge (slot < rev[slot]),
 * logzv/logze: (re, im) pairs, total: (re, im) of sum log Zv - sum log Ze,
 * flags[0] = any real(Zv) < 0, flags[1] = any real(Ze) < 0, flags[2] = any Ze == 0. */
int FN(orc_logscalars)(const orc_graph *g, const T *tens, const T *msgs, T *zv_out,
                       T *ze_out, double *logzv, double *logze, double *total, int *flags) {
  if (FN(check_graph)(g)) return ORC_ERR_ARG;
  const int64_t mx = FN(max_tensor)(g);
  T *b0 = (T *)malloc((size_t)mx * sizeof(T));
  T *b1 = (T *)malloc((size_t)mx * sizeof(T));
  double sre = 0, sim = 0;
  flags[0] = flags[1] = flags[2] = 0;
  for (int64_t u = 0; u < g->nv; ++u) {
    T zv = FN(vertex_scalar_one)(g, tens, msgs, u, b0, b1);
    if (zv_out) zv_out[u] = zv;
    if (REALP(zv) < 0) flags[0] = 1;
    double re, im;
    FN(clog2)(zv, &re, &im);
    if (logzv) { logzv[2 * u] = re; logzv[2 * u + 1] = im; }
    sre += re; sim += im;
  }
  int64_t ne = 0;
  for (int64_t s = 0; s < g->off[g->nv]; ++s) {
    if (s > g->rev[s]) continue;
    T ze = FN(edge_scalar_one)(g, msgs, s);
    if (ze_out) ze_out[ne] = ze;
    if (REALP(ze) < 0) flags[1] = 1;
    if (REALP(ze) == 0 && IMAGP(ze) == 0) flags[2] = 1;
    double re, im;
    FN(clog2)(ze, &re, &im);
    if (logze) { logze[2 * ne] = re; logze[2 * ne + 1] = im; }
    sre -= re; sim -= im;
    ++ne;
  }
  total[0] = sre; total[1] = sim;
  free(b0); free(b1);
  return ORC_OK;
}

#undef FN
#undef CAT
#undef CAT2
