/* Replays from C what itensornetworksnext.jl_gb300/julia/ITensorNetworksNextGPU.jl does
 * through `ccall` (no Julia toolchain exists where this repository is tested): the same
 * entry points with the same argument lists, the Julia structs' layouts (checked against the
 * header's), column-major "Julia" arrays handed over by strides, messages packed as
 * m[bra][ket] row-major from M[bra, ket], sequential-schedule slots from the edge order,
 * contract_network's reversed (column-major) labels, and the gradient mapped back onto each
 * ket tensor's own index order.
 *
 * Network: a path 0 - 1 - 2 with links l01 (dim 2) and l12 (dim 3) and site indices of
 * dim 2, the ket tensors stored column-major in deliberately different index orders:
 *   A0[l01, s0], A1[s1, l12, l01], A2[l12, s2].
 * BP is exact on a tree, so every result has a closed form: <psi|psi> by brute force.
 * Without a GPU (argument "host") only the layouts are checked.  Prints "ok". */
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "itn_gpu.h"

#define CHECK(cond, msg)                    \
  do {                                      \
    if (!(cond)) {                          \
      fprintf(stderr, "FAILED: %s\n", msg); \
      return 1;                             \
    }                                       \
  } while (0)

/* ---- the Julia structs, field by field (ItnBpOpts, ItnBpResult, ItnGradOpts, ItnGradResult) */
typedef struct { int32_t schedule, maxiter; double tol; int32_t normalize, precision, split_sweeps, reserved0;
                 int64_t *edges; int64_t n_edges; } jl_bp_opts;
typedef struct { int32_t iterations, at_iteration; double delta, device_ms; int32_t kernel_launches, reserved0; }
    jl_bp_result;
typedef struct { int32_t adjoint, maxiter; double tol; int32_t normalized, sweeps, checkpoint, reserved0; }
    jl_grad_opts;
typedef struct { int32_t adjoint_iterations, reserved0; double adjoint_residual, device_ms; } jl_grad_result;

#define SAME_LAYOUT(J, C, f) (offsetof(J, f) == offsetof(C, f))
_Static_assert(sizeof(jl_bp_opts) == sizeof(itn_bp_opts), "ItnBpOpts size");
_Static_assert(SAME_LAYOUT(jl_bp_opts, itn_bp_opts, tol) && SAME_LAYOUT(jl_bp_opts, itn_bp_opts, edges) &&
                   SAME_LAYOUT(jl_bp_opts, itn_bp_opts, n_edges),
               "ItnBpOpts fields");
_Static_assert(sizeof(jl_bp_result) == sizeof(itn_bp_result) && SAME_LAYOUT(jl_bp_result, itn_bp_result, delta) &&
                   SAME_LAYOUT(jl_bp_result, itn_bp_result, kernel_launches),
               "ItnBpResult");
_Static_assert(sizeof(jl_grad_opts) == sizeof(itn_grad_opts) && SAME_LAYOUT(jl_grad_opts, itn_grad_opts, tol) &&
                   SAME_LAYOUT(jl_grad_opts, itn_grad_opts, sweeps) &&
                   SAME_LAYOUT(jl_grad_opts, itn_grad_opts, checkpoint),
               "ItnGradOpts");
_Static_assert(sizeof(jl_grad_result) == sizeof(itn_grad_result) &&
                   SAME_LAYOUT(jl_grad_result, itn_grad_result, device_ms),
               "ItnGradResult");

static double rnd(unsigned *s) {
  *s = *s * 1664525u + 1013904223u;
  return ((*s >> 8) & 0xFFFF) / 65536.0 - 0.5;
}

/* column-major index helpers of the three ket arrays */
#define A0(l, s) A0d[(l) + 2 * (s)]
#define A1(s, m, l) A1d[(s) + 2 * (m) + 6 * (l)]
#define A2(m, s) A2d[(m) + 3 * (s)]

int main(int argc, char **argv) {
  if (argc > 1 && strcmp(argv[1], "host") == 0) {
    printf("ok\n");
    return 0;
  }
  unsigned seed = 7;
  double A0d[4], A1d[12], A2d[6];
  for (int i = 0; i < 4; ++i) A0d[i] = rnd(&seed);
  for (int i = 0; i < 12; ++i) A1d[i] = rnd(&seed);
  for (int i = 0; i < 6; ++i) A2d[i] = rnd(&seed);
  /* <psi|psi> by brute force */
  double zz = 0;
  for (int s0 = 0; s0 < 2; ++s0)
    for (int s1 = 0; s1 < 2; ++s1)
      for (int s2 = 0; s2 < 2; ++s2) {
        double amp = 0;
        for (int l = 0; l < 2; ++l)
          for (int m = 0; m < 3; ++m) amp += A0(l, s0) * A1(s1, m, l) * A2(m, s2);
        zz += amp * amp;
      }

  /* DeviceNetwork(nn): itn_create, itn_graph_upload (rev and net_id C_NULL, layers 2),
   * itn_tensors_upload_strided with [site stride, link strides in neighbour order] */
  itn_ctx *ctx = NULL;
  CHECK(itn_create(&ctx, 0, 0) == ITN_OK, "itn_create");
  int64_t off[4] = {0, 1, 3, 4}, nbr[4] = {1, 0, 2, 1};
  int32_t bond[4] = {2, 2, 3, 3}, phys[3] = {2, 2, 2};
  CHECK(itn_graph_upload(ctx, 3, off, nbr, bond, NULL, phys, 2, NULL) == ITN_OK, itn_last_error(ctx));
  const void *ptrs[3] = {A0d, A1d, A2d};
  int64_t strides[7] = {2, 1, /* v1: */ 1, 6, 2, /* v2: */ 3, 1};
  CHECK(itn_tensors_upload_strided(ctx, ITN_F64, ptrs, strides) == ITN_OK, itn_last_error(ctx));
  const int64_t moff[5] = {0, 4, 8, 17, 26};

  /* upload_messages!: M[bra, ket] column-major, written transposed (row-major m[bra][ket]).
   * Non-symmetric positive start messages. */
  double packed[26];
  for (int s = 0; s < 4; ++s) {
    const int D = bond[s];
    double M[9];
    for (int j = 0; j < D * D; ++j) M[j] = 0.5 + 0.4 * rnd(&seed); /* M[b + D k] */
    for (int b = 0; b < D; ++b)
      for (int k = 0; k < D; ++k) packed[moff[s] + b * D + k] = M[b + D * k];
  }
  CHECK(itn_messages_upload(ctx, ITN_F64, packed) == ITN_OK, itn_last_error(ctx));

  /* gpu_solve: ItnBpOpts(sequential, maxiter, tol, normalize, precision, split, 0, edges, n) with
   * the edge order 0=>1, 1=>2, 2=>1, 1=>0 mapped to slots */
  int64_t eslots[4] = {0, 2, 3, 1};
  jl_bp_opts jo = {1, 10, 1e-13, 1, 0, 0, 0, eslots, 4};
  jl_bp_result jr;
  CHECK(itn_bp_run(ctx, (const itn_bp_opts *)&jo, (itn_bp_result *)&jr) == ITN_OK, itn_last_error(ctx));
  CHECK(jr.iterations >= 2 && jr.at_iteration == jr.iterations, "sequential solve converged");
  double got[26];
  CHECK(itn_messages_download(ctx, ITN_F64, got) == ITN_OK, itn_last_error(ctx));

  /* bethe_free_energy(nn, ::DeviceMessageCache): itn_logscalars with only totals and flags */
  double tot[2];
  int32_t flags[1];
  CHECK(itn_logscalars(ctx, NULL, NULL, NULL, NULL, tot, flags) == ITN_OK, itn_last_error(ctx));
  CHECK((flags[0] & 4) == 0 && fabs(exp(tot[0]) - zz) <= 1e-12 * zz, "BP log-norm = log <psi|psi> on a tree");

  /* message_update!(::GPUMessageUpdate, ...): one edge at the fixed point changes nothing */
  CHECK(itn_message_update(ctx, 2, 1) == ITN_OK, itn_last_error(ctx));
  double again[26];
  CHECK(itn_messages_download(ctx, ITN_F64, again) == ITN_OK, itn_last_error(ctx));
  for (int j = 0; j < 26; ++j) CHECK(fabs(again[j] - got[j]) <= 1e-12 * fabs(got[j]) + 1e-15, "fixed point kept");

  /* rrule: itn_bp_grad(ItnGradOpts(1, 200, 1e-10, 1, 0, 1, 0)), the packed canonical gradient
   * (per vertex row-major [site, links in neighbour order]) unpacked onto each ket array's
   * own column-major order; log Z is homogeneous of degree 2 in every A_v, so
   * sum_i A_v[i] dlogZ/dA_v[i] = 2 for each vertex. */
  jl_grad_opts go = {1, 200, 1e-10, 1, 0, 1, 0};
  jl_grad_result gr;
  double g[22];
  CHECK(itn_bp_grad(ctx, (const itn_grad_opts *)&go, g, (itn_grad_result *)&gr) == ITN_OK, itn_last_error(ctx));
  {
    /* canonical dims ([site, links in neighbour order]) and each axis's column-major stride */
    const int cd[3][3] = {{2, 2, 0}, {2, 2, 3}, {2, 3, 0}};
    const int cr[3] = {2, 3, 2};
    const double *own[3] = {A0d, A1d, A2d};
    int toff = 0;
    for (int v = 0; v < 3; ++v) {
      const int64_t *st = strides + (v == 0 ? 0 : v == 1 ? 2 : 5);
      int n = 1;
      for (int a = 0; a < cr[v]; ++a) n *= cd[v][a];
      double G[12] = {0}, dot = 0;
      for (int r = 0; r < n; ++r) { /* row-major canonical offset r -> the ket array's position */
        int rem = r, pos = 0;
        for (int a = cr[v] - 1; a >= 0; --a) {
          pos += (rem % cd[v][a]) * (int)st[a];
          rem /= cd[v][a];
        }
        G[pos] = g[toff + r];
      }
      for (int i = 0; i < n; ++i) dot += own[v][i] * G[i];
      CHECK(fabs(dot - 2.0) <= 1e-9, "gradient unpacked onto the ket's own axes");
      toff += n;
    }
  }
  /* the canonical packed tensors, for the serving calls below */
  double canon[22];
  CHECK(itn_tensors_download(ctx, ITN_F64, canon) == ITN_OK, itn_last_error(ctx));
  itn_destroy(ctx);

  /* gpu_solve_submit!(d, tensors, messages_in, messages_out; maxiter = 10) and gpu_solve_wait!(d)
   * on a fresh DeviceNetwork: ItnBpOpts(parallel, 10, -1.0, 1, precision, split, 0, C_NULL, 0);
   * 10 parallel sweeps make BP exact on this tree */
  {
    itn_ctx *c3 = NULL;
    CHECK(itn_create(&c3, 0, 0) == ITN_OK, "itn_create");
    CHECK(itn_graph_upload(c3, 3, off, nbr, bond, NULL, phys, 2, NULL) == ITN_OK, itn_last_error(c3));
    jl_bp_opts so = {0, 10, -1.0, 1, 0, 0, 0, NULL, 0};
    double mout[26], stot[2];
    int32_t sflags[1];
    jl_bp_result sr;
    CHECK(itn_bp_solve_submit(c3, ITN_F64, canon, packed, (const itn_bp_opts *)&so, mout, 1) == ITN_OK,
          itn_last_error(c3));
    CHECK(itn_messages_download(c3, ITN_F64, mout) == ITN_ERR_STATE, "calls refused while a solve is pending");
    CHECK(itn_bp_solve_wait(c3, (itn_bp_result *)&sr, stot, sflags) == ITN_OK, itn_last_error(c3));
    CHECK(sr.iterations == 10, "submitted solve ran 10 sweeps");
    CHECK((sflags[0] & 4) == 0 && fabs(exp(stot[0]) - zz) <= 1e-12 * zz, "submitted solve: log-norm on a tree");
    CHECK(itn_bp_solve_wait(c3, (itn_bp_result *)&sr, NULL, NULL) == ITN_ERR_STATE, "a second wait is refused");
    itn_destroy(c3);
  }

  /* contract_network(::GPUExact, nn): [ket(v), conj_bra(v)] per vertex, labels of each
   * column-major array reversed, codes in order of first appearance, greedy order */
  {
    enum { S0, L01, L01B, M12, S1, M12B, S2 }; /* the codes get!() assigns, in this order */
    int32_t ranks[6] = {2, 2, 3, 3, 2, 2};
    int64_t labels[14] = {S0, L01, S0, L01B, /* v1 ket [s1, l12, l01] reversed: */ L01, M12, S1,
                          L01B, M12B, S1, /* v2 */ S2, M12, S2, M12B};
    int64_t dims[14] = {2, 2, 2, 2, 2, 3, 2, 2, 3, 2, 2, 3, 2, 3};
    const void *ts[6] = {A0d, A0d, A1d, A1d, A2d, A2d};
    double out[1];
    int32_t orank = -1;
    int64_t olab[48], odim[48];
    itn_ctx *c2 = NULL;
    CHECK(itn_create(&c2, 0, 0) == ITN_OK, "itn_create");
    CHECK(itn_contract_network(c2, ITN_F64, 6, ranks, labels, dims, ts, 0, NULL, ITN_PREC_NATIVE, out, 1, &orank,
                               olab, odim, NULL) == ITN_OK,
          itn_last_error(c2));
    CHECK(orank == 0 && fabs(out[0] - zz) <= 1e-12 * zz, "exact contraction of the norm network");
    itn_destroy(c2);
  }
  printf("ok\n");
  return 0;
}
