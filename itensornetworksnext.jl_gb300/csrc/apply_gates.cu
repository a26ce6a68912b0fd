// apply_gates.cu -- BP simple-update gate application on the GPU, one CTA per gate.
//
// Follows apply_gate_bp! (src/apply/apply_operators.jl:209-283).  All arithmetic is FP64
// (complex128 for complex networks) on CUDA cores: the matrices are small (Gram and theta
// matrices of at most 128 x 128) and the work is dominated by synchronisation, not flops.
// Every dense factorisation is a Hermitian eigendecomposition by parallel cyclic Jacobi:
//   * gauges   X = diag(sqrt w) U^H, X^+ = U diag(1/sqrt w)  from env = U diag(w) U^H
//   * split    A = Q R with R = diag(sqrt l) W^H, Q = A W diag(1/sqrt l)  from A^H A = W diag(l) W^H
//   * SVD      theta = U S V^H with U, S^2 from theta theta^H, V^H = S^-1 U^H theta
#include <math.h>
#include <stdint.h>

#include "itn_apply.h"
#include "itn_common.cuh"

namespace itn {

namespace {

constexpr int kGateThreads = 256;
constexpr int kMaxJacobi = 128;        // largest matrix handed to the eigensolver
constexpr int kMaxSweeps = 40;
constexpr double kGramRtol = 1e-12;    // eigenvalues of A^H A kept: l > kGramRtol * l_max
constexpr double kSvdRtol2 = 1e-14;    // singular values kept: s^2 > kSvdRtol2 * s_max^2
constexpr double kPinvRtol = 1e-12;    // environment eigenvalues inverted: w > kPinvRtol * w_max

// ---- scalar helpers (double / complex128) --------------------------------------------------
__device__ __forceinline__ double abs2x(double a) { return a * a; }
__device__ __forceinline__ double abs2x(c128 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double scl_re(double a) { return a; }
__device__ __forceinline__ double scl_re(c128 a) { return a.x; }
__device__ __forceinline__ double scale(double a, double s) { return a * s; }
__device__ __forceinline__ c128 scale(c128 a, double s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ double sub(double a, double b) { return a - b; }
__device__ __forceinline__ c128 sub(c128 a, c128 b) { return {a.x - b.x, a.y - b.y}; }
template <typename T> __device__ __forceinline__ T from_re(double r);
template <> __device__ __forceinline__ double from_re<double>(double r) { return r; }
template <> __device__ __forceinline__ c128 from_re<c128>(double r) { return {r, 0.0}; }

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int k = 16; k >= 1; k >>= 1) v += __shfl_xor_sync(0xffffffffu, v, k);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
  __syncthreads();
  return t;
}

// out[p][a][q] = sum_c M[a][c] in[p][c][q]   (p < pre, a < dout, c < din, q < post)
template <typename T>
__device__ void apply_axis(const T* in, T* out, int64_t pre, int din, int64_t post, const T* M, int dout) {
  const int64_t total = pre * dout * post;
  for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
    const int64_t q = e % post, pa = e / post;
    const int a = (int)(pa % dout);
    const int64_t p = pa / dout;
    T acc = tzero<T>();
    const T* src = in + p * din * post + q;
    for (int c = 0; c < din; ++c) acc = fmac(M[a * din + c], src[c * post], acc);
    out[e] = acc;
  }
  __syncthreads();
}

// C[m][n] = sum_k A[m][k] B[k][n]
template <typename T>
__device__ void matmul(const T* A, const T* B, T* C, int64_t M, int K, int64_t N) {
  for (int64_t e = threadIdx.x; e < M * N; e += blockDim.x) {
    const int64_t m = e / N, n = e % N;
    T acc = tzero<T>();
    for (int k = 0; k < K; ++k) acc = fmac(A[m * K + k], B[(int64_t)k * N + n], acc);
    C[e] = acc;
  }
  __syncthreads();
}

// G[x][y] = sum_p conj(A[p][x]) A[p][y]
template <typename T>
__device__ void gram(const T* A, int64_t P, int n, T* G) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int x = e / n, y = e % n;
    T acc = tzero<T>();
    for (int64_t p = 0; p < P; ++p) acc = fmac(conjx(A[p * n + x]), A[p * n + y], acc);
    G[e] = acc;
  }
  __syncthreads();
}

struct Rot {
  int p, q;
  double c, s;
  double phr, phi;  // e^{i phi} of A[p][q] (real case: +-1, 0)
};

// Eigendecomposition of the Hermitian n x n matrix A (destroyed): A = V diag(w) V^H with w
// descending.  Parallel cyclic Jacobi with the round-robin pairing (n/2 disjoint 2 x 2
// rotations per round, n - 1 rounds per sweep), J = diag(1, e^{-i phi}) R(c, s) per pair.
// `V` receives the eigenvectors as columns, `tmp` needs n * n scratch entries.
template <typename T>
__device__ void herm_eig(T* A, int n, T* V, double* w, T* tmp, Rot* rot, double* red, int* perm) {
  const int N = n + (n & 1);  // even number of players; index n is a dummy when n is odd
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    V[e] = from_re<T>(i == j ? 1.0 : 0.0);
    // symmetrise: A <- (A + A^H) / 2
    if (i <= j) {
      const T a = A[i * n + j], b = conjx(A[j * n + i]);
      const T h = scale(add(a, b), 0.5);
      tmp[i * n + j] = h;
      tmp[j * n + i] = conjx(h);
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = tmp[e];
  __syncthreads();
  if (n == 1) {
    if (threadIdx.x == 0) w[0] = scl_re(A[0]);
    __syncthreads();
    return;
  }
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    double off = 0, dia = 0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e / n, j = e % n;
      if (i == j) dia += abs2x(A[e]);
      else off += abs2x(A[e]);
    }
    off = block_sum(off, red);
    dia = block_sum(dia, red);
    if (off <= 1e-30 * dia || off == 0.0) break;
    for (int r = 0; r < N - 1; ++r) {
      // rotation parameters of this round's pairs, all from the same A
      if (threadIdx.x < N / 2) {
        const int k = threadIdx.x;
        auto pos = [&](int j) { return j == 0 ? 0 : ((j - 1 + r) % (N - 1)) + 1; };
        int p = pos(k), q = pos(N - 1 - k);
        if (p > q) { const int t = p; p = q; q = t; }
        Rot R{p, q, 1.0, 0.0, 1.0, 0.0};
        if (q < n) {
          const T b = A[p * n + q];
          const double ab = sqrt(abs2x(b));
          const double a = scl_re(A[p * n + p]), d = scl_re(A[q * n + q]);
          if (ab > 1e-300 && ab > 1e-17 * (fabs(a) + fabs(d))) {
            const double tau = (d - a) / (2.0 * ab);
            const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            R.c = 1.0 / sqrt(1.0 + t * t);
            R.s = t * R.c;
            R.phr = re_d(b) / ab;
            R.phi = im_d(b) / ab;
          }
        }
        rot[k] = R;
      }
      __syncthreads();
      // columns p, q of A and V: A <- A J, V <- V J
      for (int e = threadIdx.x; e < (N / 2) * n; e += blockDim.x) {
        const Rot R = rot[e / n];
        if (R.s == 0.0) continue;
        const int i = e % n;
        T em;  // e^{-i phi}
        if constexpr (is_cplx<T>::value) em = T{R.phr, -R.phi}; else em = from_re<T>(R.phr);
        const T ap = A[i * n + R.p], aq = A[i * n + R.q];
        A[i * n + R.p] = sub(scale(ap, R.c), scale(mul(em, aq), R.s));
        A[i * n + R.q] = add(scale(ap, R.s), scale(mul(em, aq), R.c));
        const T vp = V[i * n + R.p], vq = V[i * n + R.q];
        V[i * n + R.p] = sub(scale(vp, R.c), scale(mul(em, vq), R.s));
        V[i * n + R.q] = add(scale(vp, R.s), scale(mul(em, vq), R.c));
      }
      __syncthreads();
      // rows p, q of A: A <- J^H A
      for (int e = threadIdx.x; e < (N / 2) * n; e += blockDim.x) {
        const Rot R = rot[e / n];
        if (R.s == 0.0) continue;
        const int j = e % n;
        T ep;  // e^{+i phi}
        if constexpr (is_cplx<T>::value) ep = T{R.phr, R.phi}; else ep = from_re<T>(R.phr);
        const T ap = A[R.p * n + j], aq = A[R.q * n + j];
        A[R.p * n + j] = sub(scale(ap, R.c), scale(mul(ep, aq), R.s));
        A[R.q * n + j] = add(scale(ap, R.s), scale(mul(ep, aq), R.c));
      }
      __syncthreads();
    }
  }
  // eigenvalues, sorted descending; eigenvector columns permuted alike
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int i = 0; i < n; ++i) {
      int best = i;
      for (int j = i + 1; j < n; ++j)
        if (scl_re(A[perm[j] * n + perm[j]]) > scl_re(A[perm[best] * n + perm[best]])) best = j;
      const int t = perm[i]; perm[i] = perm[best]; perm[best] = t;
    }
    for (int i = 0; i < n; ++i) w[i] = scl_re(A[perm[i] * n + perm[i]]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) tmp[e] = V[(e / n) * n + perm[e % n]];
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) V[e] = tmp[e];
  __syncthreads();
}

// herm_eig with the working matrices staged in shared memory when they fit (n <= kSmemJacobi):
// the rounds then read and write on-chip instead of making L2 round trips.
constexpr int kSmemJacobi = 64;
template <typename T>
__device__ void herm_eig_s(T* A, int n, T* V, double* w, T* tmp, Rot* rot, double* red, int* perm, T* sbuf) {
  if (n > kSmemJacobi) {
    herm_eig(A, n, V, w, tmp, rot, red, perm);
    return;
  }
  T* sA = sbuf;
  T* sV = sbuf + kSmemJacobi * kSmemJacobi;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) sA[e] = A[e];
  __syncthreads();
  herm_eig(sA, n, sV, w, tmp, rot, red, perm);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) V[e] = sV[e];
  __syncthreads();
}

// Gauge of one leg: X = diag(sqrt w+) U^H and X^+ = U diag(1/sqrt w) on w > rtol * w_max.
template <typename T>
__device__ void leg_gauge(const T* env, int D, T* X, T* Xp, T* a, T* v, T* tmp, double* w, Rot* rot,
                          double* red, int* perm, T* sbuf) {
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) a[e] = env[e];
  __syncthreads();
  herm_eig_s(a, D, v, w, tmp, rot, red, perm, sbuf);
  const double wmax = fmax(w[0], 0.0);
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    const int i = e / D, j = e % D;
    const double wi = fmax(w[i], 0.0), wj = fmax(w[j], 0.0);
    X[e] = scale(conjx(v[j * D + i]), sqrt(wi));                     // X[i][j] = sqrt(w_i) conj(U[j][i])
    Xp[e] = wj > kPinvRtol * wmax && wj > 0 ? scale(v[i * D + j], 1.0 / sqrt(wj)) : tzero<T>();
  }
  __syncthreads();
}

// Workspace of one gate, offsets in elements of T (host and device agree through this).
struct GateWs {
  int64_t X[2][kGateMaxLegs], Xp[2][kGateMaxLegs];
  int64_t A[2], buf[2], G[2], W[2], lam[2], R[2], C[2], B[2], B2[2];
  int64_t theta, H, U, lamH, Vh, ea, ev, etmp, ew, total;
};

__host__ __device__ inline void gate_ws(const GateJob& J, GateWs& L) {
  int64_t o = 0;
  auto take = [&](int64_t n) { const int64_t r = o; o += (n + 1) & ~int64_t(1); return r; };
  int64_t P[2] = {1, 1}, nn[2] = {0, 0}, maxD = 1;
  const int ns = J.nsite;
  for (int i = 0; i < ns; ++i) {
    for (int j = 0; j < J.nleg[i]; ++j) {
      P[i] *= J.leg_dim[i][j];
      maxD = J.leg_dim[i][j] > maxD ? J.leg_dim[i][j] : maxD;
      L.X[i][j] = take((int64_t)J.leg_dim[i][j] * J.leg_dim[i][j]);
      L.Xp[i][j] = take((int64_t)J.leg_dim[i][j] * J.leg_dim[i][j]);
    }
    nn[i] = (int64_t)J.d[i] * (ns == 2 ? J.bond : 1);
  }
  const int64_t chi = J.chi_cap > 0 ? J.chi_cap : 1;
  int64_t mcap = 1, ncap = 1;
  if (ns == 2) {
    mcap = J.d[0] * (P[0] < nn[0] ? P[0] : nn[0]);
    ncap = J.d[1] * (P[1] < nn[1] ? P[1] : nn[1]);
  }
  for (int i = 0; i < ns; ++i) {
    const int64_t big = P[i] * nn[i] > P[i] * J.d[i] * chi ? P[i] * nn[i] : P[i] * J.d[i] * chi;
    L.A[i] = take(P[i] * nn[i]);
    L.buf[i] = take(big);
    L.G[i] = take(nn[i] * nn[i]);
    L.W[i] = take(nn[i] * nn[i]);
    L.lam[i] = take(nn[i]);
    L.R[i] = take(nn[i] * nn[i]);
    L.C[i] = take(nn[i] * J.d[i] * chi);
    L.B[i] = take(big);
    L.B2[i] = take(big);
  }
  L.theta = take(mcap * ncap);
  L.H = take(mcap * mcap);
  L.U = take(mcap * mcap);
  L.lamH = take(mcap);
  L.Vh = take(mcap * ncap);
  const int64_t emax = (maxD > mcap ? maxD : mcap) > nn[0] ? (maxD > mcap ? maxD : mcap) : nn[0];
  const int64_t em = emax > nn[1] ? emax : nn[1];
  L.ea = take(em * em);
  L.ev = take(em * em);
  L.etmp = take(em * em);
  L.ew = take(em);
  L.total = o;
}

template <typename T>
__global__ void __launch_bounds__(kGateThreads) gate_kernel(const GateJob* jobs, const T* sites, const T* envs,
                                                            const T* ops, T* out, double* out_s, int* out_bond,
                                                            T* ws_base, int max_rank, double cutoff,
                                                            int normalize) {
  __shared__ Rot rot[kMaxJacobi / 2];
  __shared__ double red[32];
  __shared__ int perm[kMaxJacobi];
  __shared__ int s_chi;
  extern __shared__ __align__(16) unsigned char gate_smem[];
  T* sbuf = reinterpret_cast<T*>(gate_smem);  // 2 x kSmemJacobi^2 entries for the eigensolver
  const GateJob J = jobs[blockIdx.x];
  GateWs L;
  gate_ws(J, L);
  T* ws = ws_base + J.ws;
  double* wv = reinterpret_cast<double*>(ws + L.ew);
  const int ns = J.nsite;
  int64_t P[2] = {1, 1};
  for (int i = 0; i < ns; ++i)
    for (int j = 0; j < J.nleg[i]; ++j) P[i] *= J.leg_dim[i][j];
  // gauges of every other leg
  for (int i = 0; i < ns; ++i)
    for (int j = 0; j < J.nleg[i]; ++j)
      if (J.env_off[i][j] >= 0)
        leg_gauge(envs + J.env_off[i][j], J.leg_dim[i][j], ws + L.X[i][j], ws + L.Xp[i][j], ws + L.ea, ws + L.ev,
                  ws + L.etmp, wv, rot, red, perm, sbuf);

  if (ns == 1) {
    const int d = J.d[0];
    T* o = out + J.out_off[0];
    apply_axis(sites + J.site_off[0], o, P[0], d, 1, ops + J.op_off, d);
    if (normalize) {
      // norm of the result with every leg gauged
      T* g = ws + L.A[0];
      T* h = ws + L.buf[0];
      for (int64_t e = threadIdx.x; e < P[0] * d; e += blockDim.x) g[e] = o[e];
      __syncthreads();
      int64_t pre = 1;
      for (int j = 0; j < J.nleg[0]; ++j) {
        const int D = J.leg_dim[0][j];
        const int64_t post = P[0] / pre / D * d;
        if (J.env_off[0][j] >= 0) {
          apply_axis(g, h, pre, D, post, ws + L.X[0][j], D);
          T* t = g; g = h; h = t;
        }
        pre *= D;
      }
      double nrm = 0;
      for (int64_t e = threadIdx.x; e < P[0] * d; e += blockDim.x) nrm += abs2x(g[e]);
      nrm = block_sum(nrm, red);
      const double inv = nrm > 0 ? 1.0 / sqrt(nrm) : 1.0;
      for (int64_t e = threadIdx.x; e < P[0] * d; e += blockDim.x) o[e] = scale(o[e], inv);
    }
    if (threadIdx.x == 0) out_bond[blockIdx.x] = 0;
    return;
  }

  // two-site gate: gauge, split, theta, SVD, reassemble
  const int bond = J.bond;
  int rk[2];
  for (int i = 0; i < 2; ++i) {
    const int d = J.d[i], n = d * bond;
    T* a = ws + L.A[i];
    T* b = ws + L.buf[i];
    for (int64_t e = threadIdx.x; e < P[i] * n; e += blockDim.x) a[e] = sites[J.site_off[i] + e];
    __syncthreads();
    int64_t pre = 1;
    for (int j = 0; j < J.nleg[i]; ++j) {
      const int D = J.leg_dim[i][j];
      const int64_t post = P[i] / pre / D * n;
      if (J.env_off[i][j] >= 0) {
        apply_axis(a, b, pre, D, post, ws + L.X[i][j], D);
        for (int64_t e = threadIdx.x; e < P[i] * n; e += blockDim.x) a[e] = b[e];
        __syncthreads();
      }
      pre *= D;
    }
    // A^H A = W diag(l) W^H; R = diag(sqrt l) W^H over the kept l
    T* G = ws + L.G[i];
    T* W = ws + L.W[i];
    double* lam = reinterpret_cast<double*>(ws + L.lam[i]);
    gram(a, P[i], n, G);
    herm_eig_s(G, n, W, lam, ws + L.etmp, rot, red, perm, sbuf);
    if (threadIdx.x == 0) {
      int r = 0;
      const double lmax = fmax(lam[0], 0.0);
      while (r < n && lam[r] > kGramRtol * lmax && lam[r] > 0) ++r;
      if (r > P[i]) r = (int)P[i];  // rank of A (P x n) is at most P
      s_chi = r > 0 ? r : 1;
    }
    __syncthreads();
    rk[i] = s_chi;
    T* R = ws + L.R[i];
    for (int e = threadIdx.x; e < rk[i] * n; e += blockDim.x) {
      const int k = e / n, x = e % n;
      R[e] = scale(conjx(W[x * n + k]), sqrt(fmax(lam[k], 0.0)));
    }
    __syncthreads();
  }
  const int d1 = J.d[0], d2 = J.d[1];
  const int m = rk[0] * d1, nc = rk[1] * d2;
  // theta[(k1,s1')][(k2,s2')] = sum op[s1',s2',s1,s2] R1[k1][(s1,b)] R2[k2][(s2,b)]
  T* th = ws + L.theta;
  {
    const T* R1 = ws + L.R[0];
    const T* R2 = ws + L.R[1];
    const T* op = ops + J.op_off;
    const int n1 = d1 * bond, n2 = d2 * bond;
    for (int e = threadIdx.x; e < m * nc; e += blockDim.x) {
      const int x = e / nc, y = e % nc;
      const int k1 = x / d1, t1 = x % d1, k2 = y / d2, t2 = y % d2;
      T acc = tzero<T>();
      for (int s1 = 0; s1 < d1; ++s1)
        for (int s2 = 0; s2 < d2; ++s2) {
          const T o = op[((t1 * d2 + t2) * d1 + s1) * d2 + s2];
          if (is_zero(o)) continue;
          T inner = tzero<T>();
          for (int b = 0; b < bond; ++b) inner = fmac(R1[k1 * n1 + s1 * bond + b], R2[k2 * n2 + s2 * bond + b], inner);
          acc = fmac(o, inner, acc);
        }
      th[e] = acc;
    }
    __syncthreads();
  }
  // theta theta^H = U diag(s^2) U^H; V^H = diag(1/s) U^H theta
  T* H = ws + L.H;
  T* U = ws + L.U;
  double* s2 = reinterpret_cast<double*>(ws + L.lamH);
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int x = e / m, y = e % m;
    T acc = tzero<T>();
    for (int k = 0; k < nc; ++k) acc = fmac(th[x * nc + k], conjx(th[y * nc + k]), acc);
    H[e] = acc;
  }
  __syncthreads();
  herm_eig_s(H, m, U, s2, ws + L.etmp, rot, red, perm, sbuf);
  if (threadIdx.x == 0) {
    const double smax2 = fmax(s2[0], 0.0);
    int chi = 0;
    while (chi < m && s2[chi] > kSvdRtol2 * smax2 && s2[chi] > 0) ++chi;
    if (max_rank > 0 && chi > max_rank) chi = max_rank;
    if (cutoff > 0) {
      int k = 0;
      while (k < chi && sqrt(s2[k]) > cutoff) ++k;
      chi = k;
    }
    if (chi < 1) chi = 1;
    if (chi > J.chi_cap) chi = J.chi_cap;
    s_chi = chi;
  }
  __syncthreads();
  const int chi = s_chi;
  // singular values (optionally normalised)
  double* S = out_s + J.s_off;
  double snorm = 0;
  for (int k = threadIdx.x; k < chi; k += blockDim.x) snorm += fmax(s2[k], 0.0);
  snorm = block_sum(snorm, red);
  const double sfac = normalize && snorm > 0 ? 1.0 / sqrt(snorm) : 1.0;
  for (int k = threadIdx.x; k < chi; k += blockDim.x) S[k] = sqrt(fmax(s2[k], 0.0)) * sfac;
  if (threadIdx.x == 0) out_bond[blockIdx.x] = chi;
  __syncthreads();
  // R1'[(k1,s1')][c] = U[(k1,s1')][c] sqrt(S_c);  R2'[c][(k2,s2')] = sqrt(S_c) V^H[c][(k2,s2')]
  T* Vh = ws + L.Vh;
  for (int e = threadIdx.x; e < chi * nc; e += blockDim.x) {
    const int c = e / nc, y = e % nc;
    T acc = tzero<T>();
    for (int x = 0; x < m; ++x) acc = fmac(conjx(U[x * m + c]), th[x * nc + y], acc);
    const double sv = sqrt(fmax(s2[c], 0.0));
    // sqrt(S_c) / s_c with S_c = s_c * sfac
    Vh[e] = sv > 0 ? scale(acc, sqrt(sv * sfac) / sv) : tzero<T>();
  }
  __syncthreads();
  for (int i = 0; i < 2; ++i) {
    const int d = J.d[i], n = d * bond, r = rk[i];
    const T* W = ws + L.W[i];
    const double* lam = reinterpret_cast<const double*>(ws + L.lam[i]);
    // C[x][(s',c)] = sum_k W[x][k] l_k^{-1/2} R'[k, s', c]
    T* C = ws + L.C[i];
    for (int e = threadIdx.x; e < n * d * chi; e += blockDim.x) {
      const int x = e / (d * chi), sc = e % (d * chi), sp = sc / chi, c = sc % chi;
      T acc = tzero<T>();
      for (int k = 0; k < r; ++k) {
        T rp;
        if (i == 0) {
          const double sv = sqrt(fmax(s2[c], 0.0));
          rp = scale(U[(k * d1 + sp) * m + c], sqrt(sv * sfac));
        } else {
          rp = Vh[c * nc + k * d2 + sp];
        }
        acc = fmac(scale(W[x * n + k], 1.0 / sqrt(lam[k])), rp, acc);
      }
      C[e] = acc;
    }
    __syncthreads();
    // B = A C, then the inverse gauges leg by leg
    T* B = ws + L.B[i];
    T* B2 = ws + L.B2[i];
    matmul(ws + L.A[i], C, B, P[i], n, (int64_t)d * chi);
    int64_t pre = 1;
    for (int j = 0; j < J.nleg[i]; ++j) {
      const int D = J.leg_dim[i][j];
      const int64_t post = P[i] / pre / D * d * chi;
      if (J.env_off[i][j] >= 0) {
        apply_axis(B, B2, pre, D, post, ws + L.Xp[i][j], D);
        T* t = B; B = B2; B2 = t;
      }
      pre *= D;
    }
    T* o = out + J.out_off[i];
    for (int64_t e = threadIdx.x; e < P[i] * d * chi; e += blockDim.x) o[e] = B[e];
    __syncthreads();
  }
}

}  // namespace

int64_t gate_workspace(GateJob& J) {
  GateWs L;
  gate_ws(J, L);
  return L.total;
}

cudaError_t launch_gates(bool complex_data, int n, const GateJob* d_jobs, const void* d_sites, const void* d_envs,
                         const void* d_ops, void* d_out, double* d_s, int* d_bond, void* d_ws, int max_rank,
                         double cutoff, int normalize, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = 2 * kSmemJacobi * kSmemJacobi * (complex_data ? sizeof(c128) : sizeof(double));
  cudaError_t e = complex_data
                      ? cudaFuncSetAttribute(gate_kernel<c128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                      : cudaFuncSetAttribute(gate_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (complex_data)
    gate_kernel<c128><<<n, kGateThreads, smem, st>>>(d_jobs, (const c128*)d_sites, (const c128*)d_envs, (const c128*)d_ops,
                                                  (c128*)d_out, d_s, d_bond, (c128*)d_ws, max_rank, cutoff, normalize);
  else
    gate_kernel<double><<<n, kGateThreads, smem, st>>>(d_jobs, (const double*)d_sites, (const double*)d_envs,
                                                    (const double*)d_ops, (double*)d_out, d_s, d_bond, (double*)d_ws,
                                                    max_rank, cutoff, normalize);
  return cudaGetLastError();
}

}  // namespace itn
