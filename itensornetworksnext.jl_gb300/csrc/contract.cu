// contract.cu -- exact network contraction (contract_network(tn; alg = Exact(order_alg)),
// src/contract_network.jl:7-58) on the GPU.
//
// Host: a pairwise evaluation order (greedy: contract the pair whose result grows the
// network least, preferring pairs that share an index; or left-associative; or explicit)
// is chosen in C++ exactly as the CPU oracle chooses it.  Device: every pairwise step
// permutes its two operands into GEMM form -- A as [free_A, shared], B as [shared, free_B]
// (row-major) -- with a strided permute kernel and multiplies them with a tiled GEMM:
//   * CUDA cores for float / double / complex (64 x 64 tiles, 4 x 4 register blocking);
//   * tcgen05 for float in BF16 or TF32 split precision (hi/lo operands, 3 MMAs per product,
//     FP32 accumulation in TMEM) -- contract_gemm_tc in this file.
// The result carries the labels free_A ++ free_B.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include <cuda_bf16.h>

#include "itn_common.cuh"
#include "itn_contract.h"
#include "itn_tc.h"
#include "tc_ptx.cuh"

namespace itn {

// ---- order optimisation (host) ---------------------------------------------------------------
static double prod_dims(const std::vector<int64_t>& labels, const std::map<int64_t, int64_t>& dim) {
  double p = 1;
  for (int64_t l : labels) p *= (double)dim.at(l);
  return p;
}

// Multiply-adds of a pairwise order (the sum over steps of the product of the dimensions of
// every index of the two operands): the cost the sweep order is compared by.
double order_cost(const std::vector<std::vector<int64_t>>& labels, const std::map<int64_t, int64_t>& dim,
                  const std::vector<std::pair<int, int>>& steps) {
  std::vector<std::vector<int64_t>> L = labels;
  double total = 0;
  for (const auto& st : steps) {
    const std::vector<int64_t>&a = L[st.first], &b = L[st.second];
    std::vector<int64_t> all = a, lo;
    for (int64_t x : b)
      if (std::find(a.begin(), a.end(), x) == a.end()) all.push_back(x);
    for (int64_t x : a)
      if (std::find(b.begin(), b.end(), x) == b.end()) lo.push_back(x);
    for (int64_t x : b)
      if (std::find(a.begin(), a.end(), x) == a.end()) lo.push_back(x);
    total += prod_dims(all, dim);
    std::vector<std::vector<int64_t>> nl;
    for (int k = 0; k < (int)L.size(); ++k)
      if (k != st.first && k != st.second) nl.push_back(L[k]);
    nl.push_back(lo);
    L.swap(nl);
  }
  return total;
}

// Dense form of a network for the sweep search: label ids 0..m-1 per tensor, their dimensions
// and each tensor's size.
struct DenseNet {
  std::vector<std::vector<int>> lab;
  std::vector<double> dim, size;
};

static DenseNet dense_net(const std::vector<std::vector<int64_t>>& labels, const std::map<int64_t, int64_t>& dim) {
  DenseNet d;
  std::map<int64_t, int> id;
  for (const auto& l : labels) {
    std::vector<int> v;
    double sz = 1;
    for (int64_t x : l) {
      auto it = id.find(x);
      if (it == id.end()) {
        it = id.emplace(x, (int)d.dim.size()).first;
        d.dim.push_back((double)dim.at(x));
      }
      v.push_back(it->second);
      sz *= d.dim[it->second];
    }
    d.lab.push_back(v);
    d.size.push_back(sz);
  }
  return d;
}

// Sweep order from tensor `start`: one running product absorbs, at every step, the tensor
// that leaves it smallest (among those sharing an index with it; ties: fewer multiply-adds).
// On lattices this finds boundary-sweep orders (the running product is a boundary state).
// Returns the order's multiply-adds and writes it as working-list steps.
static double sweep_from(const DenseNet& net, int start, std::vector<std::pair<int, int>>& steps) {
  const int n = (int)net.lab.size();
  steps.clear();
  std::vector<int> pos(n);  // current position of each input tensor in the working list
  for (int t = 0; t < n; ++t) pos[t] = t;
  std::vector<char> used(n, 0), in_run(net.dim.size(), 0);
  used[start] = 1;
  for (int x : net.lab[start]) in_run[x] = 1;
  double run_size = net.size[start], total = 0;
  int run_pos = start, live = n;
  for (int k = 1; k < n; ++k) {
    int best = -1;
    bool bsh = false;
    double bsize = 0, bflops = 0;
    for (int j = 0; j < n; ++j) {
      if (used[j]) continue;
      double sh = 1;
      bool shared = false;
      for (int x : net.lab[j])
        if (in_run[x]) {
          shared = true;
          sh *= net.dim[x];
        }
      const double flops = run_size * net.size[j] / sh, size = flops / sh;
      const bool better = best < 0 || (shared && !bsh) ||
                          (shared == bsh && (size < bsize || (size == bsize && flops < bflops)));
      if (better) {
        best = j; bsh = shared; bsize = size; bflops = flops;
      }
    }
    // the product's labels: the running labels not on `best`, then best's not on the product
    for (int x : net.lab[best]) in_run[x] ^= 1;
    run_size = bsize;
    total += bflops;
    // working list: drop both operands, append the product
    const int i0 = std::min(run_pos, pos[best]), i1 = std::max(run_pos, pos[best]);
    steps.push_back({i0, i1});
    for (int t = 0; t < n; ++t)
      if (!used[t] && t != best) pos[t] -= (pos[t] > i1) + (pos[t] > i0);
    used[best] = 1;
    --live;
    run_pos = live - 1;
  }
  return total;
}

int contraction_order(const std::vector<std::vector<int64_t>>& labels, const std::map<int64_t, int64_t>& dim,
                      int alg, std::vector<std::pair<int, int>>& steps) {
  steps.clear();
  std::vector<std::vector<int64_t>> L = labels;
  const int n = (int)L.size();
  if (alg == 3) {
    // the cheaper (in multiply-adds) of the pairwise greedy order and the sweep orders from
    // every start tensor (at most 64 starts, evenly spaced, for larger networks)
    contraction_order(labels, dim, 0, steps);
    double best = order_cost(labels, dim, steps);
    const DenseNet net = dense_net(labels, dim);
    const int starts = std::min(n, 64);
    std::vector<std::pair<int, int>> cand;
    for (int k = 0; k < starts && n > 1; ++k) {
      const double cost = sweep_from(net, (int)((int64_t)k * n / starts), cand);
      if (cost < best) {
        best = cost;
        steps = cand;
      }
    }
    return 0;
  }
  if (alg == 1) {
    // left-associative ((t0 t1) t2) ...: in the shrinking working list the running
    // product sits last; every step contracts it (first operand) with the next input,
    // which is always at position 0
    if (n >= 2) steps.push_back({0, 1});
    for (int k = 2; k < n; ++k) steps.push_back({n - k, 0});
    return 0;
  }
  // A pair sharing an index always beats one that shares none (k0 below), so while any pair
  // shares an index only those pairs -- found through the holders of each label -- are
  // scanned, in the (i, j) order of the full scan: the same choice and tie-breaks as scanning
  // every pair, in time linear in the number of linked pairs instead of quadratic in n.
  while (L.size() > 1) {
    int bi = -1, bj = -1;
    double bk0 = 0, bk1 = 0, bk2 = 0;
    std::vector<int64_t> blo;
    std::map<int64_t, std::vector<int>> holders;
    for (int i = 0; i < (int)L.size(); ++i)
      for (int64_t x : L[i]) holders[x].push_back(i);
    std::vector<std::pair<int, int>> linked;
    for (const auto& kv : holders)
      for (size_t a = 0; a < kv.second.size(); ++a)
        for (size_t b = a + 1; b < kv.second.size(); ++b)
          if (kv.second[a] != kv.second[b])
            linked.push_back({std::min(kv.second[a], kv.second[b]), std::max(kv.second[a], kv.second[b])});
    std::sort(linked.begin(), linked.end());
    linked.erase(std::unique(linked.begin(), linked.end()), linked.end());
    std::vector<std::pair<int, int>> all_pairs;
    if (linked.empty())
      for (int i = 0; i < (int)L.size(); ++i)
        for (int j = i + 1; j < (int)L.size(); ++j) all_pairs.push_back({i, j});
    for (const auto& pr : linked.empty() ? all_pairs : linked) {
        const int i = pr.first, j = pr.second;
        std::vector<int64_t> lo;
        bool shared = false;
        for (int64_t x : L[i]) {
          if (std::find(L[j].begin(), L[j].end(), x) != L[j].end()) shared = true;
          else lo.push_back(x);
        }
        for (int64_t x : L[j])
          if (std::find(L[i].begin(), L[i].end(), x) == L[i].end()) lo.push_back(x);
        const double so = prod_dims(lo, dim), sa = prod_dims(L[i], dim), sb = prod_dims(L[j], dim);
        const double k0 = shared ? 0 : 1, k1 = so - sa - sb, k2 = so;
        const bool better = bi < 0 || k0 < bk0 || (k0 == bk0 && (k1 < bk1 || (k1 == bk1 && k2 < bk2)));
        if (better) {
          bi = i; bj = j; bk0 = k0; bk1 = k1; bk2 = k2; blo = lo;
        }
      }
    steps.push_back({bi, bj});
    std::vector<std::vector<int64_t>> nl;
    for (int k = 0; k < (int)L.size(); ++k)
      if (k != bi && k != bj) nl.push_back(L[k]);
    nl.push_back(blo);
    L.swap(nl);
  }
  return 0;
}

// ---- device kernels ----------------------------------------------------------------------------
constexpr int kMaxRank = 48;

struct PermArgs {
  int rank;
  long long out_dims[kMaxRank];
  long long in_stride[kMaxRank];  // input stride of the input axis that becomes output axis a
};

template <typename T>
__global__ void permute_tensor_kernel(const T* __restrict__ in, T* __restrict__ out, long long n, PermArgs p) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
    long long rem = j, off = 0;
    for (int a = p.rank - 1; a >= 0; --a) {
      const long long d = p.out_dims[a];
      const long long idx = rem % d;
      rem /= d;
      off += idx * p.in_stride[a];
    }
    out[j] = in[off];
  }
}

// The same for tensors of fewer than 2^31 entries: 32-bit index arithmetic (a 64-bit division
// costs several times a 32-bit one, and a permute of a boundary-sweep product is dominated by
// its index arithmetic, not its bytes).
struct PermArgs32 {
  int rank;
  int out_dims[kMaxRank];
  int in_stride[kMaxRank];
};

template <typename T>
__global__ void permute_tensor32_kernel(const T* __restrict__ in, T* __restrict__ out, int n, PermArgs32 p) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    int rem = j, off = 0;
    for (int a = p.rank - 1; a >= 0; --a) {
      const int d = p.out_dims[a];
      const int q = rem / d;
      off += (rem - q * d) * p.in_stride[a];
      rem = q;
    }
    out[j] = in[off];
  }
}

// C[M,N] = A[M,K] * B[K,N], row-major, CUDA cores: 64 x 64 tile per CTA, 256 threads,
// 4 x 4 outputs per thread, K staged through shared memory in slices of 16.
template <typename T>
__global__ void __launch_bounds__(256) gemm_cc_kernel(const T* __restrict__ A, const T* __restrict__ B,
                                                      T* __restrict__ C, long long M, long long N, long long K) {
  __shared__ T As[16][64 + 1];
  __shared__ T Bs[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long long tiles_n = (N + 63) / 64;
  const long long tile = blockIdx.x;
  const long long m0 = (tile / tiles_n) * 64, n0 = (tile % tiles_n) * 64;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = tzero<T>();
  for (long long k0 = 0; k0 < K; k0 += 16) {
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const int r = e >> 4, kk = e & 15;  // A tile: 64 rows x 16 k
      const long long gm = m0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < K) ? A[gm * K + gk] : tzero<T>();
      const int kb = e >> 6, c = e & 63;  // B tile: 16 k x 64 cols
      const long long gk2 = k0 + kb, gn = n0 + c;
      Bs[kb][c] = (gk2 < K && gn < N) ? B[gk2 * N + gn] : tzero<T>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmac(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
      if (gm < M && gn < N) C[gm * N + gn] = acc[i][j];
    }
}

template <typename T>
cudaError_t permute_t(const void* in, void* out, const std::vector<int64_t>& in_dims, const std::vector<int>& perm,
                      cudaStream_t st) {
  const int r = (int)in_dims.size();
  if (r > kMaxRank) return cudaErrorInvalidValue;
  std::vector<long long> istr(r, 1);
  for (int a = r - 2; a >= 0; --a) istr[a] = istr[a + 1] * in_dims[a + 1];
  long long n = 1;
  for (int a = 0; a < r; ++a) n *= in_dims[a];
  if (n == 0) return cudaSuccess;
  // merge runs of output axes that are consecutive input axes in the same order (one axis of
  // the product of their dimensions, strided like the run's innermost axis); unit axes drop
  std::vector<long long> od, os;
  for (int a = 0; a < r;) {
    int b = a;
    long long d = in_dims[perm[a]];
    while (b + 1 < r && perm[b + 1] == perm[b] + 1) d *= in_dims[perm[++b]];
    if (d != 1) {
      od.push_back(d);
      os.push_back(istr[perm[b]]);
    }
    a = b + 1;
  }
  if (od.empty()) {
    od.push_back(1);
    os.push_back(1);
  }
  const int rank = (int)od.size();
  const int grid = (int)std::min<long long>((n + 255) / 256, 65535);
  if (n < (1LL << 31)) {
    PermArgs32 p;
    p.rank = rank;
    for (int a = 0; a < rank; ++a) {
      p.out_dims[a] = (int)od[a];
      p.in_stride[a] = (int)os[a];
    }
    permute_tensor32_kernel<T><<<grid, 256, 0, st>>>(reinterpret_cast<const T*>(in), reinterpret_cast<T*>(out), (int)n,
                                                    p);
  } else {
    PermArgs p;
    p.rank = rank;
    for (int a = 0; a < rank; ++a) {
      p.out_dims[a] = od[a];
      p.in_stride[a] = os[a];
    }
    permute_tensor_kernel<T><<<grid, 256, 0, st>>>(reinterpret_cast<const T*>(in), reinterpret_cast<T*>(out), n, p);
  }
  return cudaGetLastError();
}

// C[M,N] = A[M,K] B[K,N] when one side is thin (at most kThin rows of A or columns of B) and
// K <= kThinK: the thin operand (at most 32 x 64 entries) is staged in shared memory and each
// thread computes entries of C directly, grid-stride, consecutive threads on consecutive
// entries of C, so the long operand's loads are coalesced (SMALL_A) or shared by the threads
// of one row (SMALL_B) and C's stores are coalesced.  gemm_cc_kernel's 64 x 64 tiles with
// K slices of 16 would compute mostly padding on such shapes (the steps of a boundary-sweep
// contraction: M ~ 1e6, N and K ~ 3-18).
constexpr int kThin = 32, kThinK = 64;

template <typename T, bool SMALL_B>
__global__ void __launch_bounds__(256) gemm_thin_kernel(const T* __restrict__ A, const T* __restrict__ B,
                                                        T* __restrict__ C, long long M, long long N, int K) {
  extern __shared__ __align__(16) unsigned char thin_sm[];
  T* S = reinterpret_cast<T*>(thin_sm);
  const long long sn = SMALL_B ? (long long)K * N : M * (long long)K;
  const T* src = SMALL_B ? B : A;
  for (long long i = threadIdx.x; i < sn; i += blockDim.x) S[i] = src[i];
  __syncthreads();
  const long long total = M * N;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total;
       j += (long long)gridDim.x * blockDim.x) {
    const long long m = j / N, n = j - m * N;
    T acc = tzero<T>();
    if (SMALL_B) {
      const T* a = A + m * K;
      for (int k = 0; k < K; ++k) acc = fmac(a[k], S[k * N + n], acc);
    } else {
      const T* b = B + n;
      for (int k = 0; k < K; ++k) acc = fmac(S[m * K + k], b[(long long)k * N], acc);
    }
    C[j] = acc;
  }
}

// The same product with the long operand read in place, in its own index order: `v` lists its
// free axes (adjacent ones merged) with their strides and the element offset of each of the K
// contracted positions.  Saves the permute of the long operand (a read and a write of the whole
// tensor) at the price of per-entry index arithmetic, which the FP64 product hides.
template <typename T, bool SMALL_B>
__global__ void __launch_bounds__(256) gemm_thin_view_kernel(const T* __restrict__ A, const T* __restrict__ B,
                                                             T* __restrict__ C, long long M, long long N, int K,
                                                             ThinView v) {
  extern __shared__ __align__(16) unsigned char thin_sm[];
  T* S = reinterpret_cast<T*>(thin_sm);
  const long long sn = SMALL_B ? (long long)K * N : M * (long long)K;
  long long* koff = reinterpret_cast<long long*>(thin_sm + ((sn * (long long)sizeof(T) + 15) & ~15LL));
  const T* src = SMALL_B ? B : A;
  for (long long i = threadIdx.x; i < sn; i += blockDim.x) S[i] = src[i];
  for (int i = threadIdx.x; i < K; i += blockDim.x) koff[i] = v.koff[i];
  __syncthreads();
  const T* L = SMALL_B ? A : B;
  const long long total = M * N;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total;
       j += (long long)gridDim.x * blockDim.x) {
    const long long m = j / N, n = j - m * N;
    long long rem = SMALL_B ? m : n, off = 0;
    for (int a = v.rank - 1; a >= 0; --a) {
      const long long d = v.dims[a], q = rem / d;
      off += (rem - q * d) * v.stride[a];
      rem = q;
    }
    T acc = tzero<T>();
    if (SMALL_B) {
      for (int k = 0; k < K; ++k) acc = fmac(L[off + koff[k]], S[k * N + n], acc);
    } else {
      for (int k = 0; k < K; ++k) acc = fmac(S[m * K + k], L[off + koff[k]], acc);
    }
    C[j] = acc;
  }
}

template <typename T>
cudaError_t gemm_view_t(const void* A, const void* B, void* C, long long M, long long N, long long K, bool small_b,
                        const ThinView& v, cudaStream_t st) {
  if (M == 0 || N == 0) return cudaSuccess;
  const size_t smem = (((size_t)(small_b ? N : M) * K * sizeof(T) + 15) & ~(size_t)15) + (size_t)K * sizeof(long long);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)std::max<long long>(1, std::min<long long>((M * N + 255) / 256, (long long)sms * 8));
  if (small_b)
    gemm_thin_view_kernel<T, true><<<grid, 256, smem, st>>>(reinterpret_cast<const T*>(A), reinterpret_cast<const T*>(B),
                                                           reinterpret_cast<T*>(C), M, N, (int)K, v);
  else
    gemm_thin_view_kernel<T, false><<<grid, 256, smem, st>>>(reinterpret_cast<const T*>(A), reinterpret_cast<const T*>(B),
                                                            reinterpret_cast<T*>(C), M, N, (int)K, v);
  return cudaGetLastError();
}

template <typename T>
cudaError_t gemm_t(const void* A, const void* B, void* C, long long M, long long N, long long K, cudaStream_t st) {
  if (M == 0 || N == 0) return cudaSuccess;
  if (K <= kThinK && (N <= kThin || M <= kThin) && std::max(M, N) >= 256) {
    const bool small_b = N <= kThin;
    const size_t smem = (size_t)(small_b ? N : M) * K * sizeof(T);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::max<long long>(1, std::min<long long>((M * N + 255) / 256, (long long)sms * 8));
    if (small_b)
      gemm_thin_kernel<T, true><<<grid, 256, smem, st>>>(reinterpret_cast<const T*>(A), reinterpret_cast<const T*>(B),
                                                        reinterpret_cast<T*>(C), M, N, (int)K);
    else
      gemm_thin_kernel<T, false><<<grid, 256, smem, st>>>(reinterpret_cast<const T*>(A), reinterpret_cast<const T*>(B),
                                                         reinterpret_cast<T*>(C), M, N, (int)K);
    return cudaGetLastError();
  }
  const long long tiles = ((N + 63) / 64) * ((M + 63) / 64);
  if (tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  gemm_cc_kernel<T><<<(unsigned)tiles, 256, 0, st>>>(reinterpret_cast<const T*>(A), reinterpret_cast<const T*>(B),
                                         reinterpret_cast<T*>(C), M, N, K);
  return cudaGetLastError();
}

cudaError_t contract_permute(int dtype, const void* in, void* out, const std::vector<int64_t>& in_dims,
                             const std::vector<int>& perm, cudaStream_t st) {
  switch (dtype) {
    case 0: return permute_t<float>(in, out, in_dims, perm, st);
    case 1: return permute_t<double>(in, out, in_dims, perm, st);
    case 2: return permute_t<c64>(in, out, in_dims, perm, st);
    case 3: return permute_t<c128>(in, out, in_dims, perm, st);
  }
  return cudaErrorInvalidValue;
}

bool contract_thin_shape(long long M, long long N, long long K) {
  return K <= kThinK && (N <= kThin || M <= kThin) && std::max(M, N) >= 256;
}

bool contract_thin_small_b(long long M, long long N) { return N <= kThin; }

cudaError_t contract_gemm_view(int dtype, const void* A, const void* B, void* C, long long M, long long N,
                               long long K, bool small_b, const ThinView& v, cudaStream_t st) {
  if (v.rank > kMaxRank || K > kThinK) return cudaErrorInvalidValue;
  switch (dtype) {
    case 0: return gemm_view_t<float>(A, B, C, M, N, K, small_b, v, st);
    case 1: return gemm_view_t<double>(A, B, C, M, N, K, small_b, v, st);
    case 2: return gemm_view_t<c64>(A, B, C, M, N, K, small_b, v, st);
    case 3: return gemm_view_t<c128>(A, B, C, M, N, K, small_b, v, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t contract_gemm(int dtype, const void* A, const void* B, void* C, long long M, long long N, long long K,
                          cudaStream_t st) {
  switch (dtype) {
    case 0: return gemm_t<float>(A, B, C, M, N, K, st);
    case 1: return gemm_t<double>(A, B, C, M, N, K, st);
    case 2: return gemm_t<c64>(A, B, C, M, N, K, st);
    case 3: return gemm_t<c128>(A, B, C, M, N, K, st);
  }
  return cudaErrorInvalidValue;
}


// ---- tcgen05 GEMM with hi/lo split operands (float32 in, float32 out) --------------------------
// Two operand modes: BF16 hi/lo (x = hi + lo, both BF16: ~16 significant bits, kind::f16) and
// TF32 hi/lo (hi = the TF32 rounding of x, lo = the TF32 rounding of x - hi: ~21 bits, the
// accuracy of FP32 arithmetic, kind::tf32).  Each product is hi*hi + lo*hi + hi*lo (3 MMAs).
// Operands are packed into K-major core-matrix tiles (cores of 8 rows x 16 bytes): A tile
// (mt, kt) = 128 rows x 64 k, B tile (nt, kt) = 64 columns of B (as rows) x 64 k; each tile
// holds its hi part followed by its lo part.  One CTA computes a 128 x 64 block of C with D in
// 64 TMEM columns, streaming K through a two-stage bulk-TMA pipeline.
namespace {

template <int MODE> struct GemmMode;  // 0: BF16 hi/lo, 1: TF32 hi/lo
template <> struct GemmMode<0> {
  static constexpr uint32_t blk = 8192;   // 64 x 64 block
  static constexpr uint32_t sbo = 1024;   // bytes between 8-row core groups
  static constexpr int ksteps = 4;        // MMAs per K = 64
};
template <> struct GemmMode<1> {
  static constexpr uint32_t blk = 16384;
  static constexpr uint32_t sbo = 2048;
  static constexpr int ksteps = 8;
};
template <int MODE> constexpr uint32_t a_tile() { return 4 * GemmMode<MODE>::blk; }  // 2 blocks hi + 2 lo
template <int MODE> constexpr uint32_t b_tile() { return 2 * GemmMode<MODE>::blk; }  // 1 block hi + 1 lo
constexpr uint32_t kTcPolls = 1u << 26;

// byte offset of element (r, k) inside a 64 x 64 block of the mode
template <int MODE>
__host__ __device__ __forceinline__ uint32_t cblk_off(int r, int k) {
  if constexpr (MODE == 1)
    return (uint32_t)((((r >> 3) << 4) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
  else
    return (uint32_t)((((r >> 3) << 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// hi and lo parts of x, stored at the element's offset in the hi and lo planes
template <int MODE>
__device__ __forceinline__ void put_split(unsigned char* hi, unsigned char* lo, uint32_t o, float x) {
  if constexpr (MODE == 1) {
    const uint32_t h = ptx::to_tf32(x);
    *reinterpret_cast<uint32_t*>(hi + o) = h;
    *reinterpret_cast<uint32_t*>(lo + o) = ptx::to_tf32(x - __uint_as_float(h));
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    *reinterpret_cast<__nv_bfloat16*>(hi + o) = h;
    *reinterpret_cast<__nv_bfloat16*>(lo + o) = __float2bfloat16_rn(x - __bfloat162float(h));
  }
}

template <int MODE>
__global__ void pack_a_kernel(const float* __restrict__ A, long long M, long long K, long long kt_n,
                              unsigned char* __restrict__ out, long long tiles) {
  constexpr uint32_t blk = GemmMode<MODE>::blk;
  // one thread per (tile, row, k): element A[m][k]
  const long long total = tiles * 128 * 64;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total; j += (long long)gridDim.x * blockDim.x) {
    const long long t = j >> 13;
    const int r = (int)((j >> 6) & 127), k = (int)(j & 63);
    const long long mt = t / kt_n, kt = t % kt_n;
    const long long m = mt * 128 + r, kk = kt * 64 + k;
    const float x = (m < M && kk < K) ? A[m * K + kk] : 0.f;
    unsigned char* base = out + t * a_tile<MODE>();
    const uint32_t o = (r >> 6) * blk + cblk_off<MODE>(r & 63, k);
    put_split<MODE>(base, base + 2 * blk, o, x);
  }
}

template <int MODE>
__global__ void pack_b_kernel(const float* __restrict__ B, long long K, long long N, long long kt_n,
                              unsigned char* __restrict__ out, long long tiles) {
  constexpr uint32_t blk = GemmMode<MODE>::blk;
  const long long total = tiles * 64 * 64;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total; j += (long long)gridDim.x * blockDim.x) {
    const long long t = j >> 12;
    const int r = (int)((j >> 6) & 63), k = (int)(j & 63);  // r: column n of B, k: row k of B
    const long long nt = t / kt_n, kt = t % kt_n;
    const long long n = nt * 64 + r, kk = kt * 64 + k;
    const float x = (n < N && kk < K) ? B[kk * N + n] : 0.f;
    unsigned char* base = out + t * b_tile<MODE>();
    put_split<MODE>(base, base + blk, cblk_off<MODE>(r, k), x);
  }
}

// The tensor core sums each K = 64 tile into TMEM; after every tile the 128 threads read the
// tile's partial products and add them to FP32 registers (one row of 64 columns per thread),
// so that the long sum over K runs in round-to-nearest FP32 on the CUDA cores.  Loads of tile
// kt + 1 overlap the MMAs of tile kt (two smem stages); the readout of tile kt precedes the
// MMAs of tile kt + 1, which overwrite the same 64 TMEM columns.
template <int MODE>
__global__ void __launch_bounds__(128) gemm_tc_kernel(const unsigned char* __restrict__ Ap,
                                                      const unsigned char* __restrict__ Bp, float* __restrict__ C,
                                                      long long M, long long N, long long kt_n, long long nt_n,
                                                      int* err) {
  using G = GemmMode<MODE>;
  constexpr uint32_t kA = a_tile<MODE>(), kB = b_tile<MODE>();
  extern __shared__ __align__(1024) unsigned char sm[];
  // stage s: A tile at s * (A + B), B tile after it
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * (kA + kB));  // load[2], mma
  uint32_t* taddr_s = reinterpret_cast<uint32_t*>(bar + 4);
  // the warp index and TMEM base are broadcast from lane 0 so that the compiler treats them as
  // warp-uniform; warp 0 issues the MMAs from one elected lane (faster than a tid == 0 branch)
  const int tid = threadIdx.x, lane = tid & 31;
  const int warp = __shfl_sync(0xffffffffu, tid >> 5, 0);
  const long long mt = blockIdx.x / nt_n, nt = blockIdx.x % nt_n;
  if (warp == 0) {
    ptx::tmem_alloc(taddr_s, 64);
    ptx::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 3; ++i) ptx::mbar_init(bar + i, 1);
    ptx::fence_mbar_init();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = __shfl_sync(0xffffffffu, *taddr_s, 0);
  const uint32_t sb = ptx::smem_u32(sm);
  constexpr uint32_t idesc = MODE == 1 ? ptx::idesc_tf32_f32(128, 64) : ptx::idesc_bf16_f32(128, 64);
  auto load = [&](long long kt, int s) {
    unsigned char* dst = sm + s * (kA + kB);
    ptx::mbar_arrive_expect_tx(bar + s, kA + kB);
    ptx::bulk_g2s(dst, Ap + (mt * kt_n + kt) * kA, kA, bar + s);
    ptx::bulk_g2s(dst + kA, Bp + (nt * kt_n + kt) * kB, kB, bar + s);
  };
  auto mma = [&](uint32_t a, uint32_t b, uint32_t acc) {
    const uint64_t ad = ptx::smem_desc(a, 128, G::sbo), bd = ptx::smem_desc(b, 128, G::sbo);
    if constexpr (MODE == 1) ptx::mma_tf32(tmem, ad, bd, idesc, acc);
    else ptx::mma_bf16(tmem, ad, bd, idesc, acc);
  };
  uint32_t ph_load[2] = {0, 0}, ph_mma = 0;
  bool ld_pend[2] = {false, false};  // tid 0: copies in flight per stage
  float acc[64];
#pragma unroll
  for (int i = 0; i < 64; ++i) acc[i] = 0.f;
  if (tid == 0) {
    load(0, 0);
    ld_pend[0] = true;
  }
  bool ok = true, mma_lost = false;
  for (long long kt = 0; kt < kt_n; ++kt) {
    const int s = (int)(kt & 1);
    bool mine = true;
    if (warp == 0) {
      // stage s ^ 1 was last read by the MMAs of tile kt - 1, which completed before the
      // readout below
      if (lane == 0 && kt + 1 < kt_n) {
        load(kt + 1, s ^ 1);
        ld_pend[s ^ 1] = true;
      }
      mine = ptx::mbar_wait_bounded(bar + s, ph_load[s], kTcPolls);
      if (mine) ld_pend[s] = false;
      ph_load[s] ^= 1;
      mine = __all_sync(0xffffffffu, mine);  // the elected block below needs the whole warp
      if (mine) {
        ptx::tc_fence_after();
        const uint32_t a = sb + s * (kA + kB), b = a + kA;
        if (ptx::elect_one()) {
#pragma unroll
          for (int j = 0; j < G::ksteps; ++j) {
            const uint32_t ko = (uint32_t)(2 * j) * 128;  // two core columns per MMA
            mma(a + ko, b + ko, j > 0 ? 1u : 0u);
            mma(a + 2 * G::blk + ko, b + ko, 1);
            mma(a + ko, b + G::blk + ko, 1);
          }
          ptx::mma_commit(bar + 2);
        }
        __syncwarp();
      }
    }
    if (!__syncthreads_and(mine)) {
      ok = false;
      break;
    }
    if (!__syncthreads_and(ptx::mbar_wait_bounded(bar + 2, ph_mma, kTcPolls))) {
      ok = false;
      mma_lost = true;
      break;
    }
    ph_mma ^= 1;
    ptx::tc_fence_after();
#pragma unroll
    for (int cb = 0; cb < 4; ++cb) {
      float v[16];
      ptx::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + cb * 16, v);
      ptx::tmem_wait_ld();
#pragma unroll
      for (int e = 0; e < 16; ++e) acc[cb * 16 + e] += v[e];
    }
    ptx::tc_fence_before();
    __syncthreads();
  }
  if (!ok && tid == 0) {
    atomicExch(err, 1);
    // let copies still in flight land before the shared memory is released (bounded)
    for (int st = 0; st < 2; ++st)
      if (ld_pend[st]) ptx::mbar_wait_bounded(bar + st, ph_load[st], kTcPolls);
    // and MMAs whose completion was not seen, before the tensor memory is released
    if (mma_lost) ptx::mbar_wait_bounded(bar + 2, ph_mma, kTcPolls);
  }
  if (ok) {
    const int row = warp * 32 + lane;
    const long long m = mt * 128 + row;
    if (m < M) {
#pragma unroll
      for (int e = 0; e < 64; ++e) {
        const long long n = nt * 64 + e;
        if (n < N) C[m * N + n] = acc[e];
      }
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, 64);
  }
}

int* g_tc_err = nullptr;

template <int MODE>
cudaError_t gemm_tc_run(const float* A, const float* B, float* C, long long M, long long N, long long K,
                        cudaStream_t st) {
  constexpr uint32_t kA = a_tile<MODE>(), kB = b_tile<MODE>();
  const long long mt_n = (M + 127) / 128, nt_n = (N + 63) / 64, kt_n = (K + 63) / 64;
  if (mt_n * nt_n > 0x7fffffffLL) return cudaErrorInvalidValue;
  unsigned char *Ap = nullptr, *Bp = nullptr;
  cudaError_t e = cudaMallocAsync(&Ap, (size_t)(mt_n * kt_n) * kA, st);
  if (e != cudaSuccess) return e;
  e = cudaMallocAsync(&Bp, (size_t)(nt_n * kt_n) * kB, st);
  if (e != cudaSuccess) {
    cudaFreeAsync(Ap, st);
    return e;
  }
  if (!g_tc_err) {
    e = cudaMalloc(&g_tc_err, sizeof(int));
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(g_tc_err, 0, sizeof(int), st);
  }
  const long long at = mt_n * kt_n, bt = nt_n * kt_n;
  pack_a_kernel<MODE><<<(int)std::min<long long>((at * 8192 + 255) / 256, 1 << 20), 256, 0, st>>>(A, M, K, kt_n, Ap,
                                                                                                  at);
  pack_b_kernel<MODE><<<(int)std::min<long long>((bt * 4096 + 255) / 256, 1 << 20), 256, 0, st>>>(B, K, N, kt_n, Bp,
                                                                                                  bt);
  const size_t smem = 2 * (kA + kB) + 64;
  cudaFuncSetAttribute(gemm_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  gemm_tc_kernel<MODE><<<(unsigned)(mt_n * nt_n), 128, smem, st>>>(Ap, Bp, C, M, N, kt_n, nt_n, g_tc_err);
  e = cudaGetLastError();
  cudaFreeAsync(Ap, st);
  cudaFreeAsync(Bp, st);
  return e;
}

}  // namespace

cudaError_t contract_gemm_tc(const float* A, const float* B, float* C, long long M, long long N, long long K,
                             cudaStream_t st, bool tf32) {
  if (M == 0 || N == 0) return cudaSuccess;
  int m128 = 0, m64 = 0;
  cudaError_t e = tc_run_probe(st, &m128, &m64, nullptr, nullptr);
  if (e != cudaSuccess) return e;
  if (!m128 || (tf32 && !tc_tf32_ok())) return cudaErrorNotSupported;
  if (K == 0) return cudaMemsetAsync(C, 0, (size_t)M * N * sizeof(float), st);
  return tf32 ? gemm_tc_run<1>(A, B, C, M, N, K, st) : gemm_tc_run<0>(A, B, C, M, N, K, st);
}

}  // namespace itn
