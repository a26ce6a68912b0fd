// contract.cu -- exact network contraction (contract_network(tn; alg = Exact(order_alg)),
// src/contract_network.jl:7-58) on the GPU.
//
// Host: a pairwise evaluation order (greedy: contract the pair whose result grows the
// network least, preferring pairs that share an index; or left-associative; or explicit)
// is chosen in C++ exactly as the CPU oracle chooses it.  Device: every pairwise step
// permutes its two operands into GEMM form -- A as [free_A, shared], B as [shared, free_B]
// (row-major) -- with a strided permute kernel and multiplies them with a tiled GEMM:
//   * CUDA cores for float / double / complex (64 x 64 tiles, 4 x 4 register blocking);
//   * tcgen05 for float in BF16 split precision (hi/lo operands, 3 MMAs per product,
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

int contraction_order(const std::vector<std::vector<int64_t>>& labels, const std::map<int64_t, int64_t>& dim,
                      int alg, std::vector<std::pair<int, int>>& steps) {
  steps.clear();
  std::vector<std::vector<int64_t>> L = labels;
  const int n = (int)L.size();
  if (alg == 1) {
    // left-associative ((t0 t1) t2) ...: in the shrinking working list the running
    // product sits last; every step contracts it (first operand) with the next input,
    // which is always at position 0
    if (n >= 2) steps.push_back({0, 1});
    for (int k = 2; k < n; ++k) steps.push_back({n - k, 0});
    return 0;
  }
  while (L.size() > 1) {
    int bi = -1, bj = -1;
    double bk0 = 0, bk1 = 0, bk2 = 0;
    std::vector<int64_t> blo;
    for (int i = 0; i < (int)L.size(); ++i)
      for (int j = i + 1; j < (int)L.size(); ++j) {
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
  PermArgs p;
  p.rank = r;
  std::vector<long long> istr(r, 1);
  for (int a = r - 2; a >= 0; --a) istr[a] = istr[a + 1] * in_dims[a + 1];
  long long n = 1;
  for (int a = 0; a < r; ++a) {
    p.out_dims[a] = in_dims[perm[a]];
    p.in_stride[a] = istr[perm[a]];
    n *= in_dims[a];
  }
  if (n == 0) return cudaSuccess;
  const int grid = (int)std::min<long long>((n + 255) / 256, 65535);
  permute_tensor_kernel<T><<<grid, 256, 0, st>>>(reinterpret_cast<const T*>(in), reinterpret_cast<T*>(out), n, p);
  return cudaGetLastError();
}

template <typename T>
cudaError_t gemm_t(const void* A, const void* B, void* C, long long M, long long N, long long K, cudaStream_t st) {
  if (M == 0 || N == 0) return cudaSuccess;
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


// ---- tcgen05 GEMM, BF16 hi/lo split (float32 in, float32 out) --------------------------------
// Operands are packed into K-major core-matrix tiles: A tile (mt, kt) = 128 rows x 64 k,
// B tile (nt, kt) = 64 columns of B (as rows) x 64 k; each tile holds its hi part followed by
// its lo part.  One CTA computes a 128 x 64 block of C with D in 64 TMEM columns, streaming K
// through a two-stage bulk-TMA pipeline.
namespace {

constexpr int kTcBlk = 8192;                      // 64 x 64 BF16 block
constexpr uint32_t kTcATile = 4 * kTcBlk;          // 128 rows: 2 blocks hi + 2 blocks lo
constexpr uint32_t kTcBTile = 2 * kTcBlk;          // 64 rows: 1 block hi + 1 block lo
constexpr uint32_t kTcPolls = 1u << 26;

__host__ __device__ __forceinline__ uint32_t cblk_off(int r, int k) {
  return (uint32_t)((((r >> 3) << 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__global__ void pack_a_kernel(const float* __restrict__ A, long long M, long long K, long long kt_n,
                              unsigned char* __restrict__ out, long long tiles) {
  // one thread per (tile, row, k): element A[m][k]
  const long long total = tiles * 128 * 64;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total; j += (long long)gridDim.x * blockDim.x) {
    const long long t = j >> 13;
    const int r = (int)((j >> 6) & 127), k = (int)(j & 63);
    const long long mt = t / kt_n, kt = t % kt_n;
    const long long m = mt * 128 + r, kk = kt * 64 + k;
    const float x = (m < M && kk < K) ? A[m * K + kk] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    unsigned char* base = out + t * kTcATile;
    const uint32_t o = (r >> 6) * kTcBlk + cblk_off(r & 63, k);
    *reinterpret_cast<__nv_bfloat16*>(base + o) = h;
    *reinterpret_cast<__nv_bfloat16*>(base + 2 * kTcBlk + o) = l;
  }
}

__global__ void pack_b_kernel(const float* __restrict__ B, long long K, long long N, long long kt_n,
                              unsigned char* __restrict__ out, long long tiles) {
  const long long total = tiles * 64 * 64;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total; j += (long long)gridDim.x * blockDim.x) {
    const long long t = j >> 12;
    const int r = (int)((j >> 6) & 63), k = (int)(j & 63);  // r: column n of B, k: row k of B
    const long long nt = t / kt_n, kt = t % kt_n;
    const long long n = nt * 64 + r, kk = kt * 64 + k;
    const float x = (n < N && kk < K) ? B[kk * N + n] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    unsigned char* base = out + t * kTcBTile;
    *reinterpret_cast<__nv_bfloat16*>(base + cblk_off(r, k)) = h;
    *reinterpret_cast<__nv_bfloat16*>(base + kTcBlk + cblk_off(r, k)) = l;
  }
}

__global__ void __launch_bounds__(128) gemm_tc_kernel(const unsigned char* __restrict__ Ap,
                                                      const unsigned char* __restrict__ Bp, float* __restrict__ C,
                                                      long long M, long long N, long long kt_n, long long nt_n,
                                                      int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  // stage s: A tile at s * (A + B), B tile after it
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * (kTcATile + kTcBTile));  // load[2], mma[2]
  uint32_t* taddr_s = reinterpret_cast<uint32_t*>(bar + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long mt = blockIdx.x / nt_n, nt = blockIdx.x % nt_n;
  if (warp == 0) {
    ptx::tmem_alloc(taddr_s, 64);
    ptx::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) ptx::mbar_init(bar + i, 1);
    ptx::fence_mbar_init();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *taddr_s;
  bool ok = true;
  if (tid == 0) {
    const uint32_t sb = ptx::smem_u32(sm);
    constexpr uint32_t idesc = ptx::idesc_bf16_f32(128, 64);
    uint32_t ph_load[2] = {0, 0}, ph_mma[2] = {0, 0};
    auto load = [&](long long kt, int s) {
      unsigned char* dst = sm + s * (kTcATile + kTcBTile);
      ptx::mbar_arrive_expect_tx(bar + s, kTcATile + kTcBTile);
      ptx::bulk_g2s(dst, Ap + (mt * kt_n + kt) * kTcATile, kTcATile, bar + s);
      ptx::bulk_g2s(dst + kTcATile, Bp + (nt * kt_n + kt) * kTcBTile, kTcBTile, bar + s);
    };
    load(0, 0);
    for (long long kt = 0; kt < kt_n && ok; ++kt) {
      const int s = (int)(kt & 1);
      if (kt + 1 < kt_n) {
        const int s2 = (int)((kt + 1) & 1);
        if (kt + 1 >= 2) {  // stage s2 was last read by the MMAs of step kt - 1
          ok = ptx::mbar_wait_bounded(bar + 2 + s2, ph_mma[s2], kTcPolls);
          ph_mma[s2] ^= 1;
        }
        if (ok) load(kt + 1, s2);
      }
      if (ok) ok = ptx::mbar_wait_bounded(bar + s, ph_load[s], kTcPolls);
      ph_load[s] ^= 1;
      if (!ok) break;
      ptx::tc_fence_after();
      const uint32_t a = sb + s * (kTcATile + kTcBTile), b = a + kTcATile;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t ko = (uint32_t)(2 * j) * 128;
        const uint32_t acc = (kt > 0 || j > 0) ? 1u : 0u;
        ptx::mma_bf16(tmem, ptx::smem_desc(a + ko, 128, 1024), ptx::smem_desc(b + ko, 128, 1024), idesc, acc);
        ptx::mma_bf16(tmem, ptx::smem_desc(a + 2 * kTcBlk + ko, 128, 1024), ptx::smem_desc(b + ko, 128, 1024), idesc, 1);
        ptx::mma_bf16(tmem, ptx::smem_desc(a + ko, 128, 1024), ptx::smem_desc(b + kTcBlk + ko, 128, 1024), idesc, 1);
      }
      ptx::mma_commit(bar + 2 + s);
    }
    if (ok) {
      // the last commit covers every MMA issued before it
      const int sl = (int)((kt_n - 1) & 1);
      ok = ptx::mbar_wait_bounded(bar + 2 + sl, ph_mma[sl], kTcPolls);
    }
    if (!ok) atomicExch(err, 1);
  }
  ok = __syncthreads_and(tid == 0 ? ok : true);
  ptx::tc_fence_after();
  if (ok) {
    const int row = warp * 32 + lane;
    const long long m = mt * 128 + row;
#pragma unroll
    for (int cb = 0; cb < 4; ++cb) {
      float v[16];
      ptx::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + cb * 16, v);
      ptx::tmem_wait_ld();
      if (m < M) {
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const long long n = nt * 64 + cb * 16 + e;
          if (n < N) C[m * N + n] = v[e];
        }
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

}  // namespace

cudaError_t contract_gemm_tc(const float* A, const float* B, float* C, long long M, long long N, long long K,
                             cudaStream_t st) {
  if (M == 0 || N == 0) return cudaSuccess;
  int m128 = 0, m64 = 0;
  cudaError_t e = tc_run_probe(st, &m128, &m64, nullptr, nullptr);
  if (e != cudaSuccess) return e;
  if (!m128) return cudaErrorNotSupported;
  if (K == 0) return cudaMemsetAsync(C, 0, (size_t)M * N * sizeof(float), st);
  const long long mt_n = (M + 127) / 128, nt_n = (N + 63) / 64, kt_n = (K + 63) / 64;
  if (mt_n * nt_n > 0x7fffffffLL) return cudaErrorInvalidValue;
  unsigned char *Ap = nullptr, *Bp = nullptr;
  e = cudaMallocAsync(&Ap, (size_t)(mt_n * kt_n) * kTcATile, st);
  if (e != cudaSuccess) return e;
  e = cudaMallocAsync(&Bp, (size_t)(nt_n * kt_n) * kTcBTile, st);
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
  pack_a_kernel<<<(int)std::min<long long>((at * 8192 + 255) / 256, 1 << 20), 256, 0, st>>>(A, M, K, kt_n, Ap, at);
  pack_b_kernel<<<(int)std::min<long long>((bt * 4096 + 255) / 256, 1 << 20), 256, 0, st>>>(B, K, N, kt_n, Bp, bt);
  const size_t smem = 2 * (kTcATile + kTcBTile) + 64;
  cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  gemm_tc_kernel<<<(unsigned)(mt_n * nt_n), 128, smem, st>>>(Ap, Bp, C, M, N, kt_n, nt_n, g_tc_err);
  e = cudaGetLastError();
  cudaFreeAsync(Ap, st);
  cudaFreeAsync(Bp, st);
  return e;
}

}  // namespace itn
