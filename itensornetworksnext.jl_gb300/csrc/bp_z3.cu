// bp_z3.cu -- grouped parallel sweep for norm networks whose vertices all have three legs
// (random 3-regular graphs and the like, with uneven bond dimensions up to 8): every message
// update of a sweep, across every network of a batch, in one launch.
//
// The message update is the reference's (beliefpropagation.jl:242-257, factor
// A * conj(A) with the site index shared, normnetwork.jl:49-54):
//   m_{u->v}[b, k] = sum A_u[s, k..] conj(A_u[s, b..]) prod_{w != v} m_{w->u}[b_w, k_w]
// normalised by the sum of its entries unless that sum is zero.  A vertex with legs 0, 1, 2
// (dims D0, D1, D2, tensor A[s][k0][k1][k2]) gets its three outgoing messages from the
// leave-one-out program
//   T0 = A x0 m0;  T01 = T0 x1 m1 -> out2;  T02 = T0 x2 m2 -> out1;
//   T1 = A x1 m1;  T12 = T1 x2 m2 -> out0
// (x_l: absorb the message on leg l into the ket index, leaving its bra index), each "out"
// the contraction of the remaining tensor with conj(A) over everything but the open leg.
//
// A group of 1, 2, 4 or 8 warps owns one vertex at a time, with its site tensor, two work
// buffers and the three incoming messages in its own slice of shared memory; a group
// synchronises with __syncwarp or its own named barrier.  The work list is sorted by tensor
// size and cut into size classes; the launch's CTAs are divided among the classes (a
// "grouped" launch), and each class has its own tile shape: warps per vertex and vertices in
// flight per CTA, chosen so that the class's slices fit the CTA's shared-memory budget with as
// many warps busy as possible.  The host autotuner chooses the budget and the number of CTAs
// by timing sweeps.
#include <cuda_runtime.h>
#include <math.h>

#include "itn_common.cuh"
#include "itn_conv.cuh"
#include "itn_z3.h"

namespace itn {
namespace {

template <typename T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v = add(v, shfl_xor(v, o));
  return v;
}
__device__ __forceinline__ double wsum_d(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Asynchronous copy of one element (4, 8 or 16 bytes) from global to shared memory
// (cp.async); cp_async_wait_all waits for this thread's copies.
template <int B>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  static_assert(B == 4 || B == 8 || B == 16, "cp.async copies 4, 8 or 16 bytes");
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(s), "l"(gmem), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// floor(x / d) for 0 <= x < 4096 and 1 <= d <= 4096 from a float reciprocal: the quotient of
// (x + 0.5) / d stays at least 0.5 / d away from an integer, far more than the rounding error.
__device__ __forceinline__ int qdiv(int x, float inv) { return (int)(((float)x + 0.5f) * inv); }

// A group of `nt` threads (1, 2, 4 or 8 warps) working on one vertex; tid in [0, nt).  One
// warp synchronises with __syncwarp, larger groups with their own named barrier.
struct Grp {
  int tid, nt, bar;
  __device__ __forceinline__ void sync() const {
    if (nt == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nt) : "memory");
  }
};

// dst[o][b][i] = sum_k src[o][k][i] m[b][k]  (n entries, the leg of dimension D with
// `inner` entries after it)
template <typename T>
__device__ __forceinline__ void z3_absorb(const T* src, T* dst, int n, int D, int inner, const T* m, const Grp& g) {
  const float inv_in = 1.f / (float)inner, inv_d = 1.f / (float)D;
  for (int j = g.tid; j < n; j += g.nt) {
    const int t = qdiv(j, inv_in), i = j - t * inner;
    const int o = qdiv(t, inv_d), b = t - o * D;
    const T* sp = src + o * D * inner + i;
    const T* mp = m + b * D;
    T acc = tzero<T>();
    for (int k = 0; k < D; ++k) acc = fmac(sp[k * inner], mp[k], acc);
    dst[j] = acc;
  }
}

// out[b][k] = sum_{o,i} src[o][k][i] conj(A[o][b][i]) over the R = n / D positions (o, i),
// for the leg of dimension D with `inner` entries after it; thread tid returns entries
// q = tid and q = tid + nt (those with q < Q = D * D) in v0, v1.  Q >= nt: each thread sums
// its own entries over every position; Q < nt: G = nt / Q thread sets split the positions and
// their partial sums meet in `red` (nt entries).
template <typename T>
__device__ __forceinline__ void z3_final(const T* src, const T* A, int n, int D, int inner, T* red, const Grp& g,
                                         T& v0, T& v1) {
  const int Q = D * D, R = n / D;
  const float inv_in = 1.f / (float)inner;
  v0 = tzero<T>();
  v1 = tzero<T>();
  // When `inner` is a multiple of 16, threads of different k (or b) reading the same position
  // hit the same shared-memory banks; each thread then walks the positions from its own
  // offset (mod R), so that threads reading at the same moment hit different banks (uniform
  // D = 8 batches: 62.8 -> 58.0 ms per solve).  Other strides keep the plain order.
  const bool spread = (inner & 15) == 0;
  if (Q >= g.nt) {
    for (int h = 0; h < 2; ++h) {
      const int q = g.tid + g.nt * h;
      if (q >= Q) break;
      const int b = q / D, k = q - b * D;
      const int rot = spread ? (k + D * b) % R : 0;
      T acc = tzero<T>();
      int o = qdiv(rot, inv_in), i = rot - o * inner;
      const int O = R / inner;
      for (int r = 0; r < R; ++r) {
        acc = fmac(src[(o * D + k) * inner + i], conjx(A[(o * D + b) * inner + i]), acc);
        if (++i == inner) {
          i = 0;
          if (++o == O) o = 0;
        }
      }
      if (h == 0) v0 = acc;
      else v1 = acc;
    }
    return;
  }
  const int G = g.nt / Q, gs = g.tid / Q, q = g.tid - gs * Q;
  T acc = tzero<T>();
  if (gs < G) {
    const int b = q / D, k = q - b * D;
    const int rot = spread ? (k + D * b) % R : 0;
    for (int r = gs; r < R; r += G) {
      int rr = r + rot;
      if (rr >= R) rr -= R;
      const int o = qdiv(rr, inv_in), i = rr - o * inner;
      acc = fmac(src[(o * D + k) * inner + i], conjx(A[(o * D + b) * inner + i]), acc);
    }
  }
  red[g.tid] = acc;
  g.sync();
  if (g.tid < Q) {
    T s = red[g.tid];
    for (int gg = 1; gg < G; ++gg) s = add(s, red[gg * Q + g.tid]);
    v0 = s;
  }
  g.sync();
}

// Sum of one value over the group (every thread gets it); wred holds one entry per warp.
template <typename T>
__device__ __forceinline__ T grp_sum(T v, T* wred, const Grp& g) {
  v = wsum(v);
  if (g.nt == 32) return v;
  if ((g.tid & 31) == 0) wred[g.tid >> 5] = v;
  g.sync();
  T s = tzero<T>();
  for (int w = 0; w < (g.nt >> 5); ++w) s = add(s, wred[w]);
  g.sync();
  return s;
}
__device__ __forceinline__ double grp_sum_d(double v, double* wred, const Grp& g) {
  v = wsum_d(v);
  if (g.nt == 32) return v;
  if ((g.tid & 31) == 0) wred[g.tid >> 5] = v;
  g.sync();
  double s = 0;
  for (int w = 0; w < (g.nt >> 5); ++w) s += wred[w];
  g.sync();
  return s;
}

// Normalise (sum of entries) and store the message on `slot`; with a convergence test, the
// slot's fidelity diff against the previous message (beliefpropagation.jl:261-267).
template <typename T>
__device__ __forceinline__ void z3_store(const Z3Args& a, int slot, long long mo, int Q, T v0, T v1, T* red,
                                         const Grp& g) {
  const bool has1 = g.tid + g.nt < Q, has0 = g.tid < Q;
  const T s = grp_sum(add(has0 ? v0 : tzero<T>(), has1 ? v1 : tzero<T>()), red, g);
  const bool scale = a.normalize && !is_zero(s);
  T* dst = reinterpret_cast<T*>(a.msg_out) + mo;
  const T* old = reinterpret_cast<const T*>(a.msg_in) + mo;
  double n1 = 0, n2 = 0, dre = 0, dim = 0;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int q = g.tid + g.nt * h;
    if (q >= Q) continue;
    const T v = scale ? divx(h ? v1 : v0, s) : (h ? v1 : v0);
    dst[q] = v;
    if (a.slot_diff) {
      const T ov = old[q];
      const double vr = re_d(v), vi = im_d(v), orr = re_d(ov), oi = im_d(ov);
      n1 += vr * vr + vi * vi;
      n2 += orr * orr + oi * oi;
      dre += vr * orr + vi * oi;
      dim += vr * oi - vi * orr;
    }
  }
  if (a.slot_diff) {
    double* dred = reinterpret_cast<double*>(red);
    n1 = grp_sum_d(n1, dred, g);
    n2 = grp_sum_d(n2, dred, g);
    dre = grp_sum_d(dre, dred, g);
    dim = grp_sum_d(dim, dred, g);
    if (g.tid == 0) {
      const double val = 1.0 - (dre * dre + dim * dim) / (n1 * n2);
      a.slot_diff[slot] = val;
      if (a.conv) {
        if (val != val) atomicExch(&a.conv->nan_flag, 1);
        else atomicMax(&a.conv->dmax, enc_double(val));
        __threadfence();
      }
    }
  }
}

// Copy item `it`'s site tensor into `dst` and its three incoming messages into the staging
// `sm`, synchronously or (ASYNC) with cp.async.
template <typename T, bool ASYNC>
__device__ __forceinline__ void z3_load(const Z3Args& a, int it, T* dst, T* sm, const Grp& g) {
  const Z3Meta& mt = a.meta[it];
  const T* A = reinterpret_cast<const T*>(a.tens) + mt.t0;
  const T* min_ = reinterpret_cast<const T*>(a.msg_in);
  for (int j = g.tid; j < mt.n; j += g.nt) {
    if constexpr (ASYNC) cp_async<sizeof(T)>(dst + j, A + j);
    else dst[j] = A[j];
  }
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    const T* m = min_ + mt.moff_in[l];
    for (int j = g.tid; j < mt.D[l] * mt.D[l]; j += g.nt) {
      if constexpr (ASYNC) cp_async<sizeof(T)>(sm + 64 * l + j, m + j);
      else sm[64 * l + j] = m[j];
    }
  }
}

// The three updates of work item `it` (one vertex) by one group (slice: A, two buffers of nmax
// entries, three messages of up to 64 entries, 256 reduction entries).  `loaded`: the tensor
// and messages are already in sA and sm (prefetched by the previous item).  `next` >= 0: once
// the last absorption is done, sB and sm are free, and the next item's tensor and messages are
// copied into them asynchronously while this item's last contraction and store run; the
// caller swaps sA and sB.
template <typename T>
__device__ void z3_item(const Z3Args& a, int it, int next, bool loaded, T* sA, T* sB, T* sC, T* sm, T* red,
                        const Grp& g) {
  const Z3Meta& mt = a.meta[it];
  const int s0 = mt.s0, n = mt.n;
  const int D0 = mt.D[0], D1 = mt.D[1], D2 = mt.D[2];
  if (!loaded) {
    z3_load<T, false>(a, it, sA, sm, g);
    g.sync();
  }
  const int in0 = D1 * D2, in1 = D2, in2 = 1;
  T v0, v1;
  z3_absorb(sA, sB, n, D0, in0, sm, g);  // T0
  g.sync();
  z3_absorb(sB, sC, n, D1, in1, sm + 64, g);  // T01
  g.sync();
  z3_final(sC, sA, n, D2, in2, red, g, v0, v1);
  z3_store(a, s0 + 2, mt.moff_out[2], D2 * D2, v0, v1, red, g);
  z3_absorb(sB, sC, n, D2, in2, sm + 128, g);  // T02
  g.sync();
  z3_final(sC, sA, n, D1, in1, red, g, v0, v1);
  z3_store(a, s0 + 1, mt.moff_out[1], D1 * D1, v0, v1, red, g);
  z3_absorb(sA, sB, n, D1, in1, sm + 64, g);  // T1
  g.sync();
  z3_absorb(sB, sC, n, D2, in2, sm + 128, g);  // T12
  g.sync();
  if (next >= 0) z3_load<T, true>(a, next, sB, sm, g);
  z3_final(sC, sA, n, D0, in0, red, g, v0, v1);
  z3_store(a, s0, mt.moff_out[0], D0 * D0, v0, v1, red, g);
  if (next >= 0) cp_async_wait_all();
  g.sync();  // the slice is reused by the group's next vertex
}

template <typename T>
__global__ void __launch_bounds__(kZ3Threads) sweep_z3_kernel(Z3Args a) {
  extern __shared__ __align__(16) unsigned char z3s[];
  if (a.conv && *reinterpret_cast<const volatile int*>(&a.conv->done)) return;
  const int warp = threadIdx.x >> 5;
  int k = 0;
  while (k + 1 < a.n_classes && (int)blockIdx.x >= a.cls[k + 1].cta_start) ++k;
  const Z3Class c = a.cls[k];
  // groups of c.wpi warps; the first c.groups of them are active
  const int grp = warp / c.wpi;
  if (grp < c.groups) {
    Grp g;
    g.nt = 32 * c.wpi;
    g.tid = (int)threadIdx.x - grp * g.nt;
    g.bar = 1 + grp;
    T* base = reinterpret_cast<T*>(z3s) + (size_t)grp * c.slice;
    T* sA = base;
    T* sB = sA + c.nmax;
    T* sC = sB + c.nmax;
    T* sm = sC + c.nmax;
    T* red = sm + 192;
    const int gw = ((int)blockIdx.x - c.cta_start) * c.groups + grp, nw = c.ctas * c.groups;
    bool loaded = false;
    const int end = c.first + c.count;
    for (int it = c.first + gw; it < end; it += nw) {
      const int next = it + nw < end ? it + nw : -1;
      z3_item<T>(a, it, next, loaded, sA, sB, sC, sm, red, g);
      loaded = next >= 0;
      T* tmp = sA;
      sA = sB;
      sB = tmp;
    }
  }
  if (a.conv) conv_finish_cta(a.conv);
}

template <typename T>
cudaError_t launch_t(const Z3Args& a, int grid, size_t smem, cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(sweep_z3_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kZ3MaxSmem);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(sweep_z3_kernel<T>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    configured = true;
  }
  sweep_z3_kernel<T><<<grid, kZ3Threads, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

int z3_blocks_per_sm(int dtype, size_t smem) {
  int n = 0;
  cudaError_t e = cudaErrorInvalidValue;
  switch (dtype) {
    case 0:
      cudaFuncSetAttribute(sweep_z3_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZ3MaxSmem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_z3_kernel<float>, kZ3Threads, smem);
      break;
    case 1:
      cudaFuncSetAttribute(sweep_z3_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZ3MaxSmem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_z3_kernel<double>, kZ3Threads, smem);
      break;
    case 2:
      cudaFuncSetAttribute(sweep_z3_kernel<c64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZ3MaxSmem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_z3_kernel<c64>, kZ3Threads, smem);
      break;
    case 3:
      cudaFuncSetAttribute(sweep_z3_kernel<c128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZ3MaxSmem);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep_z3_kernel<c128>, kZ3Threads, smem);
      break;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

cudaError_t launch_sweep_z3(int dtype, const Z3Args& a, int grid, size_t smem, cudaStream_t st) {
  if (grid <= 0) return cudaSuccess;
  if (smem > kZ3MaxSmem) return cudaErrorInvalidValue;
  switch (dtype) {
    case 0: return launch_t<float>(a, grid, smem, st);
    case 1: return launch_t<double>(a, grid, smem, st);
    case 2: return launch_t<c64>(a, grid, smem, st);
    case 3: return launch_t<c128>(a, grid, smem, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace itn
