// bp_generic.cu -- CUDA-core belief-propagation kernels for any graph, bond dimensions
// and element type (float, double, complex64, complex128).
//
// Two-layer (norm network) message update, reference semantics
// (src/beliefpropagation/beliefpropagation.jl:242-257 with the factor of
// src/normnetwork.jl:49-54):
//   m_{u->v}[b, k] = sum A_u[s, k_1..k_z] conj(A_u[s, b_1..b_z]) prod_{w != v} m_{w->u}[b_w, k_w]
// with (b_v, k_v) = (b, k) left open, then m /= sum(m) unless the sum is zero.
//
// One CTA owns one vertex at a time (persistent loop over work items).  The vertex's
// site tensor and its incoming messages are staged in shared memory and an op-program
// built on the host is interpreted:
//   ABSORB(src, dst, w): dst[o][b][i] = sum_k src[o][k][i] * m_w[b][k]   (ket leg w -> bra)
//   FINAL(src, v)      : out[b][k] = sum_{o,i} src[o][k][i] * conj(A[o][b][i]), normalise, store
//   FULL(src)          : Z_u = sum_j src[j] * conj(A[j])  (vertex_scalar, messagecache.jl:139-143)
// The host program absorbs legs in a leave-one-out binary split, so the z outgoing
// messages of a vertex share partial products (8 absorptions instead of 12 at z = 4).
//
// One-layer networks (plain ITensorNetwork factors, vector messages) use a direct
// per-entry kernel; they are small known-answer cases (spin ice, Ising, trees).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <type_traits>

#include "itn_common.cuh"
#include "itn_conv.cuh"
#include "itn_internal.h"
#include "tc_ptx.cuh"

namespace itn {

namespace {

constexpr int kRedWidth = 64;  // per-warp partial-sum slots for D*D <= 64

struct LegMeta {
  uint64_t bar;            // mbarrier of the bulk copy of the site tensor
  unsigned phase;          // its current phase parity
  int bulk;                // the site tensor of the current item arrives by bulk copy
  int z, d, n;          // legs, physical dim, tensor elements
  int s0, mtot;         // first slot of the vertex; message entries staged
  int dims[kMaxLegs];
  int inner[kMaxLegs];  // prod of dims after the leg
  int outer[kMaxLegs];  // d * prod of dims before the leg
  int moffs[kMaxLegs];  // offset of the leg's incoming message in shared staging
  long long msrc[kMaxLegs];  // offset of the incoming message m_{w->u} (slot rev(s0 + l))
  long long tsrc[kMaxLegs];  // offset of the outgoing slot s0 + l (tangents of the dual kernel)
};

// Per-item set-up shared by the two-layer kernels, done by warp 0 alone and followed by
// one barrier: (1) every lane reads the vertex's slot range and physical dimension, and
// lane 0 starts the bulk copy of the site tensor into buffer 0 when `allow_bulk` and the
// tensor is 16-byte aligned and 4 KB .. 1 MB; (2) lane l < z reads leg l's bond dimension
// and incoming-message offset; (3) the prefix sums / products of the legs by shuffles.
template <typename T, bool DUAL>
__device__ void item_meta(const GenericArgs& a, int u, LegMeta* meta, T* A, bool allow_bulk) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int s0 = a.off[u], z = a.off[u + 1] - s0, dph = a.phys[u];
    if (lane == 0) {
      const long long t0 = a.toff[u], tn = a.toff[u + 1] - t0;
      const bool bulk = allow_bulk && ((t0 * (long long)sizeof(T)) & 15) == 0 &&
                        ((tn * (long long)sizeof(T)) & 15) == 0 && tn * (long long)sizeof(T) >= 4096 &&
                        tn * (long long)sizeof(T) < (1ll << 20);
      meta->bulk = bulk;
      if (bulk) {
        const T* A_g = reinterpret_cast<const T*>(a.tens) + t0;
        ptx::fence_proxy_async_smem();  // earlier generic accesses to buffer 0 come first
        ptx::mbar_arrive_expect_tx(&meta->bar, (uint32_t)(tn * sizeof(T)));
        ptx::bulk_g2s(A, A_g, (uint32_t)(tn * sizeof(T)), &meta->bar);
      }
    }
    int dim = 1;
    if (lane < z) {
      dim = a.bond[s0 + lane];
      meta->msrc[lane] = a.moff[a.rev[s0 + lane]];
      if (DUAL) meta->tsrc[lane] = a.moff[s0 + lane];
    }
    // exclusive prefix sum of dim^2 (message offsets) and inclusive suffix product of dim
    const int sq = lane < z ? dim * dim : 0;
    int psum = sq, sprod = dim;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int up = __shfl_up_sync(0xffffffffu, psum, o);
      const int dn = __shfl_down_sync(0xffffffffu, sprod, o);
      if (lane >= o) psum += up;
      if (lane + o < 32) sprod *= dn;
    }
    const int inner = __shfl_down_sync(0xffffffffu, sprod, 1);  // product of the dims after the leg
    const int all = __shfl_sync(0xffffffffu, sprod, 0);
    const int tot = __shfl_sync(0xffffffffu, psum, 31);
    const int n = dph * all;
    if (lane < z) {
      const int in = lane == 31 ? 1 : inner;
      meta->dims[lane] = dim;
      meta->moffs[lane] = psum - sq;
      meta->inner[lane] = in;
      meta->outer[lane] = n / (in * dim);
    }
    if (lane == 0) {
      meta->s0 = s0;
      meta->z = z;
      meta->d = dph;
      meta->n = n;
      meta->mtot = tot;
    }
  }
  __syncthreads();
}

// Leg of staged message entry j (messages staged back to back in leg order).
__device__ __forceinline__ int staged_leg(const LegMeta* meta, int j) {
  int l = 0;
  while (l + 1 < meta->z && j >= meta->moffs[l + 1]) ++l;
  return l;
}

// ---- warp reduce-scatter of NV (power of two) values -------------------------------
// After the call, lane holds in v[j] (j < max(NV/32, 1)) the warp sum of index base+j.
template <typename T, int NV, int STEP>
__device__ __forceinline__ void rs_step(T (&v)[NV], int lane, int& base) {
  if constexpr (STEP < 5) {
    constexpr int off = 16 >> STEP;
    constexpr int cnt = NV >> (STEP + 1);
    if constexpr (cnt >= 1) {
      const bool up = (lane & off) != 0;
#pragma unroll
      for (int j = 0; j < cnt; ++j) {
        T send = up ? v[j] : v[j + cnt];
        T keep = up ? v[j + cnt] : v[j];
        v[j] = add(keep, shfl_xor(send, off));
      }
      if (up) base += cnt;
    } else {
      v[0] = add(v[0], shfl_xor(v[0], off));
    }
    rs_step<T, NV, STEP + 1>(v, lane, base);
  }
}

template <int D> struct Pow2Of { static constexpr int v = (D * D <= 1) ? 1 : (D * D <= 2) ? 2 : (D * D <= 4) ? 4 : (D * D <= 8) ? 8 : (D * D <= 16) ? 16 : (D * D <= 32) ? 32 : 64; };

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v = add(v, shfl_xor(v, o));
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one value; result valid in every thread.  red needs nwarps slots.
template <typename T>
__device__ T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T r = tzero<T>();
  for (int w = 0; w < nw; ++w) r = add(r, red[w]);
  __syncthreads();
  return r;
}

// Row of D contiguous elements (the innermost leg): 16-byte vector accesses when the row
// length is a multiple of 16 bytes (rows then start 16-byte aligned in the buffers).
template <typename T, int D>
__device__ __forceinline__ void load_row(const T* __restrict__ p, T (&t)[D]) {
  if constexpr ((D * sizeof(T)) % 16 == 0) {
    constexpr int nv = D * sizeof(T) / 16;
    uint4 v[nv];
#pragma unroll
    for (int j = 0; j < nv; ++j) v[j] = reinterpret_cast<const uint4*>(p)[j];
    memcpy(t, v, sizeof(v));
  } else {
#pragma unroll
    for (int k = 0; k < D; ++k) t[k] = p[k];
  }
}
template <typename T, int D>
__device__ __forceinline__ void store_row(T* __restrict__ p, const T (&t)[D]) {
  if constexpr ((D * sizeof(T)) % 16 == 0) {
    constexpr int nv = D * sizeof(T) / 16;
    uint4 v[nv];
    memcpy(v, t, sizeof(v));
#pragma unroll
    for (int j = 0; j < nv; ++j) reinterpret_cast<uint4*>(p)[j] = v[j];
  } else {
#pragma unroll
    for (int k = 0; k < D; ++k) p[k] = t[k];
  }
}

// Thread-strided walk p = threadIdx.x, +blockDim.x, ... over p = o * inner + i.  Real types
// step (o, i) by additions instead of an integer division per element (6% on the FP32
// 32x32 D=8 sweep); complex types divide per element as before, with no state carried:
// their D-specialised paths are bound by instruction fetch, and carrying the walk measured
// 5% slower on the batched complex64 networks.
template <typename T, bool INC = !is_cplx<T>::value>
struct OiWalk {
  int o, i, bo, bi, inner;
  __device__ __forceinline__ explicit OiWalk(int inner_) : inner(inner_) {
    const int p0 = (int)threadIdx.x, st = (int)blockDim.x;
    o = p0 / inner_;
    i = p0 - o * inner_;
    bo = st / inner_;
    bi = st - bo * inner_;
  }
  __device__ __forceinline__ void get(int, int& oo, int& ii) const {
    oo = o;
    ii = i;
  }
  __device__ __forceinline__ void next() {
    o += bo;
    i += bi;
    if (i >= inner) {
      i -= inner;
      ++o;
    }
  }
};
template <typename T>
struct OiWalk<T, false> {
  int inner;
  __device__ __forceinline__ explicit OiWalk(int inner_) : inner(inner_) {}
  __device__ __forceinline__ void get(int p, int& oo, int& ii) const {
    oo = p / inner;
    ii = p - oo * inner;
  }
  __device__ __forceinline__ void next() {}
};

// ---- ABSORB with compile-time bond dimension ---------------------------------------
template <typename T, int D>
__device__ __forceinline__ void absorb_fixed(const T* __restrict__ src, T* __restrict__ dst,
                                             int outer, int inner, const T* __restrict__ m) {
  T mr[D * D];
#pragma unroll
  for (int j = 0; j < D * D; ++j) mr[j] = m[j];
  const int n = outer * inner;
  if (inner == 1) {  // innermost leg: whole rows per thread, vector accesses
    for (int o = threadIdx.x; o < outer; o += blockDim.x) {
      T t[D], r[D];
      load_row<T, D>(src + o * D, t);
#pragma unroll
      for (int b = 0; b < D; ++b) {
        T acc = mul(t[0], mr[b * D]);
#pragma unroll
        for (int k = 1; k < D; ++k) acc = fmac(t[k], mr[b * D + k], acc);
        r[b] = acc;
      }
      store_row<T, D>(dst + o * D, r);
    }
    return;
  }
  OiWalk<T> w(inner);
  for (int p = threadIdx.x; p < n; p += blockDim.x, w.next()) {
    int o, i;
    w.get(p, o, i);
    const T* s = src + o * D * inner + i;
    T t[D];
#pragma unroll
    for (int k = 0; k < D; ++k) t[k] = s[k * inner];
    T* dd = dst + o * D * inner + i;
#pragma unroll
    for (int b = 0; b < D; ++b) {
      T acc = mul(t[0], mr[b * D]);
#pragma unroll
      for (int k = 1; k < D; ++k) acc = fmac(t[k], mr[b * D + k], acc);
      dd[b * inner] = acc;
    }
  }
}

template <typename T>
__device__ void absorb_rt(const T* __restrict__ src, T* __restrict__ dst, int outer, int D,
                          int inner, const T* __restrict__ m) {
  const int n = outer * inner;
  OiWalk<T> w(inner);
  for (int p = threadIdx.x; p < n; p += blockDim.x, w.next()) {
    int o, i;
    w.get(p, o, i);
    const T* s = src + o * D * inner + i;
    T* dd = dst + o * D * inner + i;
    for (int b = 0; b < D; ++b) {
      T acc = tzero<T>();
      for (int k = 0; k < D; ++k) acc = fmac(s[k * inner], m[b * D + k], acc);
      dd[b * inner] = acc;
    }
  }
}

// ---- FINAL with compile-time bond dimension: out[b][k] -------------------------------
template <typename T, int D>
__device__ __forceinline__ void final_fixed(const T* __restrict__ src, const T* __restrict__ A,
                                            int outer, int inner, T* __restrict__ out,
                                            T* __restrict__ red) {
  constexpr int NV = Pow2Of<D>::v;
  T acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) acc[j] = tzero<T>();
  const int n = outer * inner;
  OiWalk<T> w(inner);
  for (int p = threadIdx.x; p < n; p += blockDim.x, w.next()) {
    int o, i;
    w.get(p, o, i);
    const T* s = src + o * D * inner + i;
    const T* a = A + o * D * inner + i;
    T t[D], c[D];
    if (inner == 1) {
      load_row<T, D>(s, t);
      load_row<T, D>(a, c);
#pragma unroll
      for (int b = 0; b < D; ++b) c[b] = conjx(c[b]);
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) t[k] = s[k * inner];
#pragma unroll
      for (int b = 0; b < D; ++b) c[b] = conjx(a[b * inner]);
    }
#pragma unroll
    for (int b = 0; b < D; ++b)
#pragma unroll
      for (int k = 0; k < D; ++k) acc[b * D + k] = fmac(t[k], c[b], acc[b * D + k]);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int base = 0;
  rs_step<T, NV, 0>(acc, lane, base);
  constexpr int keep = NV >= 32 ? NV / 32 : 1;
#pragma unroll
  for (int j = 0; j < keep; ++j) red[warp * kRedWidth + base + j] = acc[j];
  __syncthreads();
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    T r = tzero<T>();
    for (int w = 0; w < nw; ++w) r = add(r, red[w * kRedWidth + e]);
    out[e] = r;
  }
  __syncthreads();
}

template <typename T>
__device__ void final_rt(const T* __restrict__ src, const T* __restrict__ A, int outer, int D,
                         int inner, T* __restrict__ out, T* __restrict__ red) {
  const int n = outer * inner;
  for (int e = 0; e < D * D; ++e) {
    const int b = e / D, k = e - b * D;
    T acc = tzero<T>();
    OiWalk<T> w(inner);
    for (int p = threadIdx.x; p < n; p += blockDim.x, w.next()) {
      int o, i;
      w.get(p, o, i);
      acc = fmac(src[(o * D + k) * inner + i], conjx(A[(o * D + b) * inner + i]), acc);
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) out[e] = acc;
  }
  __syncthreads();
}

// Grid-wide barrier number k (1, 2, ...) of a persistent cooperative launch (every CTA
// resident): each CTA adds one arrival to a 64-bit counter that is zeroed before the launch
// and never reset during it, and barrier k is passed once the counter has reached
// k * gridDim.x.  The last CTA to arrive sees that in its own atomic's result and leaves at
// once; the others poll the counter.  The fence before the arrival (after the CTA barrier, so
// it covers every thread's writes) and the one after the wait order the launch's global
// writes across the barrier.  The wait is bounded by elapsed time (globaltimer, checked every
// 64 polls, when it also gives up once another CTA has raised *err); false means the launch
// must stop.
__device__ bool grid_barrier(unsigned long long* arrivals, unsigned k, int* err, unsigned long long wait_ns) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned long long target = (unsigned long long)k * gridDim.x;
    __threadfence();
    if (atomicAdd(arrivals, 1ull) + 1 < target) {
      volatile unsigned long long* cnt = arrivals;
      const uint64_t t0 = ptx::globaltimer();
      for (unsigned polls = 1; *cnt < target; ++polls) {
        if ((polls & 63) == 0) {
          if (*reinterpret_cast<volatile int*>(err)) {
            ok = 0;
            break;
          }
          if (ptx::globaltimer() - t0 > wait_ns) {
            atomicExch(err, 1);
            ok = 0;
            break;
          }
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Normalise out (D*D entries in shared memory) by its sum, store it to global memory
// and, when requested, record the convergence value against the previous message.
// Executed by warp 0.
template <typename T>
__device__ void store_message(const GenericArgs& a, const T* out, int n, int slot, const void* msg_in,
                              void* msg_out, unsigned long long* dmax, int* nanf) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x >= 32) return;
  T s = tzero<T>();
  for (int j = lane; j < n; j += 32) s = add(s, out[j]);
  s = warp_sum(s);
  const bool scale = a.normalize && !is_zero(s);
  T* dst = reinterpret_cast<T*>(msg_out) + a.moff[slot];
  const T* old = reinterpret_cast<const T*>(msg_in) + a.moff[slot];
  double n1 = 0, n2 = 0, dre = 0, dim = 0;
  for (int j = lane; j < n; j += 32) {
    T v = scale ? divx(out[j], s) : out[j];
    if (a.slot_diff) {
      T ov = old[j];
      const double vr = re_d(v), vi = im_d(v), orr = re_d(ov), oi = im_d(ov);
      n1 += vr * vr + vi * vi;
      n2 += orr * orr + oi * oi;
      dre += vr * orr + vi * oi;   // conj(v) * ov
      dim += vr * oi - vi * orr;
    }
    dst[j] = v;
  }
  if (a.slot_diff) {
    n1 = warp_sum_d(n1);
    n2 = warp_sum_d(n2);
    dre = warp_sum_d(dre);
    dim = warp_sum_d(dim);
    if (lane == 0) {
      const double val = 1.0 - (dre * dre + dim * dim) / (n1 * n2);
      a.slot_diff[slot] = val;
      if (dmax) {
        if (val != val) atomicExch(nanf, 1);
        else atomicMax(dmax, enc_double(val));
        __threadfence();
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void dispatch_absorb(const T* src, T* dst, int outer, int D, int inner,
                                                const T* m) {
  switch (D) {
    case 1: absorb_fixed<T, 1>(src, dst, outer, inner, m); break;
    case 2: absorb_fixed<T, 2>(src, dst, outer, inner, m); break;
    case 3: absorb_fixed<T, 3>(src, dst, outer, inner, m); break;
    case 4: absorb_fixed<T, 4>(src, dst, outer, inner, m); break;
    case 5: absorb_fixed<T, 5>(src, dst, outer, inner, m); break;
    case 6: absorb_fixed<T, 6>(src, dst, outer, inner, m); break;
    case 7: absorb_fixed<T, 7>(src, dst, outer, inner, m); break;
    case 8: absorb_fixed<T, 8>(src, dst, outer, inner, m); break;
    default: absorb_rt<T>(src, dst, outer, D, inner, m); break;
  }
}

template <typename T>
__device__ __forceinline__ void dispatch_final(const T* src, const T* A, int outer, int D,
                                               int inner, T* out, T* red) {
  switch (D) {
    case 1: final_fixed<T, 1>(src, A, outer, inner, out, red); break;
    case 2: final_fixed<T, 2>(src, A, outer, inner, out, red); break;
    case 3: final_fixed<T, 3>(src, A, outer, inner, out, red); break;
    case 4: final_fixed<T, 4>(src, A, outer, inner, out, red); break;
    case 5: final_fixed<T, 5>(src, A, outer, inner, out, red); break;
    case 6: final_fixed<T, 6>(src, A, outer, inner, out, red); break;
    case 7: final_fixed<T, 7>(src, A, outer, inner, out, red); break;
    case 8: final_fixed<T, 8>(src, A, outer, inner, out, red); break;
    default: final_rt<T>(src, A, outer, D, inner, out, red); break;
  }
}

// Shared-memory carve-up (all regions 16-byte aligned).
struct SmemLayout {
  size_t bufs, msgs, out, red, meta, total;
};
template <typename T>
__host__ __device__ inline SmemLayout smem_layout(const GenericArgs& a, int block, bool in_smem) {
  auto up = [](size_t x) { return (x + 15) & ~size_t(15); };
  SmemLayout L;
  size_t o = 0;
  L.bufs = o;
  if (in_smem) o += up((size_t)a.nbuf * a.buf_elems * sizeof(T));
  L.msgs = o;
  o += up((size_t)a.msg_cap * sizeof(T));
  L.out = o;
  o += up((size_t)(a.max_d2 > 0 ? a.max_d2 : 1) * sizeof(T));
  L.red = o;
  o += up((size_t)(block / 32) * kRedWidth * sizeof(T));
  L.meta = o;
  o += up(sizeof(LegMeta));
  L.total = o;
  return L;
}

// ---- the two-layer interpreter ---------------------------------------------------------
// MINB = 2 caps registers at 128 (see bp2_kernel_for)
template <typename T, int MINB>
__global__ void __launch_bounds__(256, MINB) bp2_kernel(GenericArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SmemLayout L = smem_layout<T>(a, blockDim.x, a.gscratch == nullptr);
  T* bufs = a.gscratch ? reinterpret_cast<T*>(a.gscratch) + (size_t)blockIdx.x * a.nbuf * a.buf_elems
                       : reinterpret_cast<T*>(smem + L.bufs);
  T* msgs = reinterpret_cast<T*>(smem + L.msgs);
  T* out = reinterpret_cast<T*>(smem + L.out);
  T* red = reinterpret_cast<T*>(smem + L.red);
  LegMeta* meta = reinterpret_cast<LegMeta*>(smem + L.meta);
  const T* tens = reinterpret_cast<const T*>(a.tens);
  const T* min_ = reinterpret_cast<const T*>(a.msg_in);

  if (a.conv && *reinterpret_cast<const volatile int*>(&a.conv->done)) return;
  const bool persist = a.pgrid != nullptr;
  const int base_iter = persist && a.conv ? a.conv->counter : 0;
  if (threadIdx.x == 0) {
    ptx::mbar_init(&meta->bar, 1);
    ptx::fence_mbar_init();
    meta->phase = 0;
  }
  __syncthreads();

  for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
    const int u = a.items[2 * it];
    const unsigned* prog = a.prog + a.items[2 * it + 1];
    // the site tensor goes to buffer 0 (a 16-byte aligned tensor in shared-memory buffers
    // by one bulk copy, started inside item_meta), the incoming messages m_{w->u} to the
    // staging area
    T* A = bufs;
    item_meta<T, false>(a, u, meta, A, a.gscratch == nullptr);
    const int n = meta->n;
    const T* A_g = tens + a.toff[u];
    const bool bulk = meta->bulk != 0;
    if (!bulk)
      for (int j = threadIdx.x; j < n; j += blockDim.x) A[j] = A_g[j];
    const int s0 = meta->s0;
    const T* min0 = persist ? reinterpret_cast<const T*>(a.msg_buf[0]) : min_;
    for (int j = threadIdx.x; j < meta->mtot; j += blockDim.x) {
      const int l = staged_leg(meta, j);
      msgs[j] = min0[meta->msrc[l] + (j - meta->moffs[l])];
    }
    if (bulk) {
      // bounded wait; on timeout the copy is re-done with plain loads
      if (!__syncthreads_and(ptx::mbar_wait_bounded(&meta->bar, meta->phase, 1u << 26))) {
        for (int j = threadIdx.x; j < n; j += blockDim.x) A[j] = A_g[j];
      }
      if (threadIdx.x == 0) meta->phase ^= 1;
    }
    __syncthreads();
    for (int sw = 0;; ++sw) {
    // sweep sw of a persistent launch reads msg_buf[sw & 1] and writes msg_buf[(sw + 1) & 1]
    const void* io_in = persist ? a.msg_buf[sw & 1] : a.msg_in;
    void* io_out = persist ? a.msg_buf[(sw + 1) & 1] : a.msg_out;
    unsigned long long* io_dmax = persist ? &a.pgrid->dmax[sw % 3] : a.conv ? &a.conv->dmax : nullptr;
    int* io_nan = persist ? &a.pgrid->nanf[sw % 3] : a.conv ? &a.conv->nan_flag : nullptr;
    const int nops = (int)prog[0];
    for (int q = 1; q <= nops; ++q) {
      const unsigned op = prog[q];
      const int type = op >> 28, srcb = (op >> 20) & 0xff, dstb = (op >> 12) & 0xff,
                leg = op & 0xfff;
      const T* src = bufs + (size_t)srcb * a.buf_elems;
      if (type == OP_ABSORB) {
        T* dst = bufs + (size_t)dstb * a.buf_elems;
        dispatch_absorb<T>(src, dst, meta->outer[leg], meta->dims[leg], meta->inner[leg],
                           msgs + meta->moffs[leg]);
        __syncthreads();
      } else if (type == OP_FINAL) {
        const int D = meta->dims[leg];
        dispatch_final<T>(src, A, meta->outer[leg], D, meta->inner[leg], out, red);
        store_message<T>(a, out, D * D, s0 + leg, io_in, io_out, io_dmax, io_nan);
        __syncthreads();
      } else {  // OP_FULL
        T acc = tzero<T>();
        for (int j = threadIdx.x; j < n; j += blockDim.x) acc = fmac(src[j], conjx(A[j]), acc);
        acc = block_sum(acc, red);
        if (threadIdx.x == 0) reinterpret_cast<T*>(a.zv_out)[u] = acc;
        __syncthreads();
      }
    }
    __syncthreads();
    if (!persist) break;
    if (a.pstall && sw == 0 && blockIdx.x == 0) break;
    // end of a persistent sweep: wait for every CTA, then every CTA takes the outer-loop step
    // of conv_step from this sweep's diff maximum (the same decision everywhere)
    if (!grid_barrier(&a.pgrid->arrivals, sw + 1, &a.pgrid->err, a.wait_ns)) break;
    const int k3 = sw % 3;
    const int iter = base_iter + sw + 1;
    const bool last = sw + 1 >= a.nsweeps;
    if (!last) {
      // the next sweep's incoming messages (the site tensor stays staged), loaded before the
      // diff maximum is read so that the two reads overlap; unused if the run stops here
      const T* mk = reinterpret_cast<const T*>(a.msg_buf[(sw + 1) & 1]);
      for (int j = threadIdx.x; j < meta->mtot; j += blockDim.x) {
        const int l = staged_leg(meta, j);
        msgs[j] = mk[meta->msrc[l] + (j - meta->moffs[l])];
      }
    }
    double delta = 0.0;
    bool conv_now = false;
    if (a.conv && a.conv->use_tol) {
      delta = *reinterpret_cast<volatile int*>(&a.pgrid->nanf[k3])
                  ? nan("")
                  : dec_double(*reinterpret_cast<volatile unsigned long long*>(&a.pgrid->dmax[k3]));
      conv_now = delta < a.conv->tol;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (a.conv) {
        a.conv->counter = iter;
        a.conv->iters = iter;
        if (a.conv->use_tol) {
          a.conv->delta = delta;
          if (conv_now) {
            a.conv->done = 1;
            a.conv->at_iter = iter;
          }
        }
      }
      a.pgrid->dmax[(sw + 2) % 3] = enc_double(-INFINITY);
      a.pgrid->nanf[(sw + 2) % 3] = 0;
      __threadfence();
    }
    __syncthreads();  // the restaged messages
    if (last || conv_now) break;
    }  // persistent sweeps
  }
  if (a.conv && a.fused_step && !persist) conv_finish_cta(a.conv);
}

// ---- dual-number interpreter (real types): value and tangent planes ------------------------
// Forward-mode companion of bp2_kernel used by the adjoint / gradient path.  Every logical
// buffer b has a value plane (b) and a tangent plane (b + nbuf); the site tensor (buffer 0)
// has no tangent.  Leg l is absorbed with (m_l, dm_l): the value message m_{w->u} from the
// incoming slot and the tangent from d.tan_in at the *outgoing* slot u -> w.
//   FINAL(src, w): the tangent part of the message on leg w, unnormalised, stored at the
//                  incoming slot rev(u -> w) of d.tan_out (the cotangent of m_{w->u});
//   DUMP(src)    : grad[u] += plane(src) * (dump_tangent ? 1 : 1 / Z_u).
template <typename T, int D>
__device__ __forceinline__ void absorb_dual_fixed(const T* __restrict__ src, const T* __restrict__ srcT,
                                                  T* __restrict__ dst, T* __restrict__ dstT, int outer,
                                                  int inner, const T* __restrict__ m,
                                                  const T* __restrict__ dm) {
  T mr[D * D], dr[D * D];
#pragma unroll
  for (int j = 0; j < D * D; ++j) {
    mr[j] = m[j];
    dr[j] = dm[j];
  }
  const int n = outer * inner;
  OiWalk<T> w(inner);
  for (int p = threadIdx.x; p < n; p += blockDim.x, w.next()) {
    int o, i;
    w.get(p, o, i);
    const int base = o * D * inner + i;
    T t[D], dt[D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      t[k] = src[base + k * inner];
      dt[k] = srcT ? srcT[base + k * inner] : T(0);
    }
#pragma unroll
    for (int b = 0; b < D; ++b) {
      T acc = 0, dacc = 0;
#pragma unroll
      for (int k = 0; k < D; ++k) {
        acc = fmac(t[k], mr[b * D + k], acc);
        dacc = fmac(dt[k], mr[b * D + k], fmac(t[k], dr[b * D + k], dacc));
      }
      dst[base + b * inner] = acc;
      dstT[base + b * inner] = dacc;
    }
  }
}

template <typename T>
__device__ void absorb_dual_rt(const T* __restrict__ src, const T* __restrict__ srcT, T* __restrict__ dst,
                               T* __restrict__ dstT, int outer, int D, int inner, const T* __restrict__ m,
                               const T* __restrict__ dm) {
  const int n = outer * inner;
  OiWalk<T> w(inner);
  for (int p = threadIdx.x; p < n; p += blockDim.x, w.next()) {
    int o, i;
    w.get(p, o, i);
    const int base = o * D * inner + i;
    for (int b = 0; b < D; ++b) {
      T acc = 0, dacc = 0;
      for (int k = 0; k < D; ++k) {
        const T t = src[base + k * inner], dt = srcT ? srcT[base + k * inner] : T(0);
        acc = fmac(t, m[b * D + k], acc);
        dacc = fmac(dt, m[b * D + k], fmac(t, dm[b * D + k], dacc));
      }
      dst[base + b * inner] = acc;
      dstT[base + b * inner] = dacc;
    }
  }
}

template <typename T>
__device__ __forceinline__ void dispatch_absorb_dual(const T* src, const T* srcT, T* dst, T* dstT, int outer,
                                                     int D, int inner, const T* m, const T* dm) {
  switch (D) {
    case 2: absorb_dual_fixed<T, 2>(src, srcT, dst, dstT, outer, inner, m, dm); break;
    case 3: absorb_dual_fixed<T, 3>(src, srcT, dst, dstT, outer, inner, m, dm); break;
    case 4: absorb_dual_fixed<T, 4>(src, srcT, dst, dstT, outer, inner, m, dm); break;
    case 6: absorb_dual_fixed<T, 6>(src, srcT, dst, dstT, outer, inner, m, dm); break;
    case 8: absorb_dual_fixed<T, 8>(src, srcT, dst, dstT, outer, inner, m, dm); break;
    default: absorb_dual_rt<T>(src, srcT, dst, dstT, outer, D, inner, m, dm); break;
  }
}

__device__ void adj_step_dev(AdjState* s);

// Grid-wide barrier k of the persistent adjoint loop (see grid_barrier).
__device__ bool adj_grid_barrier(AdjGrid* gr, unsigned k, unsigned long long wait_ns) {
  return grid_barrier(&gr->arrivals, k, &gr->err, wait_ns);
}

// MINB = 2: at most 128 registers, so that two CTAs of 256 threads share an SM (the
// autotuner's 256-thread candidate); MINB = 1 for CTAs of up to 128 threads.
template <typename T, int MINB>
__global__ void __launch_bounds__(256, MINB) bp2_dual_kernel(GenericArgs a, DualArgs d) {
  extern __shared__ __align__(16) unsigned char smem[];
  // the dual launch sizes nbuf for both planes: nbuf = 2 * logical buffers
  const SmemLayout L = smem_layout<T>(a, blockDim.x, a.gscratch == nullptr);
  const int nb = a.nbuf / 2;
  T* bufs = a.gscratch ? reinterpret_cast<T*>(a.gscratch) + (size_t)blockIdx.x * a.nbuf * a.buf_elems
                       : reinterpret_cast<T*>(smem + L.bufs);
  T* msgs = reinterpret_cast<T*>(smem + L.msgs);  // [value | tangent] staging
  T* out = reinterpret_cast<T*>(smem + L.out);
  T* red = reinterpret_cast<T*>(smem + L.red);
  LegMeta* meta = reinterpret_cast<LegMeta*>(smem + L.meta);
  const T* tens = reinterpret_cast<const T*>(a.tens);
  const T* min_ = reinterpret_cast<const T*>(a.msg_in);
  // persistent adjoint loop: the first iteration's tangents are mu_buf[0]
  const bool persist = d.grid != nullptr;
  const T* tin = reinterpret_cast<const T*>(persist ? d.mu_buf[0] : d.tan_in);
  const int half = a.msg_cap / 2;
  if (d.done && *reinterpret_cast<const volatile int*>(d.done)) return;
  if (threadIdx.x == 0) {
    ptx::mbar_init(&meta->bar, 1);
    ptx::fence_mbar_init();
    meta->phase = 0;
  }
  __syncthreads();
  double adj_dmax = 0, adj_lmax = 0;  // fused adjoint update: this thread's maxima

  for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
    const int u = a.items[2 * it];
    const unsigned* prog = a.prog + a.items[2 * it + 1];
    T* A = bufs;
    item_meta<T, true>(a, u, meta, A, a.gscratch == nullptr);
    const int n = meta->n;
    const T* A_g = tens + a.toff[u];
    const bool bulk = meta->bulk != 0;
    if (!bulk)
      for (int j = threadIdx.x; j < n; j += blockDim.x) A[j] = A_g[j];
    const int s0 = meta->s0;
    for (int j = threadIdx.x; j < meta->mtot; j += blockDim.x) {
      const int l = staged_leg(meta, j);
      const int Dl = meta->dims[l], jl = j - meta->moffs[l];
      const int jj = d.transpose ? (jl % Dl) * Dl + jl / Dl : jl;
      msgs[j] = min_[meta->msrc[l] + jj];
      msgs[half + j] = tin ? tin[meta->tsrc[l] + jj] : T(0);
    }
    if (bulk) {
      // bounded wait; on timeout the copy is re-done with plain loads
      if (!__syncthreads_and(ptx::mbar_wait_bounded(&meta->bar, meta->phase, 1u << 26))) {
        for (int j = threadIdx.x; j < n; j += blockDim.x) A[j] = A_g[j];
      }
      if (threadIdx.x == 0) meta->phase ^= 1;
    }
    __syncthreads();
    for (int iter = 0;; ++iter) {
    T* const mu_next = reinterpret_cast<T*>(persist ? d.mu_buf[(iter + 1) & 1] : d.mu_next);
    const int nops = (int)prog[0];
    for (int q = 1; q <= nops; ++q) {
      const unsigned op = prog[q];
      const int type = op >> 28, srcb = (op >> 20) & 0xff, dstb = (op >> 12) & 0xff,
                leg = op & 0xfff;
      const T* src = bufs + (size_t)srcb * a.buf_elems;
      const T* srcT = srcb == 0 ? nullptr : bufs + (size_t)(srcb + nb) * a.buf_elems;
      if (type == OP_ABSORB) {
        T* dst = bufs + (size_t)dstb * a.buf_elems;
        T* dstT = bufs + (size_t)(dstb + nb) * a.buf_elems;
        dispatch_absorb_dual<T>(src, srcT, dst, dstT, meta->outer[leg], meta->dims[leg], meta->inner[leg],
                                msgs + meta->moffs[leg], msgs + half + meta->moffs[leg]);
        __syncthreads();
      } else if (type == OP_FINAL) {
        const int D = meta->dims[leg];
        if (srcT) {
          dispatch_final<T>(srcT, A, meta->outer[leg], D, meta->inner[leg], out, red);
        } else {
          for (int e = threadIdx.x; e < D * D; e += blockDim.x) out[e] = T(0);
          __syncthreads();
        }
        const int slot = a.rev[s0 + leg];
        if (d.adj) {
          // the adjoint update of this slot: lambda <- g + (J^T mu), mu' = (lambda - <lambda, F>) / S
          const long long o0 = a.moff[slot];
          const T* g = reinterpret_cast<const T*>(d.g) + o0;
          const T* F = reinterpret_cast<const T*>(d.F) + o0;
          T* lam = reinterpret_cast<T*>(d.lam) + o0;
          T dot = 0;
          for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
            const T v = g[e] + (d.transpose ? out[(e % D) * D + e / D] : out[e]);
            adj_dmax = fmax(adj_dmax, fabs((double)(v - lam[e])));
            adj_lmax = fmax(adj_lmax, fabs((double)v));
            lam[e] = v;
            if (d.normalize) dot += v * F[e];
          }
          dot = block_sum(dot, red);
          const T is = T(1) / reinterpret_cast<const T*>(d.S)[slot];
          T* mu = mu_next + o0;
          for (int e = threadIdx.x; e < D * D; e += blockDim.x) mu[e] = (lam[e] - dot) * is;
        } else {
          T* dst = reinterpret_cast<T*>(d.tan_out) + a.moff[slot];
          for (int e = threadIdx.x; e < D * D; e += blockDim.x)
            dst[e] = d.transpose ? out[(e % D) * D + e / D] : out[e];
        }
        __syncthreads();
      } else if (type == OP_DUMP) {
        T* g = reinterpret_cast<T*>(d.grad_out) + a.toff[u];
        if (d.dump_tangent == 2) {
          // both planes: value / Z_u + tangent
          const T scale = T(1) / reinterpret_cast<const T*>(d.zv)[u];
          for (int j = threadIdx.x; j < n; j += blockDim.x) g[j] += src[j] * scale + (srcT ? srcT[j] : T(0));
        } else {
          const T* plane = d.dump_tangent ? srcT : src;
          const T scale = d.dump_tangent ? T(1) : T(1) / reinterpret_cast<const T*>(d.zv)[u];
          if (plane)
            for (int j = threadIdx.x; j < n; j += blockDim.x) g[j] += plane[j] * scale;
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (!persist) break;
    // end of a persistent iteration: fold this iteration's maxima into slot iter % 3, wait for
    // every CTA, then every CTA applies the same stopping rule to the same maxima
    const int k3 = iter % 3;
    for (int o = 16; o >= 1; o >>= 1) {
      adj_dmax = fmax(adj_dmax, __shfl_xor_sync(0xffffffffu, adj_dmax, o));
      adj_lmax = fmax(adj_lmax, __shfl_xor_sync(0xffffffffu, adj_lmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&d.grid->dmax[k3], enc_double(adj_dmax));
      atomicMax(&d.grid->lmax[k3], enc_double(adj_lmax));
    }
    adj_dmax = adj_lmax = 0;
    __threadfence();
    // (fault injection: CTA 0 leaves without arriving, so the others' waits run out)
    if (d.stall && iter == 0 && blockIdx.x == 0) break;
    if (!adj_grid_barrier(d.grid, iter + 1, d.wait_ns)) break;
    {
      // the next iteration's tangents (the site tensor and the value messages stay staged),
      // loaded before the maxima are read so that the two reads overlap; unused if the loop
      // stops here
      const T* tk = reinterpret_cast<const T*>(d.mu_buf[(iter + 1) & 1]);
      for (int j = threadIdx.x; j < meta->mtot; j += blockDim.x) {
        const int l = staged_leg(meta, j);
        const int Dl = meta->dims[l], jl = j - meta->moffs[l];
        const int jj = d.transpose ? (jl % Dl) * Dl + jl / Dl : jl;
        msgs[half + j] = tk[meta->tsrc[l] + jj];
      }
    }
    const double dm = dec_double(*reinterpret_cast<volatile unsigned long long*>(&d.grid->dmax[k3])),
                 lm = dec_double(*reinterpret_cast<volatile unsigned long long*>(&d.grid->lmax[k3]));
    const double r = lm > 0 ? dm / lm : 0.0;
    const int its = iter + 1;
    const bool nan_r = r != r;
    const bool stop = nan_r || r < d.adj->tol || its >= d.adj->maxiter;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      d.adj->iters = its;
      d.adj->resid = r;
      if (nan_r) d.adj->nan = 1;
      if (stop) d.adj->done = 1;
      d.grid->dmax[(iter + 2) % 3] = d.grid->lmax[(iter + 2) % 3] = enc_double(0.0);
      __threadfence();
    }
    __syncthreads();  // the restaged tangents
    if (stop) break;
    }  // persistent iterations
  }
  if (d.adj && !persist) {
    // fold max |lambda_new - lambda| and max |lambda_new| into the state (order-encoded); the
    // last CTA to finish runs the stopping rule (a stopped loop returns at once in every CTA,
    // so the ticket stays at zero)
    for (int o = 16; o >= 1; o >>= 1) {
      adj_dmax = fmax(adj_dmax, __shfl_xor_sync(0xffffffffu, adj_dmax, o));
      adj_lmax = fmax(adj_lmax, __shfl_xor_sync(0xffffffffu, adj_lmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&d.adj->dmax, enc_double(adj_dmax));
      atomicMax(&d.adj->lmax, enc_double(adj_lmax));
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0 && atomicAdd(&d.adj->ticket, 1u) == gridDim.x - 1) {
      __threadfence();
      adj_step_dev(d.adj);
      d.adj->ticket = 0;
      __threadfence();
    }
  }
}

// per slot s: S_s = sum(U_s); F_s = U_s / S_s (U_s when S_s == 0 or not normalising)
template <typename T>
__global__ void grad_prep_kernel(const long long* moff, int nslots, const T* U, T* F, T* S, int normalize) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nslots) return;
  T sum = 0;
  for (long long j = moff[warp] + lane; j < moff[warp + 1]; j += 32) sum += U[j];
  sum = warp_sum(sum);
  const bool sc = normalize && sum != T(0);
  for (long long j = moff[warp] + lane; j < moff[warp + 1]; j += 32) F[j] = sc ? U[j] / sum : U[j];
  if (lane == 0) S[warp] = sc ? sum : T(1);
}

// g_t = U_{rev t} / Z_{nbr t} - m_{rev t} / Z_{e(t)}   (dL/dm for the message on slot t)
template <typename T>
__global__ void grad_g_kernel(const long long* moff, const int* rev, const int* dst_vertex, const int* eidx,
                              int nslots, const T* U, const T* m, const T* zv, const T* ze, T* g) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nslots) return;
  const int r = rev[warp];
  const T iz = T(1) / zv[dst_vertex[warp]], ie = T(1) / ze[eidx[warp]];
  const long long n = moff[warp + 1] - moff[warp];
  for (long long j = lane; j < n; j += 32) g[moff[warp] + j] = U[moff[r] + j] * iz - m[moff[r] + j] * ie;
}

// mu_s = (lambda_s - <lambda_s, F_s>) / S_s  (normalised updates) or lambda_s
template <typename T>
__global__ void grad_mu_kernel(const long long* moff, int nslots, const T* lam, const T* F, const T* S, T* mu,
                               int normalize, const int* done) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nslots) return;
  if (done && *reinterpret_cast<const volatile int*>(done)) return;
  T dot = 0;
  if (normalize)
    for (long long j = moff[warp] + lane; j < moff[warp + 1]; j += 32) dot += lam[j] * F[j];
  dot = warp_sum(dot);
  const T is = T(1) / S[warp];
  for (long long j = moff[warp] + lane; j < moff[warp + 1]; j += 32) mu[j] = (lam[j] - dot) * is;
}

__global__ void adj_reset_kernel(AdjState* s, double tol, int maxiter) {
  s->dmax = s->lmax = enc_double(0.0);
  s->done = maxiter <= 0;
  s->iters = 0;
  s->nan = 0;
  s->maxiter = maxiter;
  s->tol = tol;
  s->resid = 0.0;
  s->ticket = 0;
}

// One step of the adjoint loop's stopping rule (single thread, after the update).
__device__ void adj_step_dev(AdjState* s) {
  if (s->done) return;
  const int it = ++s->iters;
  const double dmax = dec_double(*reinterpret_cast<volatile unsigned long long*>(&s->dmax)),
               lmax = dec_double(*reinterpret_cast<volatile unsigned long long*>(&s->lmax));
  const double r = lmax > 0 ? dmax / lmax : 0.0;
  s->resid = r;
  if (r != r) {
    s->nan = 1;
    s->done = 1;
  } else if (r < s->tol || it >= s->maxiter) {
    s->done = 1;
  }
  s->dmax = s->lmax = enc_double(0.0);
}

__global__ void adj_step_kernel(AdjState* s) { adj_step_dev(s); }

// ---- the one-layer kernel ----------------------------------------------------------------
// items: (vertex, leg mask); mask bit v set -> compute m_{u->v}; mask == 0 -> vertex scalar.
template <typename T>
__global__ void __launch_bounds__(256) bp1_kernel(GenericArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SmemLayout L = smem_layout<T>(a, blockDim.x, false);
  T* msgs = reinterpret_cast<T*>(smem + L.msgs);
  T* out = reinterpret_cast<T*>(smem + L.out);
  T* red = reinterpret_cast<T*>(smem + L.red);
  LegMeta* meta = reinterpret_cast<LegMeta*>(smem + L.meta);
  const T* tens = reinterpret_cast<const T*>(a.tens);
  const T* min_ = reinterpret_cast<const T*>(a.msg_in);
  if (a.conv && *reinterpret_cast<const volatile int*>(&a.conv->done)) return;

  for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
    const int u = a.items[2 * it];
    const unsigned mask = (unsigned)a.items[2 * it + 1];
    if (threadIdx.x == 0) {
      const int s0 = a.off[u];
      const int z = a.off[u + 1] - s0;
      meta->z = z;
      meta->d = a.phys[u];
      int n = meta->d, mo = 0;
      for (int l = 0; l < z; ++l) {
        meta->dims[l] = a.bond[s0 + l];
        n *= meta->dims[l];
        meta->moffs[l] = mo;
        mo += meta->dims[l];
      }
      meta->n = n;
      int inner = 1;
      for (int l = z - 1; l >= 0; --l) {
        meta->inner[l] = inner;
        inner *= meta->dims[l];
      }
    }
    __syncthreads();
    const int z = meta->z, n = meta->n;
    const int s0 = a.off[u];
    for (int l = 0; l < z; ++l) {
      const T* src = min_ + a.moff[a.rev[s0 + l]];
      for (int j = threadIdx.x; j < meta->dims[l]; j += blockDim.x) msgs[meta->moffs[l] + j] = src[j];
    }
    __syncthreads();
    const T* A = tens + a.toff[u];
    if (mask == 0) {
      T acc = tzero<T>();
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        T p = A[j];
        for (int l = 0; l < z; ++l) {
          const int kl = (j / meta->inner[l]) % meta->dims[l];
          p = mul(p, msgs[meta->moffs[l] + kl]);
        }
        acc = add(acc, p);
      }
      acc = block_sum(acc, red);
      if (threadIdx.x == 0) reinterpret_cast<T*>(a.zv_out)[u] = acc;
      __syncthreads();
      continue;
    }
    for (int v = 0; v < z; ++v) {
      if (!((mask >> v) & 1u)) continue;
      const int Dv = meta->dims[v];
      const int innv = meta->inner[v];
      const int nrest = n / Dv;
      for (int k = 0; k < Dv; ++k) {
        T acc = tzero<T>();
        for (int r = threadIdx.x; r < nrest; r += blockDim.x) {
          const int o = r / innv, i = r - o * innv;
          const int j = (o * Dv + k) * innv + i;
          T p = A[j];
          for (int l = 0; l < z; ++l) {
            if (l == v) continue;
            const int kl = (j / meta->inner[l]) % meta->dims[l];
            p = mul(p, msgs[meta->moffs[l] + kl]);
          }
          acc = add(acc, p);
        }
        acc = block_sum(acc, red);
        if (threadIdx.x == 0) out[k] = acc;
      }
      __syncthreads();
      store_message<T>(a, out, Dv, s0 + v, a.msg_in, a.msg_out, a.conv ? &a.conv->dmax : nullptr,
                       a.conv ? &a.conv->nan_flag : nullptr);
      __syncthreads();
    }
  }
  if (a.conv && a.fused_step) conv_finish_cta(a.conv);
}

// ---- vertex scalars of norm-network vertices with d = 2 and four legs of dimension 8 -------
// Z_u = sum_s <A_s| m0 (x) m1 (x) m2 (x) m3 |A_s> (vertex_scalar, messagecache.jl:139-150),
// with A_s viewed as a 64 x 64 matrix over p = (k0, k1), q = (k2, k3), as two passes of
// 8 x 8 matrix products; one CTA of 128 threads per vertex:
//   pass 1, thread (s, p):  W_s[p][(b2 b3)] = sum_{k2,k3} m2[b2,k2] A_s[p][(k2 k3)] m3[b3,k3]
//   pass 2, thread (s, c):  V_s[(b0 b1)][c] = sum_{k0,k1} m0[b0,k0] W_s[(k0 k1)][c] m1[b1,k1]
//   Z_u = sum_{s,b,c} conj(A_s[b][c]) V_s[b][c]
// (m_l[b][k]: bra index b, ket index k, the message into u on leg l).  The same 262,144
// multiply-adds per vertex as the interpreter's leg-by-leg absorption, with every 8 x 8
// product in registers.  Shared memory holds W and, for float, the site tensor (staged by
// coalesced 16-byte loads, all in flight at once); both with row stride 65, so that the row
// accesses of pass 1 and the column accesses of pass 2 are free of bank conflicts.
constexpr int kVsLd = 65;

template <typename T>
__host__ __device__ constexpr bool vs_stage() { return sizeof(T) == 4; }

template <typename T>
size_t vertex_scalar_d8_smem() {
  return (size_t)((vs_stage<T>() ? 2 : 1) * 128 * kVsLd + 256 + 4) * sizeof(T);
}

template <typename T>
__global__ void __launch_bounds__(128, vs_stage<T>() ? 3 : 1) vertex_scalar_d8_kernel(const int* __restrict__ rev,
                                                               const long long* __restrict__ moff,
                                                               const long long* __restrict__ toff,
                                                               const T* __restrict__ tens,
                                                               const T* __restrict__ msgs, T* __restrict__ zv) {
  constexpr bool STAGE = vs_stage<T>();
  extern __shared__ __align__(16) unsigned char vs_smem[];
  T* w = reinterpret_cast<T*>(vs_smem);           // [2 x 64][kVsLd]
  T* as = w + 128 * kVsLd;                        // STAGE: A_s[p][q] at (64 s + p) kVsLd + q
  T* m = as + (STAGE ? 128 * kVsLd : 0);          // [4][64]
  T* red = m + 256;                               // [4]
  const int u = blockIdx.x, t = threadIdx.x;
  const int s = t >> 6, r = t & 63;
  const T* Ag = tens + toff[u];
  if constexpr (STAGE) {
    // 8192 entries as 2048 16-byte loads (the tensor starts on a 32 KB boundary)
    const float4* src = reinterpret_cast<const float4*>(Ag);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float4 v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = __ldg(src + t + 128 * (8 * h + i));
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int j = t + 128 * (8 * h + i);
        float* d = reinterpret_cast<float*>(as) + (j >> 4) * kVsLd + (j & 15) * 4;
        d[0] = v[i].x;
        d[1] = v[i].y;
        d[2] = v[i].z;
        d[3] = v[i].w;
      }
    }
  }
  for (int j = t; j < 256; j += 128) m[j] = msgs[moff[rev[4 * u + (j >> 6)]] + (j & 63)];
  __syncthreads();
  {
    T W[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) W[i] = tzero<T>();
    const T* row = STAGE ? as + (s * 64 + r) * kVsLd : Ag + (size_t)s * 4096 + r * 64;
#pragma unroll
    for (int k2 = 0; k2 < 8; ++k2) {
      T x[8], y[8];
#pragma unroll
      for (int k3 = 0; k3 < 8; ++k3) x[k3] = row[k2 * 8 + k3];
#pragma unroll
      for (int b3 = 0; b3 < 8; ++b3) {
        T acc = tzero<T>();
#pragma unroll
        for (int k3 = 0; k3 < 8; ++k3) acc = fmac(x[k3], m[192 + b3 * 8 + k3], acc);
        y[b3] = acc;
      }
#pragma unroll
      for (int b2 = 0; b2 < 8; ++b2) {
        const T c2 = m[128 + b2 * 8 + k2];
#pragma unroll
        for (int b3 = 0; b3 < 8; ++b3) W[b2 * 8 + b3] = fmac(y[b3], c2, W[b2 * 8 + b3]);
      }
    }
    T* wr = w + (s * 64 + r) * kVsLd;
#pragma unroll
    for (int c = 0; c < 64; ++c) wr[c] = W[c];
  }
  __syncthreads();
  T part = tzero<T>();
  {
    T V[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) V[i] = tzero<T>();
    const T* col = w + s * 64 * kVsLd + r;  // W_s[p][c = r] at col[p * kVsLd]
#pragma unroll
    for (int k0 = 0; k0 < 8; ++k0) {
      T x[8], y[8];
#pragma unroll
      for (int k1 = 0; k1 < 8; ++k1) x[k1] = col[(k0 * 8 + k1) * kVsLd];
#pragma unroll
      for (int b1 = 0; b1 < 8; ++b1) {
        T acc = tzero<T>();
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) acc = fmac(x[k1], m[64 + b1 * 8 + k1], acc);
        y[b1] = acc;
      }
#pragma unroll
      for (int b0 = 0; b0 < 8; ++b0) {
        const T c0 = m[b0 * 8 + k0];
#pragma unroll
        for (int b1 = 0; b1 < 8; ++b1) V[b0 * 8 + b1] = fmac(y[b1], c0, V[b0 * 8 + b1]);
      }
    }
    const T* acol = STAGE ? as + s * 64 * kVsLd + r : Ag + (size_t)s * 4096 + r;
#pragma unroll
    for (int b = 0; b < 64; ++b) part = fmac(V[b], conjx(acol[b * (STAGE ? kVsLd : 64)]), part);
  }
  part = warp_sum(part);
  if ((t & 31) == 0) red[t >> 5] = part;
  __syncthreads();
  if (t == 0) zv[u] = add(add(red[0], red[1]), add(red[2], red[3]));
}

// ---- edge scalars: Z_e = sum_j m_{u->v}[j] * m_{v->u}[j]  (messagecache.jl:153-157) -----
template <typename T>
__global__ void edge_scalar_kernel(const long long* moff, const int* rev, const int* eslots,
                                   int n_e, const T* msgs, T* ze) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n_e) return;
  const int s = eslots[warp];
  const T* x = msgs + moff[s];
  const T* y = msgs + moff[rev[s]];
  const int n = (int)(moff[s + 1] - moff[s]);
  T acc = tzero<T>();
  for (int j = lane; j < n; j += 32) acc = fmac(x[j], y[j], acc);
  acc = warp_sum(acc);
  if (lane == 0) ze[warp] = acc;
}

// log of a scalar as (re, im) in double; real values promote like complex.(x) does in
// bethe_free_energy (messagecache.jl:189-194).
template <typename T>
__device__ __forceinline__ void log2d(T z, double& re, double& im) {
  const double a = re_d(z), b = im_d(z);
  if constexpr (is_cplx<T>::value) {
    re = 0.5 * log(a * a + b * b);
    im = atan2(b, a);
  } else {
    if (a < 0) { re = log(-a); im = M_PI; }
    else { re = log(a); im = 0.0; }
  }
}

// FP64 logs of every vertex and edge scalar, one thread each (the double-precision log is
// slow on this part, so the logs are spread over the whole grid rather than summed by one
// block per network).  With `part` non-null (a single network), each block also leaves its
// share of sum log Z_v - sum log Z_e as (re, im) in part[2 b], and its flag bits in
// pflags[b], for logsum_single_kernel.
template <typename T>
__global__ void __launch_bounds__(128) log_scalars_kernel(const T* zv, const T* ze, int nv, int ne, double* logzv,
                                                          double* logze, double* part, int* pflags) {
  __shared__ double sre[4], sim[4];
  __shared__ int sfl[4];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double re = 0, im = 0;
  int fl = 0;
  if (j < nv) {
    log2d(zv[j], re, im);
    logzv[2 * j] = re;
    logzv[2 * j + 1] = im;
    if (re_d(zv[j]) < 0) fl |= 1;
  } else if (j < nv + ne) {
    const int e = j - nv;
    log2d(ze[e], re, im);
    logze[2 * e] = re;
    logze[2 * e + 1] = im;
    if (re_d(ze[e]) < 0) fl |= 2;
    if (is_zero(ze[e])) fl |= 4;
    re = -re;
    im = -im;
  }
  if (!part) return;
  re = warp_sum_d(re);
  im = warp_sum_d(im);
  for (int o = 16; o >= 1; o >>= 1) fl |= __shfl_xor_sync(0xffffffffu, fl, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sre[warp] = re; sim[warp] = im; sfl[warp] = fl; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0, i = 0;
    int f = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { r += sre[w]; i += sim[w]; f |= sfl[w]; }
    part[2 * blockIdx.x] = r;
    part[2 * blockIdx.x + 1] = i;
    pflags[blockIdx.x] = f;
  }
}

// The single-network total: the blocks' shares summed in block order.
__global__ void __launch_bounds__(256) logsum_single_kernel(const double* part, const int* pflags, int nblocks,
                                                            double* totals, int* flags) {
  __shared__ double sre[8], sim[8];
  __shared__ int sfl[8];
  double re = 0, im = 0;
  int fl = 0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    re += part[2 * b];
    im += part[2 * b + 1];
    fl |= pflags[b];
  }
  re = warp_sum_d(re);
  im = warp_sum_d(im);
  for (int o = 16; o >= 1; o >>= 1) fl |= __shfl_xor_sync(0xffffffffu, fl, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sre[warp] = re; sim[warp] = im; sfl[warp] = fl; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0, i = 0;
    int f = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { r += sre[w]; i += sim[w]; f |= sfl[w]; }
    totals[0] = r;
    totals[1] = i;
    flags[0] = f;
  }
}

// One block per network: the Bethe sum log Z = sum_v log Z_v - sum_e log Z_e
// (messagecache.jl:185-201) over the logs above, in a fixed order.
// flags per net: bit0 any Re Z_v < 0, bit1 any Re Z_e < 0, bit2 any Z_e == 0.
template <typename T>
__global__ void logsum_kernel(const T* zv, const T* ze, const int* voff, const int* vlist,
                              const int* eoff, const int* elist, const double* logzv,
                              const double* logze, double* totals, int* flags) {
  __shared__ double sre[32], sim[32];
  __shared__ int sfl[32];
  const int net = blockIdx.x;
  double are = 0, aim = 0;
  int fl = 0;
  for (int j = voff[net] + threadIdx.x; j < voff[net + 1]; j += blockDim.x) {
    const int v = vlist[j];
    if (re_d(zv[v]) < 0) fl |= 1;
    are += logzv[2 * v];
    aim += logzv[2 * v + 1];
  }
  for (int j = eoff[net] + threadIdx.x; j < eoff[net + 1]; j += blockDim.x) {
    const int e = elist[j];
    if (re_d(ze[e]) < 0) fl |= 2;
    if (is_zero(ze[e])) fl |= 4;
    are -= logze[2 * e];
    aim -= logze[2 * e + 1];
  }
  are = warp_sum_d(are);
  aim = warp_sum_d(aim);
  for (int o = 16; o >= 1; o >>= 1) fl |= __shfl_xor_sync(0xffffffffu, fl, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sre[warp] = are; sim[warp] = aim; sfl[warp] = fl; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0, i = 0;
    int f = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { r += sre[w]; i += sim[w]; f |= sfl[w]; }
    totals[2 * net] = r;
    totals[2 * net + 1] = i;
    flags[net] = f;
  }
}

// kind 0: identity / D (message_environment(one) then normalised), 1: identity,
// 2: all ones.  One-layer messages: kind 0 -> ones / D, else ones.
template <typename T>
__global__ void init_messages_kernel(int layers, int kind, const long long* moff, const int* bond,
                                     int nslots, T* msgs) {
  const int s = blockIdx.x;
  if (s >= nslots) return;
  const int D = bond[s];
  T* m = msgs + moff[s];
  const int n = layers == 2 ? D * D : D;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double val;
    if (layers == 2) {
      const bool diag = (j / D) == (j % D);
      val = kind == 2 ? 1.0 : (diag ? (kind == 0 ? 1.0 / D : 1.0) : 0.0);
    } else {
      val = kind == 0 ? 1.0 / D : 1.0;
    }
    T t = tzero<T>();
    if constexpr (is_cplx<T>::value) t.x = (typename real_of<T>::type)val;
    else t = (T)val;
    m[j] = t;
  }
}

template <typename T>
__global__ void iterate_diff_kernel(const long long* moff, int nslots, const T* m1, const T* m2,
                                    double* slot_diff, ConvState* conv) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nslots) return;
  double n1 = 0, n2 = 0, dre = 0, dim = 0;
  for (long long j = moff[warp] + lane; j < moff[warp + 1]; j += 32) {
    const double ar = re_d(m1[j]), ai = im_d(m1[j]), br = re_d(m2[j]), bi = im_d(m2[j]);
    n1 += ar * ar + ai * ai;
    n2 += br * br + bi * bi;
    dre += ar * br + ai * bi;
    dim += ar * bi - ai * br;
  }
  n1 = warp_sum_d(n1);
  n2 = warp_sum_d(n2);
  dre = warp_sum_d(dre);
  dim = warp_sum_d(dim);
  if (lane == 0) {
    const double val = 1.0 - (dre * dre + dim * dim) / (n1 * n2);
    if (slot_diff) slot_diff[warp] = val;
    if (val != val) atomicExch(&conv->nan_flag, 1);
    else atomicMax(&conv->dmax, enc_double(val));
  }
}

// Site-tensor permutation into the canonical row-major [phys][legs...] layout.
// For vertex u, canonical axis a has extent dims[rank_off[u]+a] and source stride
// sstride[rank_off[u]+a] (elements); source tensor starts at soff[u].
template <typename T>
__global__ void permute_kernel(int nv, const long long* soff, const long long* toff,
                               const int* rank_off, const int* dims, const long long* sstride,
                               const T* src, T* dst) {
  const int u = blockIdx.y;
  if (u >= nv) return;
  const long long n = toff[u + 1] - toff[u];
  const int r0 = rank_off[u], r = rank_off[u + 1] - r0;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    long long rem = j, so = 0;
    for (int ax = r - 1; ax >= 0; --ax) {
      const int e = dims[r0 + ax];
      const long long idx = rem % e;
      rem /= e;
      so += idx * sstride[r0 + ax];
    }
    dst[toff[u] + j] = src[soff[u] + so];
  }
}

__global__ void reset_state_kernel(ConvState* s, double tol, int use_tol) {
  s->dmax = enc_double(-INFINITY);
  s->nan_flag = 0;
  s->done = 0;
  s->at_iter = -1;
  s->iters = 0;
  s->delta = INFINITY;
  s->counter = 0;
  s->tickets = 0;
  s->tol = tol;
  s->use_tol = use_tol;
}

__global__ void step_check_kernel(ConvState* s) { conv_step(s); }

// The two-layer interpreter for a CTA size.  complex64 always caps registers at 128, so that
// small CTAs co-reside (its D = 8 paths spill a little); float takes the capped variant (no
// spills) for CTAs of 128 threads or more (four resident CTAs of 128 threads per SM instead of
// three, so that every item of a 16x16 lattice has its own CTA and the sweeps can run as one
// persistent launch) and its full register budget at 64 threads; double and complex128 keep
// their full budget (capped at 128 they spill).
template <typename T>
void (*bp2_kernel_for(int block))(GenericArgs) {
  if constexpr (std::is_same<T, c64>::value) {
    return bp2_kernel<T, 2>;
  } else if constexpr (std::is_same<T, float>::value) {
    return block >= 128 ? bp2_kernel<T, 2> : bp2_kernel<T, 1>;
  } else {
    return bp2_kernel<T, 1>;
  }
}

template <typename T>
cudaError_t launch_generic_t(const GenericArgs& a, const LaunchCfg& cfg, cudaStream_t st) {
  if (cfg.grid <= 0 || a.n_items <= 0) return cudaSuccess;
  if (a.layers == 2) {
    auto k = bp2_kernel_for<T>(cfg.block);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess) return e;
    k<<<cfg.grid, cfg.block, cfg.smem, st>>>(a);
  } else {
    auto k = bp1_kernel<T>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess) return e;
    k<<<cfg.grid, cfg.block, cfg.smem, st>>>(a);
  }
  return cudaGetLastError();
}

template <typename T>
int max_active_t(int layers, int block, size_t smem) {
  int n = 0;
  if (layers == 2) {
    // complex64 (small CTAs, capped registers): all of the unified L1 / shared memory as
    // shared memory, so that more CTAs co-reside; the real types keep the default split
    auto k = bp2_kernel_for<T>(block);
    if (is_cplx<T>::value && sizeof(T) == 8)
      cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem);
  } else {
    cudaFuncSetAttribute(bp1_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, bp1_kernel<T>, block, smem);
  }
  return n;
}

}  // namespace

#define ITN_DISPATCH(dtype, ...)                         \
  switch (dtype) {                                       \
    case DT_F32: { using T = float; __VA_ARGS__; }       \
    case DT_F64: { using T = double; __VA_ARGS__; }      \
    case DT_C64: { using T = c64; __VA_ARGS__; }         \
    case DT_C128: { using T = c128; __VA_ARGS__; }       \
    default: return cudaErrorInvalidValue;               \
  }

size_t generic_smem_bytes(int dtype, const GenericArgs& a, int block, bool in_smem) {
  switch (dtype) {
    case DT_F32: return smem_layout<float>(a, block, in_smem).total;
    case DT_F64: return smem_layout<double>(a, block, in_smem).total;
    case DT_C64: return smem_layout<c64>(a, block, in_smem).total;
    case DT_C128: return smem_layout<c128>(a, block, in_smem).total;
  }
  return 0;
}

int generic_max_active(int dtype, int layers, int block, size_t smem) {
  switch (dtype) {
    case DT_F32: return max_active_t<float>(layers, block, smem);
    case DT_F64: return max_active_t<double>(layers, block, smem);
    case DT_C64: return max_active_t<c64>(layers, block, smem);
    case DT_C128: return max_active_t<c128>(layers, block, smem);
  }
  return 0;
}

cudaError_t launch_generic(int dtype, const GenericArgs& a, const LaunchCfg& cfg, cudaStream_t st) {
  ITN_DISPATCH(dtype, return launch_generic_t<T>(a, cfg, st));
}

__global__ void sweep_grid_init_kernel(SweepGrid* g) {
  if (threadIdx.x == 0) {
    g->arrivals = 0;
    for (int k = 0; k < 3; ++k) {
      g->dmax[k] = enc_double(-INFINITY);
      g->nanf[k] = 0;
    }
    g->err = 0;
  }
}

template <typename T>
cudaError_t launch_generic_persistent_t(const GenericArgs& a, const LaunchCfg& cfg, cudaStream_t st) {
  if (a.layers != 2 || !a.pgrid || cfg.grid != a.n_items || a.n_items <= 0) return cudaErrorInvalidValue;
  sweep_grid_init_kernel<<<1, 32, 0, st>>>(a.pgrid);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  auto k = bp2_kernel_for<T>(cfg.block);
  e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.gridDim = dim3(cfg.grid);
  lc.blockDim = dim3(cfg.block);
  lc.dynamicSmemBytes = cfg.smem;
  lc.stream = st;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, k, a);
}

cudaError_t launch_generic_persistent(int dtype, const GenericArgs& a, const LaunchCfg& cfg, cudaStream_t st) {
  ITN_DISPATCH(dtype, return launch_generic_persistent_t<T>(a, cfg, st));
}

// ---- FP32 sweep of a d = 2 lattice with four legs of dimension 8 per vertex -----------------
// The plain FP32 message update (beliefpropagation.jl:242-257) on CUDA cores with the
// register blocking of vertex_scalar_d8_kernel.  One CTA of 128 threads per half-vertex item
// (vertex u, half h): the two "front" legs f0, f1 (0, 1 for h = 0; 2, 3 for h = 1) are
// absorbed first and the two "back" legs g0, g1 receive the outgoing messages.  With
// M_s[f][g] = A_s[p][q] (h = 0, f = p = (k0,k1), g = q = (k2,k3)) or A_s[q][p] (h = 1):
//   pass 1, thread (s, g):  T_s[bf][g] = sum_{f0,f1} m_f0[bf0][f0] m_f1[bf1][f1] M_s[(f0,f1)][g]
//           as X = m_f0 * M_s[:, g] (8x8x8) then T = X * m_f1^T (8x8x8);
//   pass 2, thread (s, bf): out_g0[bg0][kg0] += sum_bg1 M_s[bf][(bg0,bg1)] sum_kg1 T_s[bf][(kg0,kg1)] m_g1[bg1][kg1]
//                           out_g1[bg1][kg1] += sum_bg0 M_s[bf][(bg0,bg1)] sum_kg0 m_g0[bg0][kg0] T_s[bf][(kg0,kg1)]
//           each as two 8x8x8 products in registers, then summed over the 128 threads by a
//           butterfly reduce-scatter (64 values -> 2 per lane) and the 4 warps' shares.
// 786,432 multiply-adds per vertex (the leave-one-out minimum; the algorithmic count of the
// four updates is 1,048,576).  The site tensor is staged with rows of kD8Ld floats so that
// row (LDS.128) and column (LDS.32) reads are both free of bank conflicts.
constexpr int kD8Ld = 68;
constexpr size_t kD8SmemFloats = 2 * 128 * kD8Ld + 256 + 2 * 4 * 64 + 8;

// Sum of v[0..63] over the warp, scattered: lane l returns entries 2l and 2l + 1.
__device__ __forceinline__ float2 warp_reduce_scatter64(float (&v)[64]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16, n = 32; o >= 1; o >>= 1, n >>= 1) {
    const bool hi = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < n; ++i) {
      const float keep = hi ? v[i + n] : v[i];
      const float send = hi ? v[i] : v[i + n];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return make_float2(v[0], v[1]);
}

struct SweepD8Args {
  const int* rev;
  const float* tens;
  const float* msg_in;
  float* msg_out;
  int nv;
  int normalize;
  double* slot_diff;
  ConvState* conv;
};

// 8 consecutive floats of shared memory (16-byte aligned) / 8 floats `stride` apart
__device__ __forceinline__ void lds8(const float* p, float (&x)[8]) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  const float4 b = *reinterpret_cast<const float4*>(p + 4);
  x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
  x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
}
__device__ __forceinline__ void lds8s(const float* p, int stride, float (&x)[8]) {
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = p[i * stride];
}

// Row i (8 entries over the second index pair member) of the 8x8 block of M_s:
// M_s[(i, j)][c] for j = 0..7 (COLUMN: the thread's column c) or M_s[c][(i, j)] (ROW).
// H = 0: M_s = A_s (row stride kD8Ld); H = 1: M_s = A_s^T.
template <int H, bool COLUMN>
__device__ __forceinline__ void m_block_row(const float* Ms, int c, int i, float (&x)[8]) {
  // M_s[f][g] sits at f * mrow + g * mcol
  constexpr int mrow = H ? 1 : kD8Ld, mcol = H ? kD8Ld : 1;
  if constexpr (COLUMN) {
    // M_s[(i, j)][c]: j steps by mrow
    if constexpr (mrow == 1) lds8(Ms + i * 8 + c * mcol, x);
    else lds8s(Ms + i * 8 * mrow + c * mcol, mrow, x);
  } else {
    // M_s[c][(i, j)]: j steps by mcol
    if constexpr (mcol == 1) lds8(Ms + c * mrow + i * 8, x);
    else lds8s(Ms + c * mrow + i * 8 * mcol, mcol, x);
  }
}

template <int H>
__device__ __forceinline__ void sweep_d8_item(const SweepD8Args& a, int u, const float* As, float* Ts,
                                              const float* mt, float* red) {
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  constexpr int f0 = H ? 2 : 0, f1 = f0 + 1, g0 = H ? 0 : 2, g1 = g0 + 1;
  const int s = t >> 6, c = t & 63;
  const float* Ms = As + 64 * s * kD8Ld;
  // ---- pass 1: thread (s, g = c) ----
  {
    float X[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) X[i] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < 8; ++k0) {
      float col[8];
      m_block_row<H, true>(Ms, c, k0, col);
#pragma unroll
      for (int b0 = 0; b0 < 8; ++b0) {
        const float w = mt[64 * f0 + 8 * b0 + k0];
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) X[b0 * 8 + k1] = fmaf(w, col[k1], X[b0 * 8 + k1]);
      }
    }
    float* Tc = Ts + 64 * s * kD8Ld + c;
#pragma unroll
    for (int b1 = 0; b1 < 8; ++b1) {
      float mr[8];
      lds8(mt + 64 * f1 + 8 * b1, mr);
#pragma unroll
      for (int b0 = 0; b0 < 8; ++b0) {
        float acc = 0.f;
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) acc = fmaf(X[b0 * 8 + k1], mr[k1], acc);
        Tc[(b0 * 8 + b1) * kD8Ld] = acc;
      }
    }
  }
  __syncthreads();
  // ---- pass 2: thread (s, bf = c); the bra row is M_s[c][.] ----
  const float* Tr = Ts + (64 * s + c) * kD8Ld;
  {
    // out on leg g0: P[bg0][kg0] = sum_bg1 M[c][(bg0,bg1)] V[kg0][bg1],  V = T m_g1^T
    float V[64];
    {
      float T[64];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float x[8];
        lds8(Tr + 8 * i, x);
#pragma unroll
        for (int j = 0; j < 8; ++j) T[8 * i + j] = x[j];
      }
#pragma unroll
      for (int b1 = 0; b1 < 8; ++b1) {
        float mr[8];
        lds8(mt + 64 * g1 + 8 * b1, mr);
#pragma unroll
        for (int k0 = 0; k0 < 8; ++k0) {
          float acc = 0.f;
#pragma unroll
          for (int k1 = 0; k1 < 8; ++k1) acc = fmaf(T[k0 * 8 + k1], mr[k1], acc);
          V[k0 * 8 + b1] = acc;
        }
      }
    }
    float P[64];
#pragma unroll
    for (int b0 = 0; b0 < 8; ++b0) {
      float mb[8];
      m_block_row<H, false>(Ms, c, b0, mb);
#pragma unroll
      for (int k0 = 0; k0 < 8; ++k0) {
        float acc = 0.f;
#pragma unroll
        for (int b1 = 0; b1 < 8; ++b1) acc = fmaf(mb[b1], V[k0 * 8 + b1], acc);
        P[b0 * 8 + k0] = acc;
      }
    }
    const float2 r = warp_reduce_scatter64(P);
    *reinterpret_cast<float2*>(red + warp * 64 + 2 * lane) = r;
  }
  {
    // out on leg g1: P[bg1][kg1] = sum_bg0 M[c][(bg0,bg1)] U[bg0][kg1],  U = m_g0 T
    float T[64];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float x[8];
      lds8(Tr + 8 * i, x);
#pragma unroll
      for (int j = 0; j < 8; ++j) T[8 * i + j] = x[j];
    }
    float P[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) P[i] = 0.f;
#pragma unroll
    for (int b0 = 0; b0 < 8; ++b0) {
      float mr[8];
      lds8(mt + 64 * g0 + 8 * b0, mr);
      float U[8];
#pragma unroll
      for (int k1 = 0; k1 < 8; ++k1) {
        float acc = 0.f;
#pragma unroll
        for (int k0 = 0; k0 < 8; ++k0) acc = fmaf(mr[k0], T[k0 * 8 + k1], acc);
        U[k1] = acc;
      }
      float mb[8];
      m_block_row<H, false>(Ms, c, b0, mb);
#pragma unroll
      for (int b1 = 0; b1 < 8; ++b1)
#pragma unroll
        for (int k1 = 0; k1 < 8; ++k1) P[b1 * 8 + k1] = fmaf(mb[b1], U[k1], P[b1 * 8 + k1]);
    }
    const float2 r = warp_reduce_scatter64(P);
    *reinterpret_cast<float2*>(red + 256 + warp * 64 + 2 * lane) = r;
  }
}

__global__ void __launch_bounds__(128, 3) sweep_d8_kernel(SweepD8Args a) {
  extern __shared__ __align__(16) float sd8[];
  float* As = sd8;                   // A_s[p][q] at (64 s + p) * kD8Ld + q
  float* Ts = As + 128 * kD8Ld;      // T_s[bf][g] at (64 s + bf) * kD8Ld + g
  float* mt = Ts + 128 * kD8Ld;      // incoming messages m_l[b][k] at 64 l + 8 b + k
  float* red = mt + 256;             // [2 outputs][4 warps][64]
  float* sums = red + 2 * 4 * 64;    // [2 outputs][2 warps]
  if (a.conv && *reinterpret_cast<const volatile int*>(&a.conv->done)) return;
  const int u = blockIdx.x >> 1, h = blockIdx.x & 1;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  {
    // the site tensor (8192 floats, 32 KB aligned) into padded rows; the 4 incoming messages
    const float4* src = reinterpret_cast<const float4*>(a.tens + (size_t)u * 8192);
    float4 v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __ldg(src + t + 128 * i);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int j = t + 128 * i;
      *reinterpret_cast<float4*>(As + (j >> 4) * kD8Ld + (j & 15) * 4) = v[i];
    }
    mt[t] = __ldg(a.msg_in + 64 * a.rev[4 * u + (t >> 6)] + (t & 63));
    mt[t + 128] = __ldg(a.msg_in + 64 * a.rev[4 * u + 2 + (t >> 6)] + (t & 63));
  }
  __syncthreads();
  if (h) sweep_d8_item<1>(a, u, As, Ts, mt, red);
  else sweep_d8_item<0>(a, u, As, Ts, mt, red);
  __syncthreads();
  // ---- finish: threads 0..63 the message on leg g0, 64..127 the one on leg g1 ----
  const int g0 = h ? 0 : 2;
  const int o = t >> 6, e = t & 63;
  const float* ro = red + 256 * o;
  const float val = (ro[e] + ro[64 + e]) + (ro[128 + e] + ro[192 + e]);
  float sum = val;
#pragma unroll
  for (int k = 16; k >= 1; k >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, k);
  if (lane == 0) sums[2 * o + (warp & 1)] = sum;
  __syncthreads();
  sum = sums[2 * o] + sums[2 * o + 1];
  const bool scale = a.normalize && sum != 0.f;
  const float v = scale ? val / sum : val;
  const int slot = 4 * u + g0 + o;
  a.msg_out[64 * slot + e] = v;
  if (a.slot_diff) {
    const double ov = a.msg_in[64 * slot + e];
    double n1 = (double)v * v, n2 = ov * ov, dd = (double)v * ov;
#pragma unroll
    for (int k = 16; k >= 1; k >>= 1) {
      n1 += __shfl_xor_sync(0xffffffffu, n1, k);
      n2 += __shfl_xor_sync(0xffffffffu, n2, k);
      dd += __shfl_xor_sync(0xffffffffu, dd, k);
    }
    double* ds = reinterpret_cast<double*>(red);  // red is free once every thread has read it
    __syncthreads();
    if (lane == 0) {
      ds[3 * (2 * o + (warp & 1))] = n1;
      ds[3 * (2 * o + (warp & 1)) + 1] = n2;
      ds[3 * (2 * o + (warp & 1)) + 2] = dd;
    }
    __syncthreads();
    if (e == 0) {
      const double* p0 = ds + 6 * o;
      const double N1 = p0[0] + p0[3], N2 = p0[1] + p0[4], DD = p0[2] + p0[5];
      const double val2 = 1.0 - DD * DD / (N1 * N2);
      a.slot_diff[slot] = val2;
      if (a.conv) {
        if (val2 != val2) atomicExch(&a.conv->nan_flag, 1);
        else atomicMax(&a.conv->dmax, enc_double(val2));
        __threadfence();
      }
    }
  }
  if (a.conv) conv_finish_cta(a.conv);
}

template <typename T>
cudaError_t launch_vertex_scalars_d8_t(int nv, const int* rev, const long long* moff, const long long* toff,
                                       const void* tens, const void* msgs, void* zv, cudaStream_t st) {
  const size_t smem = vertex_scalar_d8_smem<T>();
  cudaError_t e = cudaFuncSetAttribute(vertex_scalar_d8_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  vertex_scalar_d8_kernel<T><<<nv, 128, smem, st>>>(rev, moff, toff, reinterpret_cast<const T*>(tens),
                                                    reinterpret_cast<const T*>(msgs), reinterpret_cast<T*>(zv));
  return cudaGetLastError();
}

cudaError_t launch_vertex_scalars_d8(int dtype, int nv, const int* rev, const long long* moff,
                                     const long long* toff, const void* tens, const void* msgs, void* zv,
                                     cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  switch (dtype) {
    case DT_F32: return launch_vertex_scalars_d8_t<float>(nv, rev, moff, toff, tens, msgs, zv, st);
    case DT_C64: return launch_vertex_scalars_d8_t<c64>(nv, rev, moff, toff, tens, msgs, zv, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sweep_d8(const int* rev, const float* tens, const float* msg_in, float* msg_out, int nv,
                            int normalize, double* slot_diff, ConvState* conv, cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  const size_t smem = kD8SmemFloats * sizeof(float);
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(sweep_d8_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(sweep_d8_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    configured = true;
  }
  SweepD8Args a{rev, tens, msg_in, msg_out, nv, normalize, slot_diff, conv};
  sweep_d8_kernel<<<2 * nv, 128, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_edge_scalars(int dtype, int layers, const long long* moff, const int* rev,
                                const int* eslots, int n_e, const void* msgs, void* ze_out,
                                cudaStream_t st) {
  (void)layers;
  if (n_e <= 0) return cudaSuccess;
  const int block = 256, grid = (n_e * 32 + block - 1) / block;
  ITN_DISPATCH(dtype, edge_scalar_kernel<T><<<grid, block, 0, st>>>(
                          moff, rev, eslots, n_e, reinterpret_cast<const T*>(msgs),
                          reinterpret_cast<T*>(ze_out));
               return cudaGetLastError());
}

cudaError_t launch_logsum(int dtype, const void* zv, const void* ze, int nv, int ne,
                          const int* voff, const int* vlist, const int* eoff, const int* elist,
                          int n_nets, double* logzv, double* logze, double* totals, int* flags,
                          void* scratch, size_t scratch_bytes, cudaStream_t st) {
  if (n_nets <= 0) return cudaSuccess;
  const int nblocks = (nv + ne + 127) / 128;
  // one network: block shares (two doubles and a flag word per block) in `scratch`
  const bool single = n_nets == 1 && nblocks > 0 && scratch && scratch_bytes >= (size_t)nblocks * 20;
  double* part = single ? static_cast<double*>(scratch) : nullptr;
  int* pflags = single ? reinterpret_cast<int*>(part + 2 * nblocks) : nullptr;
  if (nblocks > 0) {
    ITN_DISPATCH(dtype, log_scalars_kernel<T><<<nblocks, 128, 0, st>>>(
                            reinterpret_cast<const T*>(zv), reinterpret_cast<const T*>(ze), nv, ne, logzv, logze,
                            part, pflags);
                 break);
  }
  if (single) {
    logsum_single_kernel<<<1, 256, 0, st>>>(part, pflags, nblocks, totals, flags);
    return cudaGetLastError();
  }
  ITN_DISPATCH(dtype, logsum_kernel<T><<<n_nets, 1024, 0, st>>>(
                          reinterpret_cast<const T*>(zv), reinterpret_cast<const T*>(ze), voff,
                          vlist, eoff, elist, logzv, logze, totals, flags);
               return cudaGetLastError());
}

cudaError_t launch_init_messages(int dtype, int layers, int kind, const long long* moff,
                                 const int* bond, int nslots, void* msgs, cudaStream_t st) {
  if (nslots <= 0) return cudaSuccess;
  ITN_DISPATCH(dtype, init_messages_kernel<T><<<nslots, 64, 0, st>>>(
                          layers, kind, moff, bond, nslots, reinterpret_cast<T*>(msgs));
               return cudaGetLastError());
}

cudaError_t launch_iterate_diff(int dtype, const long long* moff, int nslots, const void* m1,
                                const void* m2, double* slot_diff, ConvState* conv, cudaStream_t st) {
  if (nslots <= 0) return cudaSuccess;
  const int block = 256, grid = (nslots * 32 + block - 1) / block;
  ITN_DISPATCH(dtype, iterate_diff_kernel<T><<<grid, block, 0, st>>>(
                          moff, nslots, reinterpret_cast<const T*>(m1),
                          reinterpret_cast<const T*>(m2), slot_diff, conv);
               return cudaGetLastError());
}

cudaError_t launch_permute(int dtype, int nv, const long long* soff, const long long* toff,
                           const int* rank_off, const int* dims, const long long* sstride,
                           const void* src, void* dst, cudaStream_t st) {
  if (nv <= 0) return cudaSuccess;
  dim3 grid(8, nv);
  ITN_DISPATCH(dtype, permute_kernel<T><<<grid, 256, 0, st>>>(
                          nv, soff, toff, rank_off, dims, sstride,
                          reinterpret_cast<const T*>(src), reinterpret_cast<T*>(dst));
               return cudaGetLastError());
}


namespace {
// the dual kernel for a CTA size: more than 128 threads take the 128-register variant
template <typename T>
void (*dual_kernel_for(int block))(GenericArgs, DualArgs) {
  return block > 128 ? bp2_dual_kernel<T, 2> : bp2_dual_kernel<T, 1>;
}
}  // namespace

cudaError_t launch_dual(int dtype, const GenericArgs& a, const DualArgs& d, const LaunchCfg& cfg, cudaStream_t st) {
  if (cfg.grid <= 0 || a.n_items <= 0) return cudaSuccess;
  if (dtype == DT_F32) {
    auto k = dual_kernel_for<float>(cfg.block);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess) return e;
    k<<<cfg.grid, cfg.block, cfg.smem, st>>>(a, d);
  } else if (dtype == DT_F64) {
    auto k = dual_kernel_for<double>(cfg.block);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess) return e;
    k<<<cfg.grid, cfg.block, cfg.smem, st>>>(a, d);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_dual_persistent(int dtype, const GenericArgs& a, const DualArgs& d, const LaunchCfg& cfg,
                                   cudaStream_t st) {
  if (cfg.grid <= 0 || cfg.grid != a.n_items || !d.grid) return cudaErrorInvalidValue;
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.gridDim = dim3(cfg.grid);
  lc.blockDim = dim3(cfg.block);
  lc.dynamicSmemBytes = cfg.smem;
  lc.stream = st;
  lc.attrs = attr;
  lc.numAttrs = 1;
  if (dtype == DT_F32) {
    auto k = dual_kernel_for<float>(cfg.block);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&lc, k, a, d);
  }
  if (dtype == DT_F64) {
    auto k = dual_kernel_for<double>(cfg.block);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&lc, k, a, d);
  }
  return cudaErrorInvalidValue;
}

int dual_max_active(int dtype, int block, size_t smem) {
  int n = 0;
  if (dtype == DT_F32) {
    auto k = dual_kernel_for<float>(block);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem);
  } else {
    auto k = dual_kernel_for<double>(block);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, smem);
  }
  return n;
}

#define ITN_REAL_DISPATCH(dtype, ...)                    \
  switch (dtype) {                                       \
    case DT_F32: { using T = float; __VA_ARGS__; }       \
    case DT_F64: { using T = double; __VA_ARGS__; }      \
    default: return cudaErrorInvalidValue;               \
  }

cudaError_t launch_grad_prep(int dtype, const long long* moff, int nslots, const void* U, void* F, void* S,
                             int normalize, cudaStream_t st) {
  if (nslots <= 0) return cudaSuccess;
  const int grid = (nslots * 32 + 255) / 256;
  ITN_REAL_DISPATCH(dtype, grad_prep_kernel<T><<<grid, 256, 0, st>>>(moff, nslots, (const T*)U, (T*)F, (T*)S,
                                                                    normalize);
                    return cudaGetLastError());
}

cudaError_t launch_grad_g(int dtype, const long long* moff, const int* rev, const int* dst_vertex, const int* eidx,
                          int nslots, const void* U, const void* m, const void* zv, const void* ze, void* g,
                          cudaStream_t st) {
  if (nslots <= 0) return cudaSuccess;
  const int grid = (nslots * 32 + 255) / 256;
  ITN_REAL_DISPATCH(dtype, grad_g_kernel<T><<<grid, 256, 0, st>>>(moff, rev, dst_vertex, eidx, nslots, (const T*)U,
                                                                 (const T*)m, (const T*)zv, (const T*)ze, (T*)g);
                    return cudaGetLastError());
}

cudaError_t launch_grad_mu(int dtype, const long long* moff, int nslots, const void* lam, const void* F,
                           const void* S, void* mu, int normalize, const int* done, cudaStream_t st) {
  if (nslots <= 0) return cudaSuccess;
  const int grid = (nslots * 32 + 255) / 256;
  ITN_REAL_DISPATCH(dtype, grad_mu_kernel<T><<<grid, 256, 0, st>>>(moff, nslots, (const T*)lam, (const T*)F,
                                                                  (const T*)S, (T*)mu, normalize, done);
                    return cudaGetLastError());
}

cudaError_t launch_adj_reset(AdjState* adj, double tol, int maxiter, cudaStream_t st) {
  adj_reset_kernel<<<1, 1, 0, st>>>(adj, tol, maxiter);
  return cudaGetLastError();
}

cudaError_t launch_adj_step(AdjState* adj, cudaStream_t st) {
  adj_step_kernel<<<1, 1, 0, st>>>(adj);
  return cudaGetLastError();
}

cudaError_t launch_reset_state(ConvState* s, double tol, int use_tol, cudaStream_t st) {
  reset_state_kernel<<<1, 1, 0, st>>>(s, tol, use_tol);
  return cudaGetLastError();
}

cudaError_t launch_step_check(ConvState* s, cudaStream_t st) {
  step_check_kernel<<<1, 1, 0, st>>>(s);
  return cudaGetLastError();
}

}  // namespace itn
