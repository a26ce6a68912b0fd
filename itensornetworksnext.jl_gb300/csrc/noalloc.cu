// noalloc.cu -- Bethe log-norm of a network whose data already lives on the GPU, computed
// without allocating any device memory.
//
// Who needs this: callers whose device memory is owned by their own pooling allocator --
// a Julia process whose CUDA.jl memory pool holds the GPU, or a serving process that
// reserves all of HBM at start-up -- cannot let a library call cudaMalloc: the call either
// fails because the pool already holds the memory or silently escapes the pool's
// accounting.  itn_logz_static_scratch takes device pointers to everything it reads and
// writes and keeps its intermediates (vertex scalars Z_u, edge scalars Z_e and per-CTA
// contraction buffers) in one file-scope __device__ array of kStaticScratchBytes.
//
// The array belongs to the process: every GPU that loads the library holds it until the
// process exits.  All calls share it and it keeps the last call's contents; the one word
// that must start at zero (the bad-vertex bits) is cleared on the stream at the start of
// every call, and every other entry a call reads is written earlier in the same call.  Two
// calls that overlap on the GPU (different streams, or different host threads on one
// device) race on it and must be ordered by the caller.
//
// Limits checked on the device, where the caller's arrays are: a vertex with more than
// kNaMaxLegs legs, a vertex whose tensor exceeds max_tensor_elems, and (one-layer networks)
// a vertex whose physical dimension is not 1 each make that Z_u NaN and set a flag bit
// (bits 3, 4 and 5 of d_flags) instead of reading or writing out of bounds.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current (host code may not use the symbol
// itself: on the host its name is only a stand-in, not a device address).  That first
// call should therefore come before any stream capture on that device.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "../../include/itn_gpu.h"
#include "itn_common.cuh"

namespace itn {
namespace {

constexpr size_t kStaticScratchBytes = 16u << 20;  // 16 MiB
constexpr int kMaxDevices = 64;
constexpr int kNaThreads = 256;
constexpr int kNaMaxLegs = 16;              // legs per vertex (shared index tables)
constexpr size_t kNaHeaderBytes = 256;      // bad-vertex bits at the start of the array
constexpr int kBadTooLarge = 8;             // flag bit 3: tensor larger than max_tensor_elems
constexpr int kBadTooManyLegs = 16;         // flag bit 4: more than kNaMaxLegs legs
constexpr int kBadPlainPhys = 32;           // flag bit 5: one-layer vertex with phys != 1

__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

template <typename T>
__device__ T na_block_sum(T v, T* red) {
  for (int o = 16; o >= 1; o >>= 1) v = add(v, shfl_xor(v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  T r = tzero<T>();
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = add(r, red[w]);
  __syncthreads();
  return r;
}

// Z_u = full contraction of vertex u's factor with all incoming messages
// (vertex_scalar, messagecache.jl:139-143).  Two-layer: absorb every leg into the ket
// side (ping-pong through this CTA's two scratch planes), then sum with conj(A).
template <typename T>
__global__ void na_vertex_kernel(int layers, int nv, const int* off, const int* rev, const int* bond,
                                 const int* phys, const long long* toff, const long long* moff,
                                 const T* tens, const T* msgs, T* zv, T* planes, long long plane_elems,
                                 long long max_elems, int* bad) {
  __shared__ int dims[kNaMaxLegs], inner[kNaMaxLegs];
  __shared__ T red[32];
  T* p0 = planes + (size_t)blockIdx.x * 2 * plane_elems;
  T* p1 = p0 + plane_elems;
  for (int u = blockIdx.x; u < nv; u += gridDim.x) {
    const int s0 = off[u], z = off[u + 1] - s0;
    const long long n_ll = toff[u + 1] - toff[u];
    // block-uniform checks (every thread reads the same values): a vertex the shared tables,
    // the scratch planes or the one-layer sum cannot hold gets Z_u = NaN and a flag bit
    const int why = (z < 0 || z > kNaMaxLegs) ? kBadTooManyLegs
                    : (layers == 2 && (n_ll > max_elems || n_ll > plane_elems)) ? kBadTooLarge
                    : (layers == 1 && phys[u] != 1) ? kBadPlainPhys : 0;
    if (why) {
      if (threadIdx.x == 0) {
        T nanv = tzero<T>();
        if constexpr (is_cplx<T>::value) nanv.x = nan("");
        else nanv = (T)nan("");
        zv[u] = nanv;
        atomicOr(bad, why);
      }
      continue;
    }
    if (threadIdx.x == 0) {
      int in = 1;
      for (int l = z - 1; l >= 0; --l) {
        dims[l] = bond[s0 + l];
        inner[l] = in;
        in *= dims[l];
      }
    }
    __syncthreads();
    const T* A = tens + toff[u];
    const int n = (int)n_ll;
    T acc = tzero<T>();
    if (layers == 2) {
      const T* cur = A;
      T* nxt = p0;
      for (int l = 0; l < z; ++l) {
        const int D = dims[l], in = inner[l], outer = n / (D * in);
        const T* m = msgs + moff[rev[s0 + l]];
        for (int p = threadIdx.x; p < outer * in; p += blockDim.x) {
          const int o = p / in, i = p - o * in;
          for (int b = 0; b < D; ++b) {
            T s = tzero<T>();
            for (int k = 0; k < D; ++k) s = fmac(cur[(o * D + k) * in + i], m[b * D + k], s);
            nxt[(o * D + b) * in + i] = s;
          }
        }
        __syncthreads();
        cur = nxt;
        nxt = (nxt == p0) ? p1 : p0;
      }
      for (int j = threadIdx.x; j < n; j += blockDim.x) acc = fmac(cur[j], conjx(A[j]), acc);
    } else {
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        T p = A[j];
        for (int l = 0; l < z; ++l) p = mul(p, msgs[moff[rev[s0 + l]] + (j / inner[l]) % dims[l]]);
        acc = add(acc, p);
      }
    }
    acc = na_block_sum(acc, red);
    if (threadIdx.x == 0) zv[u] = acc;
    __syncthreads();
  }
}

// Z_e = sum_j m_{u->v}[j] m_{v->u}[j] for every slot s < rev[s] (edge_scalar,
// messagecache.jl:153-157), stored at ze[s].
template <typename T>
__global__ void na_edge_kernel(int nslots, const int* rev, const long long* moff, const T* msgs, T* ze) {
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= nslots || s > rev[s]) return;
  T acc = tzero<T>();
  for (long long j = lane; j < moff[s + 1] - moff[s]; j += 32) acc = fmac(msgs[moff[s] + j], msgs[moff[rev[s]] + j], acc);
  for (int o = 16; o >= 1; o >>= 1) acc = add(acc, shfl_xor(acc, o));
  if (lane == 0) ze[s] = acc;
}

template <typename T>
__device__ __forceinline__ void na_log(T z, double& re, double& im) {
  const double a = re_d(z), b = im_d(z);
  if constexpr (is_cplx<T>::value) {
    re = 0.5 * log(a * a + b * b);
    im = atan2(b, a);
  } else {
    if (a < 0) { re = log(-a); im = M_PI; }
    else { re = log(a); im = 0.0; }
  }
}

// One block: total = sum_u log Z_u - sum_e log Z_e in FP64 (bethe_free_energy,
// messagecache.jl:185-201); flags bit0 any Re Z_u < 0, bit1 any Re Z_e < 0, bit2 any Z_e == 0.
// Bits 3-5 come from the vertex kernel's bad-vertex word.
template <typename T>
__global__ void na_sum_kernel(int nv, int nslots, const int* rev, const T* zv, const T* ze, double* total,
                              int* flags, const int* bad) {
  __shared__ double sre[32], sim[32];
  __shared__ int sfl[32];
  double are = 0, aim = 0;
  int fl = 0;
  for (int u = threadIdx.x; u < nv; u += blockDim.x) {
    double re, im;
    na_log(zv[u], re, im);
    if (re_d(zv[u]) < 0) fl |= 1;
    are += re;
    aim += im;
  }
  for (int s = threadIdx.x; s < nslots; s += blockDim.x) {
    if (s > rev[s]) continue;
    double re, im;
    na_log(ze[s], re, im);
    if (re_d(ze[s]) < 0) fl |= 2;
    if (is_zero(ze[s])) fl |= 4;
    are -= re;
    aim -= im;
  }
  for (int o = 16; o >= 1; o >>= 1) {
    are += __shfl_xor_sync(0xffffffffu, are, o);
    aim += __shfl_xor_sync(0xffffffffu, aim, o);
    fl |= __shfl_xor_sync(0xffffffffu, fl, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sre[threadIdx.x >> 5] = are;
    sim[threadIdx.x >> 5] = aim;
    sfl[threadIdx.x >> 5] = fl;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0, i = 0;
    int f = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      r += sre[w];
      i += sim[w];
      f |= sfl[w];
    }
    total[0] = r;
    total[1] = i;
    *flags = f | *bad;
  }
}

void set_err(char* buf, int len, const char* msg) {
  if (buf && len > 0) {
    strncpy(buf, msg, (size_t)len - 1);
    buf[len - 1] = '\0';
  }
}

template <typename T>
int run_static(cudaStream_t st, int sm_count, void* scratch, int layers, int64_t nv, int64_t nslots,
               int64_t max_tensor, const int32_t* off, const int32_t* rev, const int32_t* bond,
               const int32_t* phys, const int64_t* toff, const int64_t* moff, const void* tens,
               const void* msgs, double* total, int32_t* flags, char* errbuf, int errlen) {
  const size_t es = sizeof(T);
  // checked before any size arithmetic so that nothing below can wrap around
  if (layers == 2 && max_tensor > (int64_t)(kStaticScratchBytes / (2 * es))) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "max_tensor_elems %lld needs more than the static scratch of %zu bytes for one CTA's planes",
             (long long)max_tensor, kStaticScratchBytes);
    set_err(errbuf, errlen, msg);
    return ITN_ERR_ARG;
  }
  const size_t zv_bytes = ((size_t)nv * es + 255) & ~(size_t)255;
  const size_t ze_bytes = ((size_t)nslots * es + 255) & ~(size_t)255;
  const long long plane = (max_tensor + 31) & ~31LL;
  const size_t per_cta = layers == 2 ? 2 * (size_t)plane * es : 0;
  if (kNaHeaderBytes + zv_bytes + ze_bytes + per_cta > kStaticScratchBytes) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "network needs %zu bytes of scratch (vertex/edge scalars %zu, one CTA's planes %zu); "
             "the static scratch holds %zu",
             kNaHeaderBytes + zv_bytes + ze_bytes + per_cta, zv_bytes + ze_bytes, per_cta, kStaticScratchBytes);
    set_err(errbuf, errlen, msg);
    return ITN_ERR_ARG;
  }
  int grid = (int)std::min<int64_t>(nv, (int64_t)sm_count * 2);
  if (per_cta)
    grid = (int)std::min<size_t>(grid, (kStaticScratchBytes - kNaHeaderBytes - zv_bytes - ze_bytes) / per_cta);
  grid = std::max(grid, 1);
  unsigned char* base = reinterpret_cast<unsigned char*>(scratch);
  int* bad = reinterpret_cast<int*>(base);
  T* zv = reinterpret_cast<T*>(base + kNaHeaderBytes);
  T* ze = reinterpret_cast<T*>(base + kNaHeaderBytes + zv_bytes);
  T* planes = reinterpret_cast<T*>(base + kNaHeaderBytes + zv_bytes + ze_bytes);
  // the bad-vertex bits are the only scratch that must start at zero
  cudaError_t ce = cudaMemsetAsync(bad, 0, sizeof(int), st);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    set_err(errbuf, errlen, cudaGetErrorString(ce));
    return ITN_ERR_CUDA;
  }
  if (nv > 0)
    na_vertex_kernel<T><<<grid, kNaThreads, 0, st>>>(layers, (int)nv, off, rev, bond, phys,
                                                    reinterpret_cast<const long long*>(toff),
                                                    reinterpret_cast<const long long*>(moff),
                                                    reinterpret_cast<const T*>(tens),
                                                    reinterpret_cast<const T*>(msgs), zv, planes, plane,
                                                    (long long)max_tensor, bad);
  if (nslots > 0)
    na_edge_kernel<T><<<(int)((nslots * 32 + 255) / 256), 256, 0, st>>>(
        (int)nslots, rev, reinterpret_cast<const long long*>(moff), reinterpret_cast<const T*>(msgs), ze);
  na_sum_kernel<T><<<1, 256, 0, st>>>((int)nv, (int)nslots, rev, zv, ze, total, flags, bad);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_err(errbuf, errlen, cudaGetErrorString(e));
    return ITN_ERR_CUDA;
  }
  return ITN_OK;
}

}  // namespace
}  // namespace itn

using namespace itn;

extern "C" int32_t itn_logz_static_scratch(int32_t device, void* stream, int32_t dtype, int32_t layers,
                                           int64_t nv, int64_t nslots, int64_t max_tensor_elems,
                                           const int32_t* d_off, const int32_t* d_rev,
                                           const int32_t* d_bond, const int32_t* d_phys,
                                           const int64_t* d_toff, const int64_t* d_moff,
                                           const void* d_tensors, const void* d_messages,
                                           double* d_total, int32_t* d_flags, char* errbuf,
                                           int32_t errbuf_len) {
  if (device < 0 || device >= kMaxDevices) {
    set_err(errbuf, errbuf_len, "device index out of range");
    return ITN_ERR_ARG;
  }
  if (layers != 1 && layers != 2) {
    set_err(errbuf, errbuf_len, "layers must be 1 or 2");
    return ITN_ERR_ARG;
  }
  if (nv < 0 || nslots < 0 || max_tensor_elems < 1 || nv > (1LL << 30) || nslots > (1LL << 30)) {
    set_err(errbuf, errbuf_len, "sizes out of range");
    return ITN_ERR_ARG;
  }
  if (!d_off || !d_rev || !d_bond || !d_phys || !d_toff || !d_moff || !d_tensors || !d_messages || !d_total ||
      !d_flags) {
    set_err(errbuf, errbuf_len, "null device pointer");
    return ITN_ERR_ARG;
  }
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != device && cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    set_err(errbuf, errbuf_len, "cudaSetDevice failed");
    return ITN_ERR_CUDA;
  }
  int rc = ITN_OK;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[device]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        set_err(errbuf, errbuf_len, "cudaGetSymbolAddress of the static scratch failed");
        rc = ITN_ERR_CUDA;
      } else {
        g_scratch_ptr[device] = p;
      }
    }
    scratch = g_scratch_ptr[device];
  }
  if (rc == ITN_OK) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    switch (dtype) {
      case ITN_F32:
        rc = run_static<float>(st, sms, scratch, layers, nv, nslots, max_tensor_elems, d_off, d_rev, d_bond, d_phys,
                               d_toff, d_moff, d_tensors, d_messages, d_total, d_flags, errbuf, errbuf_len);
        break;
      case ITN_F64:
        rc = run_static<double>(st, sms, scratch, layers, nv, nslots, max_tensor_elems, d_off, d_rev, d_bond, d_phys,
                                d_toff, d_moff, d_tensors, d_messages, d_total, d_flags, errbuf, errbuf_len);
        break;
      case ITN_C64:
        rc = run_static<c64>(st, sms, scratch, layers, nv, nslots, max_tensor_elems, d_off, d_rev, d_bond, d_phys,
                             d_toff, d_moff, d_tensors, d_messages, d_total, d_flags, errbuf, errbuf_len);
        break;
      case ITN_C128:
        rc = run_static<c128>(st, sms, scratch, layers, nv, nslots, max_tensor_elems, d_off, d_rev, d_bond, d_phys,
                              d_toff, d_moff, d_tensors, d_messages, d_total, d_flags, errbuf, errbuf_len);
        break;
      default:
        set_err(errbuf, errbuf_len, "unknown dtype");
        rc = ITN_ERR_ARG;
    }
  }
  if (prev >= 0 && prev != device) cudaSetDevice(prev);
  return rc;
}
