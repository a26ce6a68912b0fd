// itn_common.cuh -- element types and small device helpers shared by all kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace itn {

// Complex number with the same layout as C99 `float _Complex` / numpy complex64
// (and double/complex128): {re, im}.
template <typename R>
struct __align__(2 * sizeof(R)) cplx {
  R x, y;
};
using c64 = cplx<float>;
using c128 = cplx<double>;

template <typename T> struct real_of { using type = T; };
template <typename R> struct real_of<cplx<R>> { using type = R; };
template <typename T> struct is_cplx { static constexpr bool value = false; };
template <typename R> struct is_cplx<cplx<R>> { static constexpr bool value = true; };

__host__ __device__ __forceinline__ float zero_of(float) { return 0.f; }
__host__ __device__ __forceinline__ double zero_of(double) { return 0.0; }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> zero_of(cplx<R>) { return {R(0), R(0)}; }

template <typename T> __host__ __device__ __forceinline__ T tzero() { return zero_of(T()); }

// a * b
__device__ __forceinline__ float mul(float a, float b) { return a * b; }
__device__ __forceinline__ double mul(double a, double b) { return a * b; }
template <typename R>
__device__ __forceinline__ cplx<R> mul(cplx<R> a, cplx<R> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * b + c
__device__ __forceinline__ float fmac(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmac(double a, double b, double c) { return fma(a, b, c); }
template <typename R>
__device__ __forceinline__ cplx<R> fmac(cplx<R> a, cplx<R> b, cplx<R> c) {
  cplx<R> r;
  r.x = fma(a.x, b.x, fma(-a.y, b.y, c.x));
  r.y = fma(a.x, b.y, fma(a.y, b.x, c.y));
  return r;
}
__device__ __forceinline__ float add(float a, float b) { return a + b; }
__device__ __forceinline__ double add(double a, double b) { return a + b; }
template <typename R>
__device__ __forceinline__ cplx<R> add(cplx<R> a, cplx<R> b) { return {a.x + b.x, a.y + b.y}; }

__device__ __forceinline__ float conjx(float a) { return a; }
__device__ __forceinline__ double conjx(double a) { return a; }
template <typename R>
__device__ __forceinline__ cplx<R> conjx(cplx<R> a) { return {a.x, -a.y}; }

__device__ __forceinline__ double re_d(float a) { return a; }
__device__ __forceinline__ double re_d(double a) { return a; }
template <typename R> __device__ __forceinline__ double re_d(cplx<R> a) { return (double)a.x; }
__device__ __forceinline__ double im_d(float) { return 0.0; }
__device__ __forceinline__ double im_d(double) { return 0.0; }
template <typename R> __device__ __forceinline__ double im_d(cplx<R> a) { return (double)a.y; }

__device__ __forceinline__ bool is_zero(float a) { return a == 0.f; }
__device__ __forceinline__ bool is_zero(double a) { return a == 0.0; }
template <typename R> __device__ __forceinline__ bool is_zero(cplx<R> a) {
  return a.x == R(0) && a.y == R(0);
}

// a / s  (complex division by the textbook formula; s != 0)
__device__ __forceinline__ float divx(float a, float s) { return a / s; }
__device__ __forceinline__ double divx(double a, double s) { return a / s; }
template <typename R>
__device__ __forceinline__ cplx<R> divx(cplx<R> a, cplx<R> s) {
  R den = s.x * s.x + s.y * s.y;
  return {(a.x * s.x + a.y * s.y) / den, (a.y * s.x - a.x * s.y) / den};
}

__device__ __forceinline__ float shfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
template <typename R>
__device__ __forceinline__ cplx<R> shfl_xor(cplx<R> v, int m) {
  return {__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)};
}

// Order-preserving map of doubles to unsigned 64-bit integers, so atomicMax on the
// encoded value is a max over doubles (negative values included).
__device__ __forceinline__ unsigned long long enc_double(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double dec_double(unsigned long long u) {
  unsigned long long v = (u & 0x8000000000000000ull) ? (u & ~0x8000000000000000ull) : ~u;
  double d;
  memcpy(&d, &v, sizeof(d));
  return d;
}

}  // namespace itn
