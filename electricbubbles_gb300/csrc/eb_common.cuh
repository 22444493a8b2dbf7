// Shared device helpers for the GB300 ElectricBubbles library: complex arithmetic on
// double2/float2, launch bookkeeping and error propagation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/eb_gb300.h"

#define EB_PI 3.14159265358979323846

// ---------------------------------------------------------------------------------
// Complex helpers. Values are (re, im) pairs; T is double or float.
// ---------------------------------------------------------------------------------
template <typename T> struct cvec;
template <> struct cvec<double> { typedef double2 type; };
template <> struct cvec<float> { typedef float2 type; };

template <typename T> using c_t = typename cvec<T>::type;

template <typename T> __host__ __device__ __forceinline__ c_t<T> cmk(T re, T im) {
  c_t<T> r;
  r.x = re;
  r.y = im;
  return r;
}
template <typename T> __host__ __device__ __forceinline__ c_t<T> cadd(c_t<T> a, c_t<T> b) {
  return cmk<T>(a.x + b.x, a.y + b.y);
}
template <typename T> __host__ __device__ __forceinline__ c_t<T> csub(c_t<T> a, c_t<T> b) {
  return cmk<T>(a.x - b.x, a.y - b.y);
}
template <typename T> __host__ __device__ __forceinline__ c_t<T> cmul(c_t<T> a, c_t<T> b) {
  return cmk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> __host__ __device__ __forceinline__ c_t<T> cmulc(c_t<T> a, c_t<T> b) {
  return cmk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T> __host__ __device__ __forceinline__ c_t<T> cconj(c_t<T> a) {
  return cmk<T>(a.x, -a.y);
}
template <typename T> __host__ __device__ __forceinline__ c_t<T> cscale(c_t<T> a, T s) {
  return cmk<T>(a.x * s, a.y * s);
}
// acc += a * b
template <typename T> __host__ __device__ __forceinline__ void cfma(c_t<T>& acc, c_t<T> a, c_t<T> b) {
  acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}
// acc += s * a (s real)
template <typename T> __host__ __device__ __forceinline__ void crfma(c_t<T>& acc, T s, c_t<T> a) {
  acc.x = fma(s, a.x, acc.x);
  acc.y = fma(s, a.y, acc.y);
}
template <typename T> __host__ __device__ __forceinline__ c_t<T> cinv(c_t<T> a) {
  T d = T(1) / (a.x * a.x + a.y * a.y);
  return cmk<T>(a.x * d, -a.y * d);
}
template <typename T> __host__ __device__ __forceinline__ c_t<T> cdiv(c_t<T> a, c_t<T> b) {
  return cmul<T>(a, cinv<T>(b));
}

__device__ __forceinline__ double2 to_d2(float2 a) { return make_double2(a.x, a.y); }
__device__ __forceinline__ float2 to_f2(double2 a) { return make_float2((float)a.x, (float)a.y); }

// Warp sum of a double / float.
template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------------
// Error handling: every entry point returns an eb_status code (eb_gb300.h).
// ---------------------------------------------------------------------------------
#define EB_CUDA_TRY(call)                                      \
  do {                                                         \
    cudaError_t _e = (call);                                   \
    if (_e != cudaSuccess) {                                   \
      eb_set_last_cuda_error(_e, #call, __FILE__, __LINE__);   \
      return EB_ERR_CUDA;                                      \
    }                                                          \
  } while (0)

#define EB_TRY(call)              \
  do {                            \
    int _s = (call);              \
    if (_s != EB_OK) return _s;   \
  } while (0)

void eb_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);
void eb_set_last_error_msg(const char* msg);
