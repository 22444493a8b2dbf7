// Per-drop spectral building blocks shared by the spectral kernels and their adjoints:
// one thread block per drop, its samples and twiddles in shared memory. The FFT is an
// in-place radix-2 decimation-in-time transform with the unnormalised DCFFTF (exp(-i..))
// / DCFFTB (exp(+i..)) conventions (dcfft.f:1-77, 715-790), for power-of-two sizes.
#pragma once

#include "eb_internal.h"

namespace {

// tw[j] = exp(+2 pi i j / N), j < N/2: one table serves both directions (the forward
// transform uses the conjugate) and every size n dividing N.
__device__ __forceinline__ void make_twiddles(double2* tw, int N) {
  for (int j = threadIdx.x; j < N / 2; j += blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)j / (double)N, &s, &c);
    tw[j] = make_double2(c, s);
  }
}

// In-place FFT of a[0..n): sign = -1 is DCFFTF's exp(-i..), +1 is DCFFTB's exp(+i..).
__device__ void smem_fft(double2* a, int n, const double2* tw, int N, int sign) {
  int logn = 31 - __clz(n);
  int mult = N / n;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int j = (int)(__brev((unsigned)i) >> (32 - logn));
    if (i < j) {
      double2 t = a[i];
      a[i] = a[j];
      a[j] = t;
    }
  }
  __syncthreads();
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1, step = (n / len) * mult;
    for (int b = threadIdx.x; b < n / 2; b += blockDim.x) {
      int grp = b / half, j = b - grp * half;
      int i = grp * len + j;
      double2 t = tw[j * step];
      if (sign < 0) t.y = -t.y;
      double2 u = a[i], v = cmul<double>(a[i + half], t);
      a[i] = make_double2(u.x + v.x, u.y + v.y);
      a[i + half] = make_double2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
}

// Derivative in Fourier space: c_k -> i k c_k / n for |k| < n/2, Nyquist and mean zeroed
// (FDIFFF, dcfft.f:1395-1425).
__device__ void spectral_deriv(double2* a, int n) {
  double inv = 1.0 / (double)n;
  for (int m = threadIdx.x; m < n; m += blockDim.x) {
    int k = (m <= n / 2) ? m : m - n;
    if (m == n / 2 || m == 0) {
      a[m] = make_double2(0.0, 0.0);
    } else {
      double2 c = a[m];
      double f = (double)k * inv;
      a[m] = make_double2(-f * c.y, f * c.x);
    }
  }
  __syncthreads();
}

__device__ double block_sum_d(double v, double* red) {
  v = warp_sum<double>(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
    r = warp_sum<double>(r);
    if (l == 0) red[0] = r;
  }
  __syncthreads();
  r = red[0];
  __syncthreads();
  return r;
}

// Antiderivative in Fourier space (FOURINT, electric.f:1307-1331): c_k -> c_k/(i k),
// mean and Nyquist dropped.
__device__ void spectral_int(double2* a, int n) {
  for (int m = threadIdx.x; m < n; m += blockDim.x) {
    if (m == 0 || m == n / 2) {
      a[m] = make_double2(0.0, 0.0);
    } else {
      double k = (double)((m <= n / 2) ? m : m - n);
      double2 c = a[m];
      a[m] = make_double2(c.y / k, -c.x / k);  // c / (i k)
    }
  }
  __syncthreads();
}

__device__ __forceinline__ double powi25(double x) {
  double r = 1.0;
  int e = 25;
  while (e > 0) {
    if (e & 1) r *= x;
    x *= x;
    e >>= 1;
  }
  return r;
}

}  // namespace
