// Per-drop spectral kernels: one thread block per drop, the drop's samples and the
// FFT twiddles resident in shared memory (one HBM read and one write per transform).
// The FFT is an in-place radix-2 decimation-in-time transform with the unnormalised
// DCFFTF (exp(-i..)) / DCFFTB (exp(+i..)) conventions (dcfft.f:1-77, 715-790);
// drop sizes must be powers of two (as in every configuration of the reference runs).
//
// Routines: FDIFFF (dcfft.f:1371-1428), EXTRACTDAT (electric.f:636-716), the FINTERC /
// FINTER interpolation and alternating-point rule of PVINTEV (pv_integral.f:53-345),
// DIRICH_NEU_MAP (laplace.f:266-331) and INTERFACENEW (electric.f:791-912).
#include <algorithm>
#include <cmath>
#include <vector>

#include "eb_fft.cuh"
#include "eb_internal.h"

namespace {

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }
constexpr int SBS = 512;

// FDIFFF of each drop's complex samples.
__global__ void k_fdiff(const int* __restrict__ start, const double2* __restrict__ f,
                        double2* __restrict__ df, int nmax) {
  extern __shared__ double2 sm[];
  int b = blockIdx.x;
  int i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* tw = sm + nmax;
  make_twiddles(tw, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = f[i0 + i];
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) df[i0 + i] = a[i];
}

// Same, for a real input (imaginary part zero).
__global__ void k_fdiff_real(const int* __restrict__ start, const double* __restrict__ f,
                             double2* __restrict__ df, int nmax) {
  extern __shared__ double2 sm[];
  int b = blockIdx.x;
  int i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* tw = sm + nmax;
  make_twiddles(tw, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(f[i0 + i], 0.0);
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) df[i0 + i] = a[i];
}

// EXTRACTDAT per drop: zk = mean of z (its zero Fourier mode / n), z' = FDIFFF(z),
// z'' = FDIFFF(z'), kappa = -(x'y'' - y'x'')/|z'|^3, ckern = -z''/z', tha = -kappa |z'|,
// dz = -z', dsda = |dz|, area = 2 pi mean(y Re(dz)).
__global__ void k_extractdat(const int* __restrict__ start, const double2* __restrict__ z,
                             double2* __restrict__ zk, double2* __restrict__ dz,
                             double* __restrict__ dsda, double* __restrict__ kappa,
                             double2* __restrict__ ckern, double* __restrict__ tha,
                             double* __restrict__ area, int nmax) {
  extern __shared__ double2 sm[];
  __shared__ double red[32];
  int b = blockIdx.x;
  int i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* d1 = sm + nmax;
  double2* tw = d1 + nmax;
  make_twiddles(tw, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = z[i0 + i];
  smem_fft(a, n, tw, n, -1);
  if (threadIdx.x == 0) zk[b] = make_double2(a[0].x / n, a[0].y / n);
  __syncthreads();
  spectral_deriv(a, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) d1[i] = a[i];
  smem_fft(d1, n, tw, n, +1);  // d1 = z'
  // second derivative from the samples of z' (FDIFFF applied twice, as the reference)
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = d1[i];
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  smem_fft(a, n, tw, n, +1);  // a = z''
  double ysum = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double xd = d1[i].x, yd = d1[i].y, xdd = a[i].x, ydd = a[i].y;
    double dsdt = sqrt(xd * xd + yd * yd);
    double kap = -(xd * ydd - yd * xdd) / (dsdt * dsdt * dsdt);
    int t = i0 + i;
    kappa[t] = kap;
    double2 ck = cdiv<double>(make_double2(xdd, ydd), make_double2(xd, yd));
    ckern[t] = make_double2(-ck.x, -ck.y);
    tha[t] = -kap * dsdt;
    dz[t] = make_double2(-xd, -yd);
    dsda[t] = dsdt;
    ysum += z[t].y * (-xd);
  }
  ysum = block_sum_d(ysum, red);
  if (threadIdx.x == 0) area[b] = 2.0 * EB_PI * ysum / (double)n;
}

// PVINTEV interpolation (pv_integral.f:143-166): per drop, FINTERC of ucmplx and FINTER
// of x and y from n to 2n points; charges QA = U2 h on the odd fine nodes (0-based),
// zero on the even ones (the original nodes). One block per (drop, component):
// blockIdx.y = 0 the density, 1 and 2 the x and y of the fine points (launched when the
// positions are wanted). The three transforms are independent, and a drop's FP64
// transforms are bound by the FP64 rate of one SM, so each gets its own.
__global__ void k_pv_interp(const int* __restrict__ start, const double2* __restrict__ z,
                            const double2* __restrict__ uc, double2* __restrict__ zf,
                            double2* __restrict__ qf, int nmax) {
  extern __shared__ double2 sm[];
  int b = blockIdx.x;
  int i0 = start[b], n = start[b + 1] - i0, nf = 2 * n;
  double2* w = sm;             // 2n: coarse transform in w[0..n), then the padded spectrum
  double2* tw = sm + 2 * nmax; // n twiddles of the size-2n transform
  make_twiddles(tw, nf);
  double h = 2.0 * EB_PI / (double)n, inv = 1.0 / (double)n;
  int ny = n / 2;
  const int comp = blockIdx.y;
  {
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double2 v;
      if (comp == 0) v = uc[i0 + i];
      else if (comp == 1) v = make_double2(z[i0 + i].x, 0.0);
      else v = make_double2(z[i0 + i].y, 0.0);
      w[i] = v;
    }
    smem_fft(w, n, tw, nf, -1);
    if (threadIdx.x == 0) {
      if (comp == 0) {
        w[ny] = make_double2(0.0, 0.0);  // FINTERC, pv_integral.f:307
      } else {
        // FINTER zeroes WORK(IPT+2*NYK-1) and WORK(IPT+2*NYK) (pv_integral.f:235-236):
        // the imaginary part of mode n/2-1 and the real part of mode n/2.
        w[ny - 1].y = 0.0;
        w[ny].x = 0.0;
      }
    }
    __syncthreads();
    // negative modes n/2+1..n-1 move to 2n-(n-m) = n+m; the gap in between is zero
    for (int m = ny + 1 + threadIdx.x; m < n; m += blockDim.x) w[m + n] = w[m];
    __syncthreads();
    for (int m = ny + 1 + threadIdx.x; m <= n + ny; m += blockDim.x) w[m] = make_double2(0.0, 0.0);
    __syncthreads();
    for (int m = threadIdx.x; m < nf; m += blockDim.x) w[m] = make_double2(w[m].x * inv, w[m].y * inv);
    smem_fft(w, nf, tw, nf, +1);
    for (int m = threadIdx.x; m < nf; m += blockDim.x) {
      int t = 2 * i0 + m;
      if (comp == 0) qf[t] = (m & 1) ? make_double2(w[m].x * h, w[m].y * h) : make_double2(0.0, 0.0);
      else if (comp == 1) zf[t].x = w[m].x;
      else zf[t].y = w[m].x;
    }
  }
}

// GETFOURIER (electric.f:531-570) per drop: c = DCFFTF(z)/nd, fmode_0 = |c_0|,
// fmode_i = |c_i| + |c_{nd-i}| (i < nd/2), and the doubling test: a mode among the ten
// below the Nyquist mode (i = nd/2-10 .. nd/2-1) above 1e-11.
__global__ void k_getfourier(const int* __restrict__ start, const double2* __restrict__ z,
                             double* __restrict__ fmode, int* __restrict__ idoub, int nmax) {
  extern __shared__ double2 sm[];
  __shared__ int s_flag;
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0, h = n / 2;
  double2* a = sm;
  double2* tw = sm + nmax;
  make_twiddles(tw, n);
  if (threadIdx.x == 0) s_flag = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = z[i0 + i];
  smem_fft(a, n, tw, n, -1);
  const double inv = 1.0 / (double)n;
  for (int i = threadIdx.x; i < h; i += blockDim.x) {
    const double2 c = a[i];
    double f = hypot(c.x, c.y) * inv;
    if (i > 0) f += hypot(a[n - i].x, a[n - i].y) * inv;
    if (fmode) fmode[i0 + i] = f;
    if (i >= h - 10 && i >= 1 && f > 1e-11) s_flag = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) idoub[b] = s_flag;
}

// DOUBLE (electric.f:721-757): a flagged drop's nodes resampled to 2 nd points by
// FINTERC's spectral interpolation (pv_integral.f:276-328: Nyquist mode dropped, the
// spectrum zero-padded); other drops copied.
__global__ void k_double(const int* __restrict__ start, const int* __restrict__ start2,
                         const int* __restrict__ flag, const double2* __restrict__ z,
                         double2* __restrict__ z2, int nmax) {
  extern __shared__ double2 sm[];
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0, o0 = start2[b];
  if (!flag[b]) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) z2[o0 + i] = z[i0 + i];
    return;
  }
  const int nf = 2 * n, ny = n / 2;
  double2* w = sm;              // 2 n
  double2* tw = sm + 2 * nmax;  // twiddles of the size-2n transform
  make_twiddles(tw, nf);
  for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = z[i0 + i];
  smem_fft(w, n, tw, nf, -1);
  if (threadIdx.x == 0) w[ny] = make_double2(0.0, 0.0);
  __syncthreads();
  for (int m = ny + 1 + threadIdx.x; m < n; m += blockDim.x) w[m + n] = w[m];
  __syncthreads();
  for (int m = ny + threadIdx.x; m <= n + ny; m += blockDim.x) w[m] = make_double2(0.0, 0.0);
  __syncthreads();
  const double inv = 1.0 / (double)n;
  for (int m = threadIdx.x; m < nf; m += blockDim.x) w[m] = make_double2(w[m].x * inv, w[m].y * inv);
  smem_fft(w, nf, tw, nf, +1);
  for (int m = threadIdx.x; m < nf; m += blockDim.x) z2[o0 + m] = w[m];
}

// PHICMPLX = -FIELD/(2 pi i) at the even fine nodes (pv_integral.f:194-201).
__global__ void k_pv_extract(int nbk, const double2* __restrict__ cf, double2* __restrict__ phi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbk) return;
  double2 c = cf[2 * i];
  // -c/(2 pi i) = i c / (2 pi)
  phi[i] = make_double2(-c.y / (2.0 * EB_PI), c.x / (2.0 * EB_PI));
}

__global__ void k_dtn_pre(int nbk, const double* __restrict__ u, const double2* __restrict__ dz,
                          double2* __restrict__ uc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbk) return;
  uc[i] = make_double2(u[i] * dz[i].x, u[i] * dz[i].y);
}

// zphi = -u/2 - PV - z; phi = Re, psi = Im (laplace.f:304-311).
__global__ void k_dtn_mid(int nbk, const double* __restrict__ u, const double2* __restrict__ pv,
                          const double2* __restrict__ z, double* __restrict__ phi,
                          double* __restrict__ psi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbk) return;
  double zx = -0.5 * u[i] - pv[i].x - z[i].x;
  double zy = -pv[i].y - z[i].y;
  phi[i] = zx;
  psi[i] = zy;
}

__global__ void k_dtn_post(int nbk, const double2* __restrict__ dpsi, const double* __restrict__ dsda,
                           double* __restrict__ dphi) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbk) return;
  dphi[i] = -dpsi[i].x / dsda[i];
}

// REFSING (reflect.f:28-86) with zb = 0, as SETVELF and INTERFACENEW call it: the images
// across the wall y = 0 of the log sources zc at the drop centres zk, added to phi, phi'
// and psi at z. z lies above the wall and conj(zk) below it, so z - conj(zk) has a
// positive imaginary part and its principal logarithm needs no branch care.
__device__ void refsing_zc(double2 z, int k, const double2* __restrict__ zk, const double2* __restrict__ zc,
                           double2& phi, double2& phip, double2& psi) {
  for (int j = 0; j < k; ++j) {
    const double2 c = zc[j], kk = zk[j];
    const double2 zd = make_double2(z.x - kk.x, z.y + kk.y);  // z - conj(zk)
    const double2 lg = make_double2(log(hypot(zd.x, zd.y)), atan2(zd.y, zd.x));
    const double2 r1 = cinv<double>(zd), r2 = cmul<double>(r1, r1);
    phi = csub<double>(phi, cmul<double>(c, lg));
    phip = csub<double>(phip, cmul<double>(c, r1));
    psi = csub<double>(psi, cmul<double>(cconj<double>(c), lg));
    const double2 a1 = cmul<double>(cconj<double>(c), make_double2(0.0, 2.0 * kk.y));  // conj(zc)(zk - conj(zk))
    const double2 b1 = cadd<double>(cmul<double>(c, cconj<double>(kk)), a1);
    const double2 b2 = cmul<double>(a1, cconj<double>(kk));
    phi = cadd<double>(phi, cmul<double>(a1, r1));
    phip = csub<double>(phip, cmul<double>(a1, r2));
    psi = cadd<double>(psi, cadd<double>(cmul<double>(b1, r1), cmul<double>(b2, r2)));
  }
}

// INTERFACENEW corrections and normal velocity (electric.f:845-882); with iwall the
// reflected log sources of REFSING join the far field (electric.f:868-872).
__global__ void k_velocity(int nbk, int k, const int* __restrict__ drop_of,
                           const double2* __restrict__ z, const double2* __restrict__ dz,
                           const double* __restrict__ dsda, const double* __restrict__ kappa,
                           const double* __restrict__ hpt, const double2* __restrict__ ckern,
                           const double2* __restrict__ u, const double2* __restrict__ udot,
                           const double2* __restrict__ gw, const double2* __restrict__ zc,
                           const double2* __restrict__ zk, int any_zc, int iwall, double cap,
                           double* __restrict__ un, double* __restrict__ fluxpart, double2* __restrict__ gout) {
  __shared__ double red[32];
  double fl = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbk; t += gridDim.x * blockDim.x) {
    double hb = hpt[t], s = dsda[t];
    double2 zn = make_double2(dz[t].y / s, -dz[t].x / s);  // -i dz / |dz|
    double2 zz = z[t], uu = u[t];
    // zcorr = (0.5 h 2 Re(ckern) u - 2 h udot) / (2 pi i)
    double2 zcorr = make_double2(hb * ckern[t].x * uu.x - 2.0 * hb * udot[t].x,
                                 hb * ckern[t].x * uu.y - 2.0 * hb * udot[t].y);
    zcorr = make_double2(zcorr.y / (2.0 * EB_PI), -zcorr.x / (2.0 * EB_PI));
    double adz = sqrt(dz[t].x * dz[t].x + dz[t].y * dz[t].y);
    double c1 = hb * adz * 0.5 * kappa[t] / EB_PI;
    double2 zself = cscale<double>(cmul<double>(cconj<double>(uu), cmul<double>(zn, zn)), c1);
    double2 g = gw[t];
    g = cadd<double>(g, cadd<double>(zself, zcorr));
    double2 zck = make_double2(0.0, 0.0);
    if (any_zc) {
      for (int nb = 0; nb < k; ++nb) {
        double2 zd = csub<double>(zz, zk[nb]);
        double2 c = zc[nb];
        double lg = log(sqrt(zd.x * zd.x + zd.y * zd.y));
        zck = cadd<double>(zck, cscale<double>(c, 2.0 * lg));
        zck = cadd<double>(zck, cdiv<double>(cmul<double>(cconj<double>(c), zd), cconj<double>(zd)));
      }
    }
    // far field: zpsi = -i cap z / 2, gradwr = zphi + z conj(zphip) + conj(zpsi)
    double2 zpsi = make_double2(0.5 * cap * zz.y, -0.5 * cap * zz.x);
    double2 gr = cconj<double>(zpsi);
    if (iwall) {
      double2 zphi = make_double2(0.0, 0.0), zphip = zphi;
      refsing_zc(zz, k, zk, zc, zphi, zphip, zpsi);
      gr = cadd<double>(zphi, cadd<double>(cmul<double>(zz, cconj<double>(zphip)), cconj<double>(zpsi)));
    }
    g = cadd<double>(g, cadd<double>(gr, zck));
    if (gout) gout[t] = g;
    double2 zvel = make_double2(g.y, -g.x);  // -i g
    double unt = zvel.x * zn.x + zvel.y * zn.y;  // Re(zvel conj(zn))
    un[t] = unt;
    fl += hb * unt * s;
  }
  fl = block_sum_d(fl, red);
  if (threadIdx.x == 0) fluxpart[blockIdx.x] = fl;
}

__global__ void k_sum_final(int nb, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += part[i];
  *out = s;
}

int check_pow2(eb_ctx* ctx, int& nmax) {
  nmax = 0;
  for (int n : ctx->nd_host) {
    if (n < 4 || (n & (n - 1)) != 0) {
      eb_set_last_error_msg("spectral routines need power-of-two drop sizes >= 4");
      return EB_ERR_ARG;
    }
    nmax = std::max(nmax, n);
  }
  return EB_OK;
}

int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024)
    EB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return EB_OK;
}

int fdiff_dev(eb_ctx* ctx, const double2* f, double2* df) {
  int nmax;
  EB_TRY(check_pow2(ctx, nmax));
  size_t sm = sizeof(double2) * ((size_t)nmax + (size_t)nmax / 2);
  EB_TRY(set_smem((const void*)k_fdiff, sm));
  k_fdiff<<<ctx->k, SBS, sm, ctx->stream>>>(ctx->start.as<int>(), f, df, nmax);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "fdiff");
}

// PVINTEV on device: ucmplx (nbk complex) -> phicmplx (nbk complex).
int pvintev_dev(eb_ctx* ctx, const double2* uc, double2* phi, int prec) {
  int nmax;
  EB_TRY(check_pow2(ctx, nmax));
  int nbk = ctx->nbk;
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->pvz.ensure(sizeof(double2) * 2 * (size_t)nbk));
  EB_TRY(ctx->pvq.ensure(sizeof(double2) * 2 * (size_t)nbk));
  EB_TRY(ctx->pvout.ensure(sizeof(double2) * 2 * (size_t)nbk));
  size_t sm = sizeof(double2) * (size_t)nmax * 3;
  EB_TRY(set_smem((const void*)k_pv_interp, sm));
  bool need_tree = !ctx->tree_pv.valid;
  k_pv_interp<<<dim3(ctx->k, need_tree ? 3 : 1), SBS, sm, s>>>(ctx->start.as<int>(), ctx->z.as<double2>(), uc,
                                                                ctx->pvz.as<double2>(), ctx->pvq.as<double2>(), nmax);
  eb_count_launch(ctx);
  if (need_tree && ctx->nsim > 0) {
    EB_TRY(eb_batch_translate_fine(ctx, ctx->pvz.as<double2>()));
    EB_TRY(eb_tree_build(ctx, ctx->tree_pv, ctx->pvz.as<double2>(), 2 * nbk, ctx->opts.leaf64, ctx->opts.leaf_cap, ctx->b_sq,
                         ctx->b_R));
  } else if (need_tree) {
    EB_TRY(eb_tree_build(ctx, ctx->tree_pv, ctx->pvz.as<double2>(), 2 * nbk, ctx->opts.leaf64, ctx->opts.leaf_cap));
  }
  EB_TRY(eb_fmm_apply_cauchy(ctx, ctx->tree_pv, prec, ctx->pvq.as<double2>(), ctx->pvout.as<double2>()));
  k_pv_extract<<<nblk(nbk, 256), 256, 0, s>>>(nbk, ctx->pvout.as<double2>(), phi);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "pvintev");
}

}  // namespace

int eb_extractdat(eb_ctx* ctx, int k, const int* nd, const double* rku, double* zk, double* dz,
                  double* dsda, double* kappa, double* ckern, double* tha, double* area, int mem) {
  if (!ctx || k <= 0 || !nd || !rku) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int nbk = 0, nmax = 0;
  for (int b = 0; b < k; ++b) {
    if (nd[b] < 4 || (nd[b] & (nd[b] - 1)) != 0) {
      eb_set_last_error_msg("EXTRACTDAT needs power-of-two drop sizes >= 4");
      return EB_ERR_ARG;
    }
    nbk += nd[b];
    nmax = std::max(nmax, nd[b]);
  }
  cudaStream_t s = ctx->stream;
  std::vector<int> st(k + 1, 0);
  for (int b = 0; b < k; ++b) st[b + 1] = st[b] + nd[b];
  EB_TRY(ctx->start.ensure(sizeof(int) * (k + 1)));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->start.p, st.data(), sizeof(int) * (k + 1), cudaMemcpyHostToDevice, s));
  EB_TRY(ctx->fftbuf.ensure(sizeof(double2) * nbk));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->fftbuf.p, rku, sizeof(double2) * nbk,
                              mem == EB_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
  // staging buffers of the context receive the results before the install copies them
  DevBuf& zk_d = ctx->ex_zk;
  DevBuf& dz_d = ctx->ex_dz;
  DevBuf& ds_d = ctx->ex_ds;
  DevBuf& ka_d = ctx->ex_ka;
  DevBuf& area_d = ctx->ex_area;
  EB_TRY(zk_d.ensure(sizeof(double2) * k));
  EB_TRY(dz_d.ensure(sizeof(double2) * nbk));
  EB_TRY(ds_d.ensure(sizeof(double) * nbk));
  EB_TRY(ka_d.ensure(sizeof(double) * nbk));
  EB_TRY(area_d.ensure(sizeof(double) * k));
  EB_TRY(ctx->ckern.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->tha.ensure(sizeof(double) * nbk));
  size_t sm = sizeof(double2) * ((size_t)nmax * 2 + (size_t)nmax / 2);
  EB_TRY(set_smem((const void*)k_extractdat, sm));
  k_extractdat<<<k, SBS, sm, s>>>(ctx->start.as<int>(), ctx->fftbuf.as<double2>(), zk_d.as<double2>(),
                                  dz_d.as<double2>(), ds_d.as<double>(), ka_d.as<double>(),
                                  ctx->ckern.as<double2>(), ctx->tha.as<double>(), area_d.as<double>(), nmax);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "extractdat"));
  // install (the ckern / tha buffers are kept; eb_set_geometry leaves them alone)
  EB_TRY(eb_set_geometry(ctx, k, nd, ctx->fftbuf.as<double>(), dz_d.as<double>(), ds_d.as<double>(),
                         ka_d.as<double>(), zk_d.as<double>(), EB_DEVICE));
  cudaMemcpyKind ko = mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (zk) EB_CUDA_TRY(cudaMemcpyAsync(zk, zk_d.p, sizeof(double2) * k, ko, s));
  if (dz) EB_CUDA_TRY(cudaMemcpyAsync(dz, dz_d.p, sizeof(double2) * nbk, ko, s));
  if (dsda) EB_CUDA_TRY(cudaMemcpyAsync(dsda, ds_d.p, sizeof(double) * nbk, ko, s));
  if (kappa) EB_CUDA_TRY(cudaMemcpyAsync(kappa, ka_d.p, sizeof(double) * nbk, ko, s));
  if (ckern) EB_CUDA_TRY(cudaMemcpyAsync(ckern, ctx->ckern.p, sizeof(double2) * nbk, ko, s));
  if (tha) EB_CUDA_TRY(cudaMemcpyAsync(tha, ctx->tha.p, sizeof(double) * nbk, ko, s));
  if (area) EB_CUDA_TRY(cudaMemcpyAsync(area, area_d.p, sizeof(double) * k, ko, s));
  if (mem == EB_HOST) EB_CUDA_TRY(cudaStreamSynchronize(s));
  ctx->ckern_valid = true;
  return EB_OK;
}

// Per-drop starts of nd (host) on the device (in `buf`), checking the drop sizes.
static int drop_starts(eb_ctx* ctx, int k, const int* nd, DevBuf& buf, std::vector<int>& st, int& nmax,
                       int scale_flags, const int* flags) {
  st.assign(k + 1, 0);
  nmax = 0;
  for (int b = 0; b < k; ++b) {
    if (nd[b] < 4 || (nd[b] & (nd[b] - 1)) != 0) {
      eb_set_last_error_msg("spectral routines need power-of-two drop sizes >= 4");
      return EB_ERR_ARG;
    }
    st[b + 1] = st[b] + (scale_flags && flags[b] ? 2 * nd[b] : nd[b]);
    nmax = std::max(nmax, nd[b]);
  }
  EB_TRY(buf.ensure(sizeof(int) * (k + 1)));
  EB_CUDA_TRY(cudaMemcpyAsync(buf.p, st.data(), sizeof(int) * (k + 1), cudaMemcpyHostToDevice, ctx->stream));
  return EB_OK;
}

int eb_getfourier(eb_ctx* ctx, int k, const int* nd, const double* rku, int* idoub, double* fmode, int mem) {
  if (!ctx || k <= 0 || !nd || !rku || !idoub) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  std::vector<int> st;
  int nmax = 0;
  EB_TRY(drop_starts(ctx, k, nd, ctx->b_st1, st, nmax, 0, nullptr));
  const int nbk = st[k];
  const double2* zd = reinterpret_cast<const double2*>(rku);
  if (mem == EB_HOST) {
    EB_TRY(ctx->vin.ensure(sizeof(double2) * nbk));
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, rku, sizeof(double2) * nbk, cudaMemcpyHostToDevice, s));
    zd = ctx->vin.as<double2>();
  }
  EB_TRY(ctx->vout.ensure(sizeof(double) * nbk + sizeof(int) * (k + 1)));
  double* fm = ctx->vout.as<double>();
  int* fl = reinterpret_cast<int*>(fm + nbk);
  size_t sm = sizeof(double2) * ((size_t)nmax + (size_t)nmax / 2);
  EB_TRY(set_smem((const void*)k_getfourier, sm));
  k_getfourier<<<k, SBS, sm, s>>>(ctx->b_st1.as<int>(), zd, fm, fl, nmax);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "getfourier"));
  if (fmode)
    EB_CUDA_TRY(cudaMemcpyAsync(fmode, fm, sizeof(double) * nbk,
                                mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  EB_CUDA_TRY(cudaMemcpyAsync(idoub, fl, sizeof(int) * k, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

int eb_double(eb_ctx* ctx, int k, const int* nd, const double* rku, const int* idoub, double* rku2, int mem) {
  if (!ctx || k <= 0 || !nd || !rku || !idoub || !rku2) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  std::vector<int> st, st2;
  int nmax = 0;
  EB_TRY(drop_starts(ctx, k, nd, ctx->b_st1, st, nmax, 0, nullptr));
  EB_TRY(drop_starts(ctx, k, nd, ctx->b_st2, st2, nmax, 1, idoub));
  const int nbk = st[k], nbk2 = st2[k];
  EB_TRY(ctx->b_flag.ensure(sizeof(int) * k));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_flag.p, idoub, sizeof(int) * k, cudaMemcpyHostToDevice, s));
  const double2* zd = reinterpret_cast<const double2*>(rku);
  double2* z2 = reinterpret_cast<double2*>(rku2);
  if (mem == EB_HOST) {
    EB_TRY(ctx->vin.ensure(sizeof(double2) * nbk));
    EB_TRY(ctx->vout.ensure(sizeof(double2) * nbk2));
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, rku, sizeof(double2) * nbk, cudaMemcpyHostToDevice, s));
    zd = ctx->vin.as<double2>();
    z2 = ctx->vout.as<double2>();
  }
  size_t sm = sizeof(double2) * ((size_t)nmax * 2 + (size_t)nmax);
  EB_TRY(set_smem((const void*)k_double, sm));
  k_double<<<k, SBS, sm, s>>>(ctx->b_st1.as<int>(), ctx->b_st2.as<int>(), ctx->b_flag.as<int>(), zd, z2, nmax);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "double"));
  if (mem == EB_HOST)
    EB_CUDA_TRY(cudaMemcpyAsync(rku2, z2, sizeof(double2) * nbk2, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

int eb_fdiff(eb_ctx* ctx, const double* f, double* df, int mem) {
  if (!ctx || !f || !df) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int nbk = ctx->nbk;
  cudaStream_t s = ctx->stream;
  if (mem == EB_DEVICE)
    return fdiff_dev(ctx, reinterpret_cast<const double2*>(f), reinterpret_cast<double2*>(df));
  EB_TRY(ctx->vin.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->vout.ensure(sizeof(double2) * nbk));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, f, sizeof(double2) * nbk, cudaMemcpyHostToDevice, s));
  EB_TRY(fdiff_dev(ctx, ctx->vin.as<double2>(), ctx->vout.as<double2>()));
  EB_CUDA_TRY(cudaMemcpyAsync(df, ctx->vout.p, sizeof(double2) * nbk, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

int eb_pvintev(eb_ctx* ctx, const double* uc, double* phi, int prec, int mem) {
  if (!ctx || !uc || !phi) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  if (prec != EB_FP64 && prec != EB_FP32) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int nbk = ctx->nbk;
  cudaStream_t s = ctx->stream;
  if (mem == EB_DEVICE)
    return pvintev_dev(ctx, reinterpret_cast<const double2*>(uc), reinterpret_cast<double2*>(phi), prec);
  EB_TRY(ctx->vin.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->vout.ensure(sizeof(double2) * nbk));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, uc, sizeof(double2) * nbk, cudaMemcpyHostToDevice, s));
  EB_TRY(pvintev_dev(ctx, ctx->vin.as<double2>(), ctx->vout.as<double2>(), prec));
  EB_CUDA_TRY(cudaMemcpyAsync(phi, ctx->vout.p, sizeof(double2) * nbk, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

// DIRICH_NEU_MAP with any internal precision (EB_FP64, EB_FP32 or EB_PREC_DF)
static int dirich_neu_map_impl(eb_ctx* ctx, const double* u, double* phi, double* psi, double* dphi_dn,
                               int prec, int mem) {
  int nbk = ctx->nbk, nmax;
  EB_TRY(check_pow2(ctx, nmax));
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->vin.ensure(sizeof(double) * nbk));
  EB_TRY(ctx->vtmp.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->vtmp2.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->vout.ensure(sizeof(double) * 3 * nbk));
  const double* ud = u;
  if (mem == EB_HOST) {
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, u, sizeof(double) * nbk, cudaMemcpyHostToDevice, s));
    ud = ctx->vin.as<double>();
  }
  double* phd = ctx->vout.as<double>();
  double* psd = phd + nbk;
  double* dpd = psd + nbk;
  k_dtn_pre<<<nblk(nbk, 256), 256, 0, s>>>(nbk, ud, ctx->dz.as<double2>(), ctx->vtmp.as<double2>());
  eb_count_launch(ctx);
  EB_TRY(pvintev_dev(ctx, ctx->vtmp.as<double2>(), ctx->vtmp2.as<double2>(), prec));
  k_dtn_mid<<<nblk(nbk, 256), 256, 0, s>>>(nbk, ud, ctx->vtmp2.as<double2>(), ctx->z.as<double2>(), phd, psd);
  eb_count_launch(ctx);
  size_t sm = sizeof(double2) * ((size_t)nmax + (size_t)nmax / 2);
  EB_TRY(set_smem((const void*)k_fdiff_real, sm));
  k_fdiff_real<<<ctx->k, SBS, sm, s>>>(ctx->start.as<int>(), psd, ctx->vtmp.as<double2>(), nmax);
  eb_count_launch(ctx);
  k_dtn_post<<<nblk(nbk, 256), 256, 0, s>>>(nbk, ctx->vtmp.as<double2>(), ctx->dsda.as<double>(), dpd);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "dirich_neu_map"));
  cudaMemcpyKind ko = mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (phi) EB_CUDA_TRY(cudaMemcpyAsync(phi, phd, sizeof(double) * nbk, ko, s));
  if (psi) EB_CUDA_TRY(cudaMemcpyAsync(psi, psd, sizeof(double) * nbk, ko, s));
  EB_CUDA_TRY(cudaMemcpyAsync(dphi_dn, dpd, sizeof(double) * nbk, ko, s));
  if (mem == EB_HOST) EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

int eb_dirich_neu_map(eb_ctx* ctx, const double* u, double* phi, double* psi, double* dphi_dn,
                      int prec, int mem) {
  if (!ctx || !u || !dphi_dn) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  if (prec != EB_FP64 && prec != EB_FP32) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return dirich_neu_map_impl(ctx, u, phi, psi, dphi_dn, prec, mem);
}

// INTERFACENEW with any internal precision (EB_FP64, EB_FP32 or EB_PREC_DF). zc_any: 1 if
// some C_k is nonzero, 0 if all are, -1 to look (device zc: one readback). flux_async:
// FLUX goes to ctx->h_flux without a synchronisation (the caller reads it after its own).
// gout (device, optional) receives the full sum g of which Un = Re(-i g conj(zn)).
static int interface_velocity_impl(eb_ctx* ctx, const double* u, const double* zc, double cap, double* un,
                                   double* flux, int prec, int mem, int zc_any = -1,
                                   bool flux_async = false, double2* gout = nullptr) {
  int nbk = ctx->nbk, k = ctx->k;
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->vin.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->vtmp.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->vtmp2.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->vout.ensure(sizeof(double) * nbk));
  EB_TRY(ctx->redpart.ensure(sizeof(double) * 2048));
  EB_TRY(ctx->za.ensure(sizeof(double2) * k));
  const double2* ud = reinterpret_cast<const double2*>(u);
  if (mem == EB_HOST) {
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, u, sizeof(double2) * nbk, cudaMemcpyHostToDevice, s));
    ud = ctx->vin.as<double2>();
  }
  int any_zc = zc_any;
  if (mem == EB_HOST) {
    if (any_zc < 0) {
      any_zc = 0;
      for (size_t i = 0; i < 2 * (size_t)k; ++i) if (zc[i] != 0.0) any_zc = 1;
    }
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->za.p, zc, sizeof(double2) * k, cudaMemcpyHostToDevice, s));
  } else {
    if (any_zc < 0) {
      std::vector<double> zch(2 * (size_t)k);
      EB_CUDA_TRY(cudaMemcpyAsync(zch.data(), zc, sizeof(double2) * k, cudaMemcpyDeviceToHost, s));
      EB_CUDA_TRY(cudaStreamSynchronize(s));
      any_zc = 0;
      for (double v : zch) if (v != 0.0) any_zc = 1;
    }
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->za.p, zc, sizeof(double2) * k, cudaMemcpyDeviceToDevice, s));
  }
  EB_TRY(fdiff_dev(ctx, ud, ctx->vtmp.as<double2>()));
  EB_TRY(eb_stokes_sum_dev(ctx, ud, +1, ctx->vtmp2.as<double2>(), prec));
  int nbv = std::min(nblk(nbk, 256), 2048);
  double* und = mem == EB_HOST ? ctx->vout.as<double>() : un;
  k_velocity<<<nbv, 256, 0, s>>>(nbk, k, ctx->drop_of.as<int>(), ctx->z.as<double2>(), ctx->dz.as<double2>(),
                                 ctx->dsda.as<double>(), ctx->kappa.as<double>(), ctx->hpt.as<double>(),
                                 ctx->ckern.as<double2>(), ud, ctx->vtmp.as<double2>(), ctx->vtmp2.as<double2>(),
                                 ctx->za.as<double2>(), ctx->zk.as<double2>(), any_zc, ctx->iwall, cap, und,
                                 ctx->redpart.as<double>(), gout);
  eb_count_launch(ctx);
  k_sum_final<<<1, 32, 0, s>>>(nbv, ctx->redpart.as<double>(), ctx->redpart.as<double>() + 2047);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "interface velocity"));
  if (mem == EB_HOST) EB_CUDA_TRY(cudaMemcpyAsync(un, und, sizeof(double) * nbk, cudaMemcpyDeviceToHost, s));
  if (flux_async) {
    if (!ctx->h_flux) EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&ctx->h_flux), sizeof(double)));
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->h_flux, ctx->redpart.as<double>() + 2047, sizeof(double),
                                cudaMemcpyDeviceToHost, s));
    return EB_OK;
  }
  double fl = 0.0;
  EB_CUDA_TRY(cudaMemcpyAsync(&fl, ctx->redpart.as<double>() + 2047, sizeof(double), cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  if (flux) *flux = fl;
  return EB_OK;
}

int eb_interface_velocity(eb_ctx* ctx, const double* u, const double* zc, double cap, double* un,
                          double* flux, int prec, int mem) {
  if (!ctx || !u || !zc || !un) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (!ctx->ckern_valid) {
    eb_set_last_error_msg("INTERFACENEW needs ckern: install the geometry with eb_extractdat");
    return EB_ERR_NOGEOM;
  }
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  if (prec != EB_FP64 && prec != EB_FP32) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return interface_velocity_impl(ctx, u, zc, cap, un, flux, prec, mem);
}

// =================================================================================
// One RK stage F (electric.f:968-1109) and the RK2 step (electric.f:762-786), free
// space (zbond = 0), with everything resident on the GPU.
// =================================================================================
namespace {

// SETVELF (stokesbubb.f:4-135): surface tension -dz/(2|dz|) and the far field -zstr,
// zstr = -conj(psi) with psi = -i cap z/2 (:61-68); for zbond != 0 the Bond-number term
// zgrav = -(i/4)(alpha c_0 + F), F the antiderivative of zbond conj(z) dz + conj(zbond)
// z dz (:38-56), the C_k sums (:73-102) and, on a wall, minus REFSING's reflected log
// sources (:53-60); then the electric stress i E0/4 times the antiderivative of
// dz (dphi/dn)^2 (:110-128). As in the reference, the electric term uses the `alpha` left
// from the previous loops, 2 pi (nd_k - 1)/nd_k of the last drop. The wall branch of the
// reference subtracts a `zstr` it never assigns (:67); the capillary term of the
// free-space branch is taken, the term INTERFACENEW keeps on a wall (both agree for
// cap = 0). One block per drop; two FFT buffers in shared memory.
__global__ void k_setvelf(const int* __restrict__ start, const double2* __restrict__ z,
                          const double2* __restrict__ dz, const double* __restrict__ dsda,
                          const double* __restrict__ dphi, double cap, double e0,
                          double alpha_stale, const double* __restrict__ e0_drop,
                          const double* __restrict__ alpha_drop, double2 zbond, int k,
                          const double2* __restrict__ zk, const double2* __restrict__ zc, int iwall,
                          double2* __restrict__ rhs, int nmax) {
  extern __shared__ double2 sm[];
  __shared__ double2 s_c0, s_f0;
  __shared__ double s_arg0;
  int b = blockIdx.x;
  int i0 = start[b], n = start[b + 1] - i0;
  if (e0_drop) e0 = e0_drop[b];  // a batch: the drop's simulation's E0 and last-drop alpha
  if (alpha_drop) alpha_stale = alpha_drop[b];
  const bool bond = zbond.x != 0.0 || zbond.y != 0.0;
  double2* a = sm;
  double2* c = sm + nmax;                          // the C_k sums' second buffer
  double2* tw = c + (bond && zc ? nmax : 0);
  make_twiddles(tw, n);
  const double inv = 1.0 / (double)n, dal = 2.0 * EB_PI / (double)n;
  // Bond-number term (its FFT pass only for zbond != 0)
  if (bond) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double2 zz = z[i0 + i], d = dz[i0 + i];
      a[i] = cadd<double>(cmul<double>(zbond, cmul<double>(cconj<double>(zz), d)),
                          cmul<double>(cconj<double>(zbond), cmul<double>(zz, d)));
    }
    smem_fft(a, n, tw, n, -1);
    for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(a[i].x * inv, a[i].y * inv);
    __syncthreads();
    if (threadIdx.x == 0) s_c0 = a[0];
    __syncthreads();
    spectral_int(a, n);
    smem_fft(a, n, tw, n, +1);
  }
  const double2 g0 = bond ? s_c0 : make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int t = i0 + i;
    double sd = dsda[t];
    const double2 zz = z[t];
    double2 r = make_double2(-0.5 * dz[t].x / sd, -0.5 * dz[t].y / sd);
    if (bond) {  // zgrav = -(i/4)(alpha c_0 + F_i)
      const double al = dal * (double)i;
      const double2 f = make_double2(al * g0.x + a[i].x, al * g0.y + a[i].y);
      r.x += 0.25 * f.y;
      r.y -= 0.25 * f.x;
    }
    if (iwall) {  // - (zphi - z conj(zphip) - conj(zpsi)) of the reflected log sources
      double2 zphi = make_double2(0.0, 0.0), zphip = zphi, zpsi = zphi;
      refsing_zc(zz, k, zk, zc, zphi, zphip, zpsi);
      const double2 ck = csub<double>(csub<double>(zphi, cmul<double>(zz, cconj<double>(zphip))), cconj<double>(zpsi));
      r = csub<double>(r, ck);
    }
    // - zstr, zstr = -conj(-i cap z/2) = -i cap conj(z)/2
    r.x += 0.5 * cap * zz.y;
    r.y += 0.5 * cap * zz.x;
    rhs[t] = r;
  }
  // C_k: the argument of z - zk(nbod) unwrapped along the drop by integrating its
  // derivative -i (u'/u), u the unit vector, then 2 i zc arg - conj(zc) e^{2 i arg}
  if (zc && bond) {
    for (int nb = 0; nb < k; ++nb) {
      const double2 cn = zc[nb], kn = zk[nb];
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 d = csub<double>(z[i0 + i], kn);
        const double r = hypot(d.x, d.y);
        c[i] = make_double2(d.x / r, d.y / r);
        a[i] = c[i];
      }
      if (threadIdx.x == 0) {
        const double2 d0 = csub<double>(z[i0], kn);
        double g = asin(d0.y / hypot(d0.x, d0.y));
        if (d0.x < 0.0) g = EB_PI - g;
        s_arg0 = g;
      }
      smem_fft(a, n, tw, n, -1);
      spectral_deriv(a, n);
      smem_fft(a, n, tw, n, +1);
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 q = cdiv<double>(a[i], c[i]);  // -i zfi / zf
        a[i] = make_double2(q.y, -q.x);
      }
      smem_fft(a, n, tw, n, -1);
      for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(a[i].x * inv, a[i].y * inv);
      __syncthreads();
      if (threadIdx.x == 0) s_f0 = a[0];
      __syncthreads();
      const double zf1 = s_f0.x;
      spectral_int(a, n);
      smem_fft(a, n, tw, n, +1);
      const double arg0 = s_arg0, a0 = a[0].x;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double arg = arg0 + dal * (double)i * zf1 + (a[i].x - a0);
        double sn, cs;
        sincos(2.0 * arg, &sn, &cs);
        const double2 zck = csub<double>(cmul<double>(make_double2(0.0, 2.0 * arg), cn),
                                         cmul<double>(cconj<double>(cn), make_double2(cs, sn)));
        rhs[i0 + i] = csub<double>(rhs[i0 + i], zck);
      }
    }
  }
  // electric stress
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double d = dphi[i0 + i];
    a[i] = make_double2(dz[i0 + i].x * d * d, dz[i0 + i].y * d * d);
  }
  smem_fft(a, n, tw, n, -1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(a[i].x * inv, a[i].y * inv);
  __syncthreads();
  if (threadIdx.x == 0) s_c0 = a[0];
  __syncthreads();
  spectral_int(a, n);
  smem_fft(a, n, tw, n, +1);
  if (threadIdx.x == 0) s_f0 = a[0];
  __syncthreads();
  const double2 c0 = s_c0, f0 = s_f0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int t = i0 + i;
    double2 zs = make_double2(alpha_stale * c0.x + a[i].x - f0.x, alpha_stale * c0.y + a[i].y - f0.y);
    double2 r = rhs[t];
    r.x += -0.25 * e0 * zs.y;  // (i E0/4) zs
    r.y += 0.25 * e0 * zs.x;
    rhs[t] = r;
  }
}

// zc_k = i zbond area_k / (8 pi) (EXTRACTDAT, electric.f:703)
__global__ void k_zc(int k, double2 zbond, const double* __restrict__ area, double2* __restrict__ zc) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= k) return;
  const double f = area[b] / (8.0 * EB_PI);
  zc[b] = make_double2(-zbond.y * f, zbond.x * f);
}

// zc: device double2[k] of C_k (used when zbond != 0), or null
int setvelf_dev(eb_ctx* ctx, const double* dphi, double cap, double e0, double2 zbond, const double2* zc,
                double2* rhs) {
  int nmax;
  EB_TRY(check_pow2(ctx, nmax));
  const int nlast = ctx->nd_host[ctx->k - 1];
  const double alpha_stale = 2.0 * EB_PI * (double)(nlast - 1) / (double)nlast;
  const bool bond = zbond.x != 0.0 || zbond.y != 0.0;
  size_t sm = sizeof(double2) * ((bond && zc ? 2 : 1) * (size_t)nmax + (size_t)nmax / 2);
  EB_TRY(set_smem((const void*)k_setvelf, sm));
  if (ctx->iwall && !(bond && zc)) {
    eb_set_last_error_msg("SETVELF on a wall needs zbond != 0 and its zc");
    return EB_ERR_ARG;
  }
  k_setvelf<<<ctx->k, SBS, sm, ctx->stream>>>(ctx->start.as<int>(), ctx->z.as<double2>(),
                                              ctx->dz.as<double2>(), ctx->dsda.as<double>(), dphi,
                                              cap, e0, alpha_stale,
                                              ctx->nsim > 0 && ctx->sim_has_e0 ? ctx->b_e0.as<double>() : nullptr,
                                              ctx->nsim > 0 ? ctx->b_alpha.as<double>() : nullptr, zbond, ctx->k,
                                              ctx->zk.as<double2>(), bond ? zc : nullptr, ctx->iwall, rhs, nmax);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "setvelf");
}

// EQUIT (electric.f:1270-1302), then the velocity of the nodes
// (-Un i dz - T dz)/|dz|, Fourier filtered (FILTER, electric.f:1152-1187, with k/n
// formed in single precision as the reference does) and transformed back
// (electric.f:1076-1103).
__global__ void k_equit_rkup(const int* __restrict__ start, const double* __restrict__ tha,
                             const double* __restrict__ un, const double2* __restrict__ dz,
                             const double* __restrict__ dsda, double2* __restrict__ rkup, int nmax) {
  extern __shared__ double2 sm[];
  __shared__ double2 s_c0;
  int b = blockIdx.x;
  int i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* c = sm + nmax;
  double2* tw = c + nmax;
  make_twiddles(tw, n);
  const double inv = 1.0 / (double)n, dal = 2.0 * EB_PI / (double)n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(-tha[i0 + i] * un[i0 + i], 0.0);
  smem_fft(a, n, tw, n, -1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(a[i].x * inv, a[i].y * inv);
  __syncthreads();
  if (threadIdx.x == 0) {
    a[n / 2] = make_double2(0.0, 0.0);
    s_c0 = a[0];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) c[i] = a[i];
  __syncthreads();
  spectral_int(c, n);
  smem_fft(c, n, tw, n, +1);
  const double2 zf0 = s_c0;
  const double dadt = zf0.x;
  // node velocity samples (reuse a)
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    int t = i0 + i;
    double alpha = dal * (double)i;
    double T = -(zf0.x * alpha + c[i].x) + alpha * dadt;
    double u = un[t], s = dsda[t];
    double2 d = dz[t];
    a[i] = make_double2((u * d.y - T * d.x) / s, (-u * d.x - T * d.y) / s);
  }
  smem_fft(a, n, tw, n, -1);
  const int h = n / 2;
  for (int m = threadIdx.x; m < n; m += blockDim.x) {
    double2 v = make_double2(a[m].x * inv, a[m].y * inv);
    int i = (m <= h) ? m : n - m;
    double ratio = (double)__fdiv_rn((float)i, (float)h);
    double f = exp(-10.0 * powi25(ratio));
    v = make_double2(f * v.x, f * v.y);
    if (fabs(v.x) < 1e-13) v.x = 0.0;
    if (fabs(v.y) < 1e-13) v.y = 0.0;
    if (m == h) v = make_double2(0.0, 0.0);
    a[m] = v;
  }
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) rkup[i0 + i] = a[i];
}

__global__ void k_lap_bc(int nbk, const double2* __restrict__ z, double* __restrict__ rhs) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nbk) rhs[i] = -2.0 * z[i].x;  // GETBCs, laplace.f:14-18
}

__global__ void k_rk_first(int n, double dt, const double* __restrict__ y, const double* __restrict__ d,
                           double* __restrict__ phi0, double* __restrict__ y1) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double p = dt * d[i];
  phi0[i] = p;
  y1[i] = y[i] + p;
}

__global__ void k_rk_second(int n, double dt, const double* __restrict__ phi0,
                            const double* __restrict__ d, double* __restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  y[i] = y[i] + 0.5 * phi0[i] + 0.5 * (dt * d[i]);
}

// Deferred solves of a stage (ctx->defer): their control-block slots, -1 when a solve
// filled its info at once (refined mode, the host-driven loop)
struct StageSlots {
  int lap = -1, stokes = -1;
};

// gout (device, optional): INTERFACENEW's full velocity sum (interface_velocity_impl).
// Solutions (device, optional): ul_in / u_in replace the Laplace / Stokes solve by a
// solution kept from an earlier run of the same stage (the reverse pass replays a stage
// without its solves); ul_out / u_out receive this run's solutions.
int stage_f(eb_ctx* ctx, int k, const int* nd, const double* rku, double* rkup, const eb_model* m,
            eb_stage_info* info, StageSlots* slots = nullptr, double2* gout = nullptr,
            const double* ul_in = nullptr, const double* u_in = nullptr, double* ul_out = nullptr,
            double* u_out = nullptr) {
  // zbond != 0: wall-bounded (READINI's iwall, electric.f:321-326), set before the
  // install so that the tree takes the wall
  const double2 zb = make_double2(m->zbond[0], m->zbond[1]);
  const int wall = zb.x != 0.0 || zb.y != 0.0;
  if (wall && ctx->nsim > 0) {
    eb_set_last_error_msg("wall-bounded flow is not available for a batch of simulations");
    return EB_ERR_ARG;
  }
  ctx->iwall = wall;
  EB_TRY(eb_extractdat(ctx, k, nd, rku, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                       EB_DEVICE));
  int nbk = ctx->nbk, nmax;
  EB_TRY(check_pow2(ctx, nmax));
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->st_lap.ensure(sizeof(double) * 5 * (size_t)nbk));
  EB_TRY(ctx->st_rhs.ensure(sizeof(double2) * (size_t)nbk));
  EB_TRY(ctx->st_u.ensure(sizeof(double2) * (size_t)nbk));
  EB_TRY(ctx->st_zc.ensure(sizeof(double2) * (size_t)k));
  double* rl = ctx->st_lap.as<double>();
  double* ul = rl + nbk;
  double* phi = ul + nbk;
  double* psi = phi + nbk;
  double* dphi = psi + nbk;
  eb_solve_info li{}, si{};
  int s0 = ctx->ndefer;
  if (ul_in) {
    EB_CUDA_TRY(cudaMemcpyAsync(ul, ul_in, sizeof(double) * nbk, cudaMemcpyDeviceToDevice, s));
  } else {
    k_lap_bc<<<nblk(nbk, 256), 256, 0, s>>>(nbk, ctx->z.as<double2>(), rl);
    eb_count_launch(ctx);
    EB_TRY(eb_laplace_solve(ctx, nbk, rl, ul, m->mode, &li, EB_DEVICE));
    if (ul_out) EB_CUDA_TRY(cudaMemcpyAsync(ul_out, ul, sizeof(double) * nbk, cudaMemcpyDeviceToDevice, s));
  }
  const int lap_slot = ctx->ndefer > s0 ? s0 : -1;
  // the FP64 sums of the stage outside the solves: plain mode FP64 (native or
  // double-float as df64 says), refined mode the arithmetic of its FP64 residuals
  const int p64 = m->mode == EB_SOLVE_FP32_REFINED ? eb_resid_prec(ctx) : EB_FP64;
  EB_TRY(dirich_neu_map_impl(ctx, ul, phi, psi, dphi, p64, EB_DEVICE));
  if (wall) {  // zc = i zbond area / (8 pi), EXTRACTDAT (electric.f:703)
    k_zc<<<nblk(k, 128), 128, 0, s>>>(k, zb, ctx->ex_area.as<double>(), ctx->st_zc.as<double2>());
    eb_count_launch(ctx);
  } else {
    EB_CUDA_TRY(cudaMemsetAsync(ctx->st_zc.p, 0, sizeof(double2) * (size_t)k, s));
  }
  s0 = ctx->ndefer;
  if (u_in) {
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->st_u.p, u_in, sizeof(double2) * nbk, cudaMemcpyDeviceToDevice, s));
  } else {
    EB_TRY(setvelf_dev(ctx, dphi, m->cap, m->e0, zb, ctx->st_zc.as<double2>(), ctx->st_rhs.as<double2>()));
    EB_TRY(eb_stokes_solve(ctx, 2 * nbk, ctx->st_rhs.as<double>(), ctx->st_u.as<double>(), m->mode, &si,
                           EB_DEVICE));
    if (u_out) EB_CUDA_TRY(cudaMemcpyAsync(u_out, ctx->st_u.p, sizeof(double2) * nbk, cudaMemcpyDeviceToDevice, s));
  }
  const int stokes_slot = ctx->ndefer > s0 ? s0 : -1;
  if (slots) {
    slots->lap = lap_slot;
    slots->stokes = stokes_slot;
  }
  double* un = rl;  // the Laplace right-hand side is no longer needed
  // C_k is nonzero exactly in wall mode; FLUX is read by the caller after its
  // synchronisation (the stage itself waits on the host only inside the tree builds
  // and the solves)
  EB_TRY(interface_velocity_impl(ctx, ctx->st_u.as<double>(), ctx->st_zc.as<double>(), m->cap, un, nullptr,
                                 p64, EB_DEVICE, wall ? 1 : 0, true, gout));
  size_t sm2 = sizeof(double2) * ((size_t)nmax * 2 + (size_t)nmax / 2);
  EB_TRY(set_smem((const void*)k_equit_rkup, sm2));
  k_equit_rkup<<<k, SBS, sm2, s>>>(ctx->start.as<int>(), ctx->tha.as<double>(), un, ctx->dz.as<double2>(),
                                   ctx->dsda.as<double>(), reinterpret_cast<double2*>(rkup), nmax);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "stage F"));
  if (info) {  // a deferred solve's part comes from collect_stage after the caller's wait
    if (lap_slot < 0) {
      info->lap_iters += li.iters;
      info->lap_err = li.err;
      info->lap_ierr = li.ierr;
    }
    if (stokes_slot < 0) {
      info->stokes_iters += si.iters;
      info->stokes_err = si.err;
      info->stokes_ierr = si.ierr;
    }
  }
  return EB_OK;
}

// An RK call's deferred waits (ctx->defer, for its duration): solves and direct trees
// queue their results to page-locked memory; start clears the finiteness flag, finish
// queues its copy before the call's synchronisation, and collect_stage adds a stage's
// deferred solve infos after it.
struct DeferScope {
  eb_ctx* c;
  explicit DeferScope(eb_ctx* ctx) : c(ctx) {}
  int start() {
    EB_TRY(c->d_bad.ensure(sizeof(int)));
    if (!c->h_bad) EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&c->h_bad), sizeof(int)));
    EB_CUDA_TRY(cudaMemsetAsync(c->d_bad.p, 0, sizeof(int), c->stream));
    c->defer = true;
    c->ndefer = 0;
    return EB_OK;
  }
  int finish() {
    EB_CUDA_TRY(cudaMemcpyAsync(c->h_bad, c->d_bad.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    return EB_OK;
  }
  ~DeferScope() {
    c->defer = false;
    c->ndefer = 0;
  }
};

int collect_stage(eb_ctx* ctx, const StageSlots& sl, eb_stage_info* info) {
  if (*ctx->h_bad & 1) {
    eb_set_last_error_msg("non-finite node coordinate");
    return EB_ERR_NAN;
  }
  eb_solve_info li{}, si{};
  if (sl.lap >= 0) {
    EB_TRY(eb_defer_info(ctx, sl.lap, &li));
    if (info) {
      info->lap_iters += li.iters;
      info->lap_err = li.err;
      info->lap_ierr = li.ierr;
    }
  }
  if (sl.stokes >= 0) {
    EB_TRY(eb_defer_info(ctx, sl.stokes, &si));
    if (info) {
      info->stokes_iters += si.iters;
      info->stokes_err = si.err;
      info->stokes_ierr = si.ierr;
    }
  }
  return EB_OK;
}

int check_model(const eb_model* m) {
  if (!m) return EB_ERR_ARG;
  if (!std::isfinite(m->zbond[0]) || !std::isfinite(m->zbond[1])) return EB_ERR_ARG;
  if (m->mode != EB_SOLVE_FP64 && m->mode != EB_SOLVE_FP32_REFINED) return EB_ERR_ARG;
  return EB_OK;
}

}  // namespace

int eb_stage_f_keep(eb_ctx* ctx, int k, const int* nd, const double* rku, double* rkup, const eb_model* m,
                    eb_stage_info* info, double2* gout, const double* ul_in, const double* u_in, double* ul_out,
                    double* u_out) {
  EB_TRY(check_model(m));
  return stage_f(ctx, k, nd, rku, rkup, m, info, nullptr, gout, ul_in, u_in, ul_out, u_out);
}

int eb_pv_fine(eb_ctx* ctx, const double* ul) {
  int nmax;
  EB_TRY(check_pow2(ctx, nmax));
  const int nbk = ctx->nbk;
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->vtmp.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->pvz.ensure(sizeof(double2) * 2 * (size_t)nbk));
  EB_TRY(ctx->pvq.ensure(sizeof(double2) * 2 * (size_t)nbk));
  k_dtn_pre<<<nblk(nbk, 256), 256, 0, s>>>(nbk, ul, ctx->dz.as<double2>(), ctx->vtmp.as<double2>());
  eb_count_launch(ctx);
  size_t sm = sizeof(double2) * (size_t)nmax * 3;
  EB_TRY(set_smem((const void*)k_pv_interp, sm));
  k_pv_interp<<<dim3(ctx->k, 3), SBS, sm, s>>>(ctx->start.as<int>(), ctx->z.as<double2>(), ctx->vtmp.as<double2>(),
                                                ctx->pvz.as<double2>(), ctx->pvq.as<double2>(), nmax);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "pv fine points");
}

int eb_setvelf_bond(eb_ctx* ctx, const double* dphi_dn, double cap, double e0, const double* zbond,
                    const double* zc, double* rhs, int mem) {
  if (!ctx || !dphi_dn || !rhs) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  const double2 zb = zbond ? make_double2(zbond[0], zbond[1]) : make_double2(0.0, 0.0);
  const bool bond = zb.x != 0.0 || zb.y != 0.0;
  if (bond && !zc) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int nbk = ctx->nbk, k = ctx->k;
  cudaStream_t s = ctx->stream;
  const double2* zcd = reinterpret_cast<const double2*>(zc);
  if (bond && mem == EB_HOST) {
    EB_TRY(ctx->st_zc.ensure(sizeof(double2) * (size_t)k));
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->st_zc.p, zc, sizeof(double2) * k, cudaMemcpyHostToDevice, s));
    zcd = ctx->st_zc.as<double2>();
  }
  if (mem == EB_DEVICE)
    return setvelf_dev(ctx, dphi_dn, cap, e0, zb, bond ? zcd : nullptr, reinterpret_cast<double2*>(rhs));
  EB_TRY(ctx->vin.ensure(sizeof(double) * (size_t)nbk));
  EB_TRY(ctx->vout.ensure(sizeof(double2) * (size_t)nbk));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, dphi_dn, sizeof(double) * nbk, cudaMemcpyHostToDevice, s));
  EB_TRY(setvelf_dev(ctx, ctx->vin.as<double>(), cap, e0, zb, bond ? zcd : nullptr, ctx->vout.as<double2>()));
  EB_CUDA_TRY(cudaMemcpyAsync(rhs, ctx->vout.p, sizeof(double2) * nbk, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

int eb_setvelf(eb_ctx* ctx, const double* dphi_dn, double cap, double e0, double* rhs, int mem) {
  return eb_setvelf_bond(ctx, dphi_dn, cap, e0, nullptr, nullptr, rhs, mem);
}

int eb_rk_f(eb_ctx* ctx, int k, const int* nd, const double* rku, double* rkup, const eb_model* model,
            eb_stage_info* info, int mem) {
  if (!ctx || k <= 0 || !nd || !rku || !rkup) return EB_ERR_ARG;
  EB_TRY(check_model(model));
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  cudaStream_t s = ctx->stream;
  if (info) *info = eb_stage_info{};
  DeferScope dsc(ctx);
  EB_TRY(dsc.start());
  StageSlots sl;
  if (mem == EB_DEVICE) {
    EB_TRY(stage_f(ctx, k, nd, rku, rkup, model, info, &sl));
  } else {
    EB_TRY(ctx->rk_y.ensure(sizeof(double) * 2 * (size_t)nbk));
    EB_TRY(ctx->rk_d0.ensure(sizeof(double) * 2 * (size_t)nbk));
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->rk_y.p, rku, sizeof(double) * 2 * nbk, cudaMemcpyHostToDevice, s));
    EB_TRY(stage_f(ctx, k, nd, ctx->rk_y.as<double>(), ctx->rk_d0.as<double>(), model, info, &sl));
    EB_CUDA_TRY(cudaMemcpyAsync(rkup, ctx->rk_d0.p, sizeof(double) * 2 * nbk, cudaMemcpyDeviceToHost, s));
  }
  EB_TRY(dsc.finish());
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  EB_TRY(collect_stage(ctx, sl, info));
  if (info) info->flux = *ctx->h_flux;
  return EB_OK;
}

int eb_rk2_step(eb_ctx* ctx, int k, const int* nd, double dt, double* ybar, const eb_model* model,
                eb_stage_info* info, int mem) {
  if (!ctx || k <= 0 || !nd || !ybar) return EB_ERR_ARG;
  EB_TRY(check_model(model));
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  const int neq = 2 * nbk;
  cudaStream_t s = ctx->stream;
  if (info) *info = eb_stage_info{};
  EB_TRY(ctx->rk_y.ensure(sizeof(double) * (size_t)neq));
  EB_TRY(ctx->rk_y1.ensure(sizeof(double) * (size_t)neq));
  EB_TRY(ctx->rk_d0.ensure(sizeof(double) * (size_t)neq));
  EB_TRY(ctx->rk_phi.ensure(sizeof(double) * (size_t)neq));
  double* y = ctx->rk_y.as<double>();
  EB_CUDA_TRY(cudaMemcpyAsync(y, ybar, sizeof(double) * neq,
                              mem == EB_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
  // plain-mode solves and direct-sum installs wait on the host only once, at the end
  DeferScope dsc(ctx);
  EB_TRY(dsc.start());
  StageSlots sl1, sl2;
  EB_TRY(stage_f(ctx, k, nd, y, ctx->rk_d0.as<double>(), model, info, &sl1));
  k_rk_first<<<nblk(neq, 256), 256, 0, s>>>(neq, dt, y, ctx->rk_d0.as<double>(), ctx->rk_phi.as<double>(),
                                            ctx->rk_y1.as<double>());
  eb_count_launch(ctx);
  EB_TRY(stage_f(ctx, k, nd, ctx->rk_y1.as<double>(), ctx->rk_d0.as<double>(), model, info, &sl2));
  k_rk_second<<<nblk(neq, 256), 256, 0, s>>>(neq, dt, ctx->rk_phi.as<double>(), ctx->rk_d0.as<double>(), y);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "rk2 step"));
  EB_CUDA_TRY(cudaMemcpyAsync(ybar, y, sizeof(double) * neq,
                              mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  EB_TRY(dsc.finish());
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  EB_TRY(collect_stage(ctx, sl1, info));
  EB_TRY(collect_stage(ctx, sl2, info));
  if (info) info->flux = *ctx->h_flux;  // the second stage's
  return EB_OK;
}
