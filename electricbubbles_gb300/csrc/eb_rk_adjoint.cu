// Reverse mode through the RK stage F (electric.f:968-1109, free space) and the RK2
// step (electric.f:762-786): hand-written adjoint kernels; the reference has no adjoint.
//
// F is differentiated as the map with exact solves. Notation: for a real scalar J and a
// complex quantity w, wbar = dJ/dRe(w) + i dJ/dIm(w). A complex-linear map w = c z has
// zbar = conj(c) wbar, w = c conj(z) has zbar = c conj(wbar), and a real r = Re(c z) has
// zbar = conj(c) rbar. The spectral derivative D (FDIFFF) and the Fourier antiderivative
// I (FOURINT between DCFFTF/n and DCFFTB) are skew-adjoint (D^H = -D, I^H = -I), and the
// transpose of DCFFTB is DCFFTF.
//
// The reverse pass, from vbar = dJ/dF:
//   k_aj_rkup       FILTER (its 1e-13 zeroing passed through), the node velocity
//                   -(Un i dz + T dz)/|dz| and EQUIT -> dz, |dz|, tha, Un
//   k_aj_vel_local  INTERFACENEW's pointwise terms and the transpose of udot = D u
//   k_aj_stokes_*   the Stokes sums' derivatives with respect to targets, sources and
//                   charges (direct O(N^2), a block per target or per source; the
//                   target side of both sums in one pass after the transposed solve;
//                   the _df forms, in double-float on the FP32 pipes, unless
//                   eb_opts.adj_df = -1)
//   (solve)         lambda = A_S^-T ubar: eb_stokes_solve_adjoint
//   k_aj_op_local   FASMVP's drop sums (pk, za) and self terms at the density u, with
//                   cotangent -lambda; the Stokes sums follow with the same cotangent
//   k_aj_setvelf    SETVELF (zbond = 0): surface tension, the cap term, the electric
//                   stress's antiderivative, and dJ/dE0, dJ/dcap
//   k_aj_dtn        dphi/dn = -Re(D psi)/|dz| and psi = -Re(PV)/(2 pi) - Im z
//   k_aj_cauchy_*   the Cauchy sums of PVINTEV (fine sources) and of FASMVP_LAP
//   k_aj_pv_fine    the transposes of FINTERC / FINTER onto ul dz and z
//   (solve)         lambda_L = A_L^-T ulbar: eb_laplace_solve_adjoint
//   k_aj_lap_local  FASMVP_LAP's diagonal terms and GETBCs' -2 Re z
//   k_aj_extract    EXTRACTDAT: z' = D z, z'' = D z', |z'|, kappa, tha, ckern, zk -> ybar
//
// The forward values come from one rerun of the stage (eb_stage_f_keep): the geometry in
// the context, the Laplace density, psi and dphi/dn in st_lap, the Stokes density in
// st_u, INTERFACENEW's full sum g; PVINTEV's fine points from eb_pv_fine.
// eb_rk2_step_vjp transposes one RK2 step from its start state, eb_rk2_gradient runs the
// forward steps, keeps each step's start state on the device and walks them back.
#include <algorithm>
#include <cmath>
#include <vector>

#include "eb_df.cuh"
#include "eb_fft.cuh"
#include "eb_internal.h"

namespace {

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }
constexpr int SBS = 512;  // per-drop blocks
constexpr int PBS = 128;  // pair blocks: one target or one source per block

__device__ __forceinline__ double2 cmk2(double x, double y) { return make_double2(x, y); }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return cmk2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 operator-(double2 a, double2 b) { return cmk2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 operator-(double2 a) { return cmk2(-a.x, -a.y); }
__device__ __forceinline__ double2 operator*(double2 a, double2 b) { return cmul<double>(a, b); }
__device__ __forceinline__ double2 operator*(double s, double2 a) { return cmk2(s * a.x, s * a.y); }
__device__ __forceinline__ double2& operator+=(double2& a, double2 b) {
  a.x += b.x;
  a.y += b.y;
  return a;
}
__device__ __forceinline__ double2 cj(double2 a) { return cmk2(a.x, -a.y); }
__device__ __forceinline__ double2 mul_i(double2 a) { return cmk2(-a.y, a.x); }  // i a
__device__ __forceinline__ double redot(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }  // Re(conj(a) b)

// Block sums of NV doubles (blockDim.x a multiple of 32, at most 1024); every thread
// receives the totals.
template <int NV>
__device__ void block_sums(double (&v)[NV], double* red) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = warp_sum<double>(v[q]);
    if (l == 0) red[q * 32 + w] = x;
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double x = l < nw ? red[q * 32 + l] : 0.0;
      x = warp_sum<double>(x);
      if (l == 0) red[q * 32] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = red[q * 32];
  __syncthreads();
}

// FILTER's factor exp(-10 (k/n)^25) of mode m (k/n in single precision, as k_equit_rkup).
__device__ __forceinline__ double filter_factor(int m, int n) {
  const int h = n / 2;
  const int i = (m <= h) ? m : n - m;
  const double ratio = (double)__fdiv_rn((float)i, (float)h);
  return exp(-10.0 * powi25(ratio));
}

// ---------------------------------------------------------------------------------
// Node velocity, FILTER and EQUIT. FILTER's zeroing of coefficient parts below 1e-13 is
// passed through as the identity (only the exp(-10 (k/n)^25) factor and the zeroed
// Nyquist mode act on the cotangent): the zeroing moves F by at most 1e-13 per
// coefficient, and differences of F at any step above about 1e-7 see the coefficients it
// zeroes at y move linearly. T is recomputed as k_equit_rkup forms it. Writes dzb, sb,
// thb, unb.
// ---------------------------------------------------------------------------------
__global__ void k_aj_rkup(const int* __restrict__ start, const double* __restrict__ tha,
                          const double* __restrict__ un, const double2* __restrict__ dz,
                          const double* __restrict__ dsda, const double2* __restrict__ v,
                          double2* __restrict__ dzb, double* __restrict__ sb, double* __restrict__ thb,
                          double* __restrict__ unb, int nmax) {
  extern __shared__ double2 sm[];
  __shared__ double2 s_c0;
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* c = sm + nmax;
  double2* tw = c + nmax;
  make_twiddles(tw, n);
  const double inv = 1.0 / (double)n, dal = 2.0 * EB_PI / (double)n;
  // EQUIT: T = -Re(I(-tha Un))
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = cmk2(-tha[i0 + i] * un[i0 + i], 0.0);
  smem_fft(a, n, tw, n, -1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = inv * a[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    a[n / 2] = cmk2(0.0, 0.0);
    s_c0 = a[0];
  }
  __syncthreads();
  spectral_int(a, n);
  smem_fft(a, n, tw, n, +1);
  const double2 zf0 = s_c0;
  // vbar -> the spectrum's cotangent (DCFFTB^T = DCFFTF), filtered, then zfbar
  for (int i = threadIdx.x; i < n; i += blockDim.x) c[i] = v[i0 + i];
  smem_fft(c, n, tw, n, -1);
  for (int m = threadIdx.x; m < n; m += blockDim.x)
    c[m] = m == n / 2 ? cmk2(0.0, 0.0) : (filter_factor(m, n) * inv) * c[m];
  smem_fft(c, n, tw, n, +1);
  // zf = -dz W / s, W = T + i Un
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double alpha = dal * (double)i;
    const double T = -(zf0.x * alpha + a[i].x) + alpha * zf0.x;
    const double s = dsda[t];
    const double2 d = dz[t], W = cmk2(T, un[t]), zfb = c[i];
    const double2 Wb = cj((-1.0 / s) * d) * zfb;
    dzb[t] = cj((-1.0 / s) * W) * zfb;
    sb[t] = redot((1.0 / (s * s)) * (d * W), zfb);
    unb[t] = Wb.y;
    a[i] = cmk2(Wb.x, 0.0);  // Tbar
  }
  // T = -Re(I(a)), a = -tha Un: abar = Re(I(Tbar))
  smem_fft(a, n, tw, n, -1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = inv * a[i];
  spectral_int(a, n);
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double ab = a[i].x;
    thb[t] = -un[t] * ab;
    unb[t] += -tha[t] * ab;
  }
}

// ---------------------------------------------------------------------------------
// INTERFACENEW's pointwise terms: Un = Re(g conj(dz))/s, g = G_+(u) + zself + zcorr +
// i cap conj(z)/2 with zself = -conj(u) h kappa dz^2/(2 pi s), zcorr = (h Re(ckern) u -
// 2 h udot)/(2 pi i), udot = D u. Writes gwb, uB, kb, ckb, zb; adds to dzb, sb; the
// drop's dJ/dcap part goes to part[4 b + 1].
// ---------------------------------------------------------------------------------
__global__ void k_aj_vel_local(const int* __restrict__ start, const double2* __restrict__ z,
                               const double2* __restrict__ dz, const double* __restrict__ dsda,
                               const double* __restrict__ kappa, const double* __restrict__ hpt,
                               const double2* __restrict__ ckern, const double2* __restrict__ u,
                               const double* __restrict__ un, const double2* __restrict__ g,
                               const double* __restrict__ unb, double cap, double2* __restrict__ gwb,
                               double2* __restrict__ uB, double* __restrict__ kb, double* __restrict__ ckb,
                               double2* __restrict__ zb, double2* __restrict__ dzb, double* __restrict__ sb,
                               double* __restrict__ part, int nmax) {
  extern __shared__ double2 sm[];
  __shared__ double red[32];
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* tw = sm + nmax;
  make_twiddles(tw, n);
  double capp = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double s = dsda[t], kp = kappa[t], h = hpt[t], ub = unb[t];
    const double2 d = dz[t], uu = u[t], zz = z[t];
    const double2 gb = (ub / s) * d;
    gwb[t] = gb;
    double2 dzacc = (ub / s) * g[t];
    double sacc = -un[t] * ub / s;
    const double2 d2 = d * d;
    const double2 cv = (-h * kp / (2.0 * EB_PI * s)) * d2;
    double2 ubar = cv * cj(gb);
    const double2 cvb = uu * gb;
    kb[t] = redot((-h / (2.0 * EB_PI * s)) * d2, cvb);
    dzacc += cj((-h * kp / (EB_PI * s)) * d) * cvb;
    sacc += redot((h * kp / (2.0 * EB_PI * s * s)) * d2, cvb);
    ubar += (h * ckern[t].x / (2.0 * EB_PI)) * mul_i(gb);
    ckb[t] = redot(mul_i((-h / (2.0 * EB_PI)) * uu), gb);
    a[i] = (-h / EB_PI) * mul_i(gb);  // udot bar
    zb[t] = (0.5 * cap) * mul_i(cj(gb));
    capp += redot(mul_i(0.5 * cj(zz)), gb);
    dzb[t] += dzacc;
    sb[t] += sacc;
    uB[t] = ubar;
  }
  // u += D^T udotbar = -D udotbar
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    uB[t] = uB[t] - a[i];
  }
  capp = block_sum_d(capp, red);
  if (threadIdx.x == 0) part[4 * b + 1] = capp;
}

// Stokes charges qa = c0 dens dz, qb = c0 (-conj(dens) dz + dens conj(dz)), c0 = h/(2 pi i).
__global__ void k_aj_charges(int nbk, const double2* __restrict__ dens, const double2* __restrict__ dz,
                             const double* __restrict__ hpt, double2* __restrict__ qa, double2* __restrict__ qb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbk) return;
  const double2 c0 = cmk2(0.0, -hpt[t] / (2.0 * EB_PI));
  const double2 u = dens[t], d = dz[t];
  qa[t] = c0 * (u * d);
  qb[t] = c0 * (u * cj(d) - cj(u) * d);
}

// Target side of the derivatives of the two Stokes sums of the adjoint at the density u,
// gradw_t = sum_{j != t} qa_j/D + s conj(qb_j/D) - s D conj(qa_j/D^2), D = z_j - z_t, with
// s = +1 (INTERFACENEW, cotangent G1) and s = -1 (FASMVP, cotangent -G2 = -lambda): the
// sums Ta = sum conj(qa/D^2), Tb = sum qa/D^2, Tc = sum conj(qa) D conj(1/D)^3 and
// Td = sum conj(qb/D^2) do not depend on s or the cotangent, so one pass serves both:
// zb_t -= G (-Ta - s Tb) + conj(G) (2 s Tc - s Td) for each (s, G).
__global__ void __launch_bounds__(PBS) k_aj_stokes_tgt(int nbk, const double2* __restrict__ z,
                                                       const double2* __restrict__ qa,
                                                       const double2* __restrict__ qb,
                                                       const double2* __restrict__ G1,
                                                       const double2* __restrict__ G2,
                                                       double2* __restrict__ zb) {
  __shared__ double red[8 * 32];
  const int t = blockIdx.x;
  const double2 zt = z[t];
  double2 Ta = cmk2(0, 0), Tb = Ta, Tc = Ta, Td = Ta;
  for (int j = threadIdx.x; j < nbk; j += blockDim.x) {
    if (j == t) continue;
    const double2 D = z[j] - zt;
    const double2 iv = cinv<double>(D), iv2 = iv * iv;
    const double2 p = qa[j] * iv2;
    Tb += p;
    Ta += cj(p);
    Td += cj(qb[j] * iv2);
    Tc += (cj(qa[j]) * D) * cj(iv2 * iv);
  }
  double v[8] = {Ta.x, Ta.y, Tb.x, Tb.y, Tc.x, Tc.y, Td.x, Td.y};
  block_sums<8>(v, red);
  if (threadIdx.x == 0) {
    Ta = cmk2(v[0], v[1]);
    Tb = cmk2(v[2], v[3]);
    Tc = cmk2(v[4], v[5]);
    Td = cmk2(v[6], v[7]);
    const double2 g1 = G1[t], g2 = -G2[t];
    const double2 r1 = g1 * (-Ta - Tb) + cj(g1) * (2.0 * Tc - Td);
    const double2 r2 = g2 * (Tb - Ta) + cj(g2) * (Td - 2.0 * Tc);
    zb[t] = zb[t] - r1 - r2;
  }
}

// Source side: for each source j, with D = z_j - z_t over the targets t != j,
// Sa = sum G conj(1/D^2), Sb = sum G/D^2, Sc = sum D conj(G) conj(1/D)^3,
// Sq1 = sum G conj(1/D), Sq2 = sum D conj(G) conj(1/D^2), Sd = sum G/D:
// zb_j += -conj(qa) Sa - s qa Sb + 2 s conj(qa) Sc - s conj(qb) conj(Sb);
// qabar = Sq1 - s Sq2, qbbar = s conj(Sd), and through the charges dzb_j (and the
// density's cotangent uB_j when DENS).
template <int SIG, bool DENS>
__global__ void __launch_bounds__(PBS) k_aj_stokes_src(int nbk, const double2* __restrict__ z,
                                                       const double2* __restrict__ dz,
                                                       const double* __restrict__ hpt,
                                                       const double2* __restrict__ dens,
                                                       const double2* __restrict__ qa,
                                                       const double2* __restrict__ qb,
                                                       const double2* __restrict__ G, double gs,
                                                       double2* __restrict__ zb, double2* __restrict__ dzb,
                                                       double2* __restrict__ uB) {
  __shared__ double red[12 * 32];
  const int j = blockIdx.x;
  const double2 zj = z[j];
  double2 Sa = cmk2(0, 0), Sb = Sa, Sc = Sa, Sq1 = Sa, Sq2 = Sa, Sd = Sa;
  for (int t = threadIdx.x; t < nbk; t += blockDim.x) {
    if (t == j) continue;
    const double2 D = zj - z[t];
    const double2 iv = cinv<double>(D), iv2 = iv * iv;
    const double2 g = G[t], gc = cj(g);
    const double2 ci2 = cj(iv2);
    Sa += g * ci2;
    Sb += g * iv2;
    const double2 Dg = D * gc;
    Sc += Dg * cj(iv2 * iv);
    Sq1 += g * cj(iv);
    Sq2 += Dg * ci2;
    Sd += g * iv;
  }
  double v[12] = {Sa.x, Sa.y, Sb.x, Sb.y, Sc.x, Sc.y, Sq1.x, Sq1.y, Sq2.x, Sq2.y, Sd.x, Sd.y};
  block_sums<12>(v, red);
  if (threadIdx.x == 0) {
    const double s = (double)SIG;
    Sa = gs * cmk2(v[0], v[1]);
    Sb = gs * cmk2(v[2], v[3]);
    Sc = gs * cmk2(v[4], v[5]);
    Sq1 = gs * cmk2(v[6], v[7]);
    Sq2 = gs * cmk2(v[8], v[9]);
    Sd = gs * cmk2(v[10], v[11]);
    const double2 a = qa[j], bq = qb[j];
    zb[j] = zb[j] + (-(cj(a) * Sa) - s * (a * Sb) + (2.0 * s) * (cj(a) * Sc) - s * (cj(bq) * cj(Sb)));
    const double2 qab = Sq1 - s * Sq2, qbb = s * cj(Sd);
    const double2 c0 = cmk2(0.0, -hpt[j] / (2.0 * EB_PI));
    const double2 u = dens[j], d = dz[j];
    dzb[j] = dzb[j] + (cj(c0 * u) * qab - (cj(c0) * u) * qbb + (c0 * u) * cj(qbb));
    if (DENS) uB[j] = uB[j] + (cj(c0 * d) * qab + (cj(c0) * d) * qbb - (c0 * d) * cj(qbb));
  }
}

// FASMVP's drop sums and self terms at the density u, with the cotangent Gs = -lambda of
// its output: the pressure term (i/2) pk_b z, pk_b = sum (2h/pi) Re(u dz/(z - zk_b)^2) (pinf
// cancels), and zself = u h s kappa/(2 pi) + conj(u) h kappa dz^2/(2 pi s). Adds to zb,
// dzb, sb, kb; writes zkb[b].
__global__ void k_aj_op_local(const int* __restrict__ start, const double2* __restrict__ z,
                              const double2* __restrict__ dz, const double* __restrict__ dsda,
                              const double* __restrict__ kappa, const double* __restrict__ hpt,
                              const double2* __restrict__ zk, const double2* __restrict__ u,
                              const double2* __restrict__ lam, double2* __restrict__ zb,
                              double2* __restrict__ dzb, double* __restrict__ sb, double* __restrict__ kb,
                              double2* __restrict__ zkb) {
  __shared__ double red[2 * 32];
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0;
  const double2 c = zk[b];
  double v[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double2 Dl = z[t] - c;
    const double2 e = (u[t] * dz[t]) * cinv<double>(Dl * Dl);
    v[0] += (2.0 * hpt[t] / EB_PI) * e.x;
    v[1] += redot(0.5 * mul_i(z[t]), -lam[t]);
  }
  block_sums<2>(v, red);
  const double pk = v[0], pkb = v[1];
  double w[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double h = hpt[t], s = dsda[t], kp = kappa[t];
    const double2 Gs = -lam[t], uu = u[t], d = dz[t];
    const double2 Dl = z[t] - c;
    const double2 iD = cinv<double>(Dl), iD2 = iD * iD, iD3 = iD2 * iD;
    const double eb = (2.0 * h / EB_PI) * pkb;
    const double2 t3 = cj(2.0 * ((uu * d) * iD3));
    zb[t] = zb[t] + ((-0.5 * pk) * mul_i(Gs) - eb * t3);
    dzb[t] = dzb[t] + (eb * cj(uu * iD2) + cj((h * kp / (EB_PI * s)) * (cj(uu) * d)) * Gs);
    const double2 d2 = d * d;
    sb[t] += redot((h * kp / (2.0 * EB_PI)) * uu, Gs) + redot((-h * kp / (2.0 * EB_PI * s * s)) * (cj(uu) * d2), Gs);
    kb[t] += redot((h * s / (2.0 * EB_PI)) * uu, Gs) + redot((h / (2.0 * EB_PI * s)) * (cj(uu) * d2), Gs);
    const double2 zkp = eb * t3;
    w[0] += zkp.x;
    w[1] += zkp.y;
  }
  block_sums<2>(w, red);
  if (threadIdx.x == 0) zkb[b] = cmk2(w[0], w[1]);
}

// SETVELF (zbond = 0): rhs = -dz/(2 s) + i cap conj(z)/2 + (i E0/4)(alpha_c c0 + G_i - G_0),
// G = I(dz dphi^2), c0 its mean, with the cotangent lambda of rhs. Adds to dzb, sb, zb;
// writes dphib; the drop's dJ/dE0 and dJ/dcap parts go to part[4 b], part[4 b + 2].
__global__ void k_aj_setvelf(const int* __restrict__ start, const double2* __restrict__ z,
                             const double2* __restrict__ dz, const double* __restrict__ dsda,
                             const double* __restrict__ dphi, const double2* __restrict__ lam, double e0,
                             double cap, double alpha_c, double2* __restrict__ dzb, double* __restrict__ sb,
                             double2* __restrict__ zb, double* __restrict__ dphib, double* __restrict__ part,
                             int nmax) {
  extern __shared__ double2 sm[];
  __shared__ double red[3 * 32];
  __shared__ double2 s_c0, s_g0;
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* tw = sm + nmax;
  make_twiddles(tw, n);
  const double inv = 1.0 / (double)n;
  double capp = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double s = dsda[t], ph = dphi[t];
    const double2 l = lam[t], d = dz[t];
    dzb[t] = dzb[t] + (-0.5 / s) * l;
    sb[t] += redot((0.5 / (s * s)) * d, l);
    zb[t] = zb[t] + (0.5 * cap) * mul_i(cj(l));
    capp += redot(0.5 * mul_i(cj(z[t])), l);
    a[i] = (ph * ph) * d;
  }
  // forward electric term for dJ/dE0
  smem_fft(a, n, tw, n, -1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = inv * a[i];
  __syncthreads();
  if (threadIdx.x == 0) s_c0 = a[0];
  __syncthreads();
  spectral_int(a, n);
  smem_fft(a, n, tw, n, +1);
  if (threadIdx.x == 0) s_g0 = a[0];
  __syncthreads();
  double v[3] = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double2 zs = 0.25 * mul_i(alpha_c * s_c0 + a[i] - s_g0);
    v[0] += redot(zs, lam[t]);
    const double2 xb = (-0.25 * e0) * mul_i(lam[t]);
    v[1] += xb.x;
    v[2] += xb.y;
  }
  block_sums<3>(v, red);
  const double2 sx = cmk2(v[1], v[2]);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 xb = (-0.25 * e0) * mul_i(lam[i0 + i]);
    if (i == 0) xb = xb - sx;
    a[i] = xb;
  }
  smem_fft(a, n, tw, n, -1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = inv * a[i];
  spectral_int(a, n);
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double2 gb = (alpha_c * inv) * sx - a[i];
    const double ph = dphi[t];
    const double2 d = dz[t];
    dzb[t] = dzb[t] + (ph * ph) * gb;
    dphib[t] = redot((2.0 * ph) * d, gb);
  }
  capp = block_sum_d(capp, red);
  if (threadIdx.x == 0) {
    part[4 * b] = v[0];
    part[4 * b + 2] = capp;
  }
}

// DIRICH_NEU_MAP's tail: dphi = -Re(D psi)/s, psi = -Re(PV)/(2 pi) - Im z. Writes psib
// (the PV sum's cotangent is -psib/(2 pi)); adds to sb and zb.
__global__ void k_aj_dtn(const int* __restrict__ start, const double* __restrict__ dsda,
                         const double* __restrict__ dphi, const double* __restrict__ dphib,
                         double* __restrict__ sb, double2* __restrict__ zb, double* __restrict__ psib, int nmax) {
  extern __shared__ double2 sm[];
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* tw = sm + nmax;
  make_twiddles(tw, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double s = dsda[t], db = dphib[t];
    sb[t] += -dphi[t] * db / s;
    a[i] = cmk2(-db / s, 0.0);
  }
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double pb = -a[i].x;
    psib[t] = pb;
    zb[t].y -= pb;
  }
}

// Target side of a Cauchy sum cf_t = sum_j q_j/(zt_t - zs_j) (j != t when SELF), with the
// cotangent coef * x_t: the target's cotangent conj(-sum q_j/(zt_t - zs_j)^2) coef x_t is
// added to zb_t (ADD) or written there. Targets, sources and charges at strides ts, ss, qs.
template <bool SELF, bool ADD>
__global__ void __launch_bounds__(PBS) k_aj_cauchy_tgt(int nt, const double2* __restrict__ zt, int ts, int ns,
                                                       const double2* __restrict__ zs, int ss,
                                                       const double2* __restrict__ q, int qs,
                                                       const double* __restrict__ x, double2 coef,
                                                       double2* __restrict__ zb) {
  __shared__ double red[2 * 32];
  const int t = blockIdx.x;
  const double2 z = zt[(size_t)t * ts];
  double2 A = cmk2(0, 0);
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    if (SELF && j == t) continue;
    const double2 iv = cinv<double>(z - zs[(size_t)j * ss]);
    A += q[(size_t)j * qs] * (iv * iv);
  }
  double v[2] = {A.x, A.y};
  block_sums<2>(v, red);
  if (threadIdx.x == 0) {
    const double2 r = cj(-cmk2(v[0], v[1])) * (x[t] * coef);
    zb[t] = ADD ? zb[t] + r : r;
  }
}

// Source side: qbar_j = sum_t conj(1/(zt_t - zs_j)) cb_t and zsbar_j = conj(q_j) sum_t
// conj(1/(zt_t - zs_j)^2) cb_t, cb_t = coef x_t. LAP (the Laplace operator, SELF): zb_j +=
// zsbar, dzb_j += ul_j h_j qbar (q = ul dz h). Otherwise (PVINTEV): qsb_j = qbar,
// zsb_j = zsbar.
template <bool SELF, bool LAP>
__global__ void __launch_bounds__(PBS) k_aj_cauchy_src(int nt, const double2* __restrict__ zt, int ts, int ns,
                                                       const double2* __restrict__ zs, int ss,
                                                       const double2* __restrict__ q, int qs,
                                                       const double* __restrict__ x, double2 coef,
                                                       const double* __restrict__ ul,
                                                       const double* __restrict__ hpt,
                                                       double2* __restrict__ zb, double2* __restrict__ dzb,
                                                       double2* __restrict__ qsb, double2* __restrict__ zsb) {
  __shared__ double red[4 * 32];
  const int j = blockIdx.x;
  const double2 zj = zs[(size_t)j * ss];
  double2 S1 = cmk2(0, 0), S2 = S1;
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    if (SELF && t == j) continue;
    const double2 iv = cj(cinv<double>(zt[(size_t)t * ts] - zj));
    const double xt = x[t];
    S1 += xt * iv;
    S2 += xt * (iv * iv);
  }
  double v[4] = {S1.x, S1.y, S2.x, S2.y};
  block_sums<4>(v, red);
  if (threadIdx.x == 0) {
    const double2 qb = cmk2(v[0], v[1]) * coef;
    const double2 zsbar = cj(q[(size_t)j * qs]) * (cmk2(v[2], v[3]) * coef);
    if (LAP) {
      zb[j] = zb[j] + zsbar;
      dzb[j] = dzb[j] + (ul[j] * hpt[j]) * qb;
    } else {
      qsb[j] = qb;
      zsb[j] = zsbar;
    }
  }
}

// Transposes of PVINTEV's interpolation (one block per drop and component): comp 0,
// FINTERC of uc = ul dz with the charges h u2 on the odd fine nodes: ulb = Re(conj(dz)
// ucb) (written), dzb += ul ucb; comps 1 and 2, FINTER of x and y onto the fine nodes,
// the sources (odd, cotangent zsb) and the evaluation points (even, cotangent ztb):
// zb.x, zb.y += FINTER^T.
__global__ void k_aj_pv_fine(const int* __restrict__ start, const double2* __restrict__ dz,
                             const double* __restrict__ ul, const double* __restrict__ hpt,
                             const double2* __restrict__ qsb, const double2* __restrict__ zsb,
                             const double2* __restrict__ ztb, double* __restrict__ ulb, double2* __restrict__ dzb, double2* __restrict__ zb,
                             int nmax) {
  extern __shared__ double2 sm[];
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0, nf = 2 * n, ny = n / 2;
  const int comp = blockIdx.y;
  double2* w = sm;
  double2* tw = sm + 2 * nmax;
  make_twiddles(tw, nf);
  const double inv = 1.0 / (double)n;
  for (int m = threadIdx.x; m < nf; m += blockDim.x) {
    const int t = i0 + (m >> 1);
    double2 val = cmk2(0.0, 0.0);
    if (comp == 0) {
      if (m & 1) val = hpt[t] * qsb[t];
    } else {
      const double2 c = (m & 1) ? zsb[t] : ztb[t];
      val = cmk2(comp == 1 ? c.x : c.y, 0.0);
    }
    w[m] = val;
  }
  smem_fft(w, nf, tw, nf, -1);
  // keep modes 0..n/2 and the negative modes n/2+1..n-1 (at n + m of the fine spectrum)
  for (int m = ny + 1 + threadIdx.x; m < n; m += blockDim.x) w[m] = w[n + m];
  __syncthreads();
  for (int m = threadIdx.x; m < n; m += blockDim.x) {
    double2 c = inv * w[m];
    if (comp == 0) {
      if (m == ny) c = cmk2(0.0, 0.0);
    } else {
      if (m == ny - 1) c.y = 0.0;
      if (m == ny) c.x = 0.0;
    }
    w[m] = c;
  }
  smem_fft(w, n, tw, nf, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    if (comp == 0) {
      const double2 ucb = w[i];
      ulb[t] = redot(dz[t], ucb);
      dzb[t] = dzb[t] + ul[t] * ucb;
    } else {
      // the x and y blocks of a drop write separate halves of zb[t]
      reinterpret_cast<double*>(zb)[2 * (size_t)t + (comp - 1)] += w[i].x;
    }
  }
}

// FASMVP_LAP's diagonal and GETBCs (rhs = -2 Re z) with lambda_L: wb = -lambda_L;
// kb += h s ul wb/(2 pi), sb += (h kappa ul/(2 pi) - 2 h ul) wb, zb.x -= 2 lambda_L; and the
// Cauchy charges q = ul dz h.
__global__ void k_aj_lap_local(int nbk, const double2* __restrict__ dz, const double* __restrict__ dsda,
                               const double* __restrict__ kappa, const double* __restrict__ hpt,
                               const double* __restrict__ ul, const double* __restrict__ laml,
                               double2* __restrict__ zb, double* __restrict__ kb, double* __restrict__ sb,
                               double2* __restrict__ ql) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbk) return;
  const double l = laml[t], h = hpt[t], u = ul[t];
  const double wb = -l;
  zb[t].x -= 2.0 * l;
  kb[t] += h * dsda[t] * u * wb / (2.0 * EB_PI);
  sb[t] += (h * kappa[t] * u / (2.0 * EB_PI) - 2.0 * h * u) * wb;
  ql[t] = (u * h) * dz[t];
}

// EXTRACTDAT's transpose: z' = D z, z'' = D z', s = |z'|, m = Im(conj(z') z''), kappa =
// -m/s^3, tha = m/s^2, ckern = -z''/z' (Re part used), dz = -z', zk = mean(z); writes
// ybar (interleaved).
__global__ void k_aj_extract(const int* __restrict__ start, const double2* __restrict__ z,
                             const double2* __restrict__ zb, const double2* __restrict__ dzb,
                             const double* __restrict__ sb, const double* __restrict__ kb,
                             const double* __restrict__ thb, const double* __restrict__ ckb,
                             const double2* __restrict__ zkb, double* __restrict__ ybar, int nmax) {
  extern __shared__ double2 sm[];
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0;
  double2* a = sm;
  double2* d1 = sm + nmax;
  double2* tw = d1 + nmax;
  make_twiddles(tw, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = z[i0 + i];
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) d1[i] = a[i];
  smem_fft(d1, n, tw, n, +1);  // z'
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = d1[i];
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  smem_fft(a, n, tw, n, +1);  // z''
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double2 za = d1[i], zai = a[i];
    const double s = sqrt(za.x * za.x + za.y * za.y);
    const double m = za.x * zai.y - za.y * zai.x;
    const double s2 = s * s, s3 = s2 * s, s4 = s2 * s2;
    const double sbt = sb[t] + 3.0 * m / s4 * kb[t] - 2.0 * m / s3 * thb[t];
    const double mb = -kb[t] / s3 + thb[t] / s2;
    const double2 iza = cinv<double>(za);
    const double ck = ckb[t];
    const double2 zab = -dzb[t] + (sbt / s) * za - mb * mul_i(zai) + ck * cj(zai * (iza * iza));
    const double2 zaib = mb * mul_i(za) - ck * cj(iza);
    d1[i] = zab;
    a[i] = zaib;
  }
  // z' bar += D^T z''bar = -D z''bar; z bar += -D z'bar
  smem_fft(a, n, tw, n, -1);
  spectral_deriv(a, n);
  smem_fft(a, n, tw, n, +1);
  for (int i = threadIdx.x; i < n; i += blockDim.x) d1[i] = d1[i] - a[i];
  smem_fft(d1, n, tw, n, -1);
  spectral_deriv(d1, n);
  smem_fft(d1, n, tw, n, +1);
  const double2 zkm = (1.0 / (double)n) * zkb[b];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int t = i0 + i;
    const double2 r = zb[t] - d1[i] + zkm;
    ybar[2 * t] = r.x;
    ybar[2 * t + 1] = r.y;
  }
}

// Taylor deformation per drop: zk = mean(z), L = max |z - zk|, B = min |z - zk| (first
// index on ties), J_b = (L - B)/(L + B) into part[b]; with ybar, its gradient.
__global__ void k_deformation(const int* __restrict__ start, const double* __restrict__ y,
                              double* __restrict__ part, double* __restrict__ ybar) {
  __shared__ double red[2 * 32];
  __shared__ double s_v[32];
  __shared__ int s_i[32];
  const int b = blockIdx.x, i0 = start[b], n = start[b + 1] - i0;
  double v[2] = {0.0, 0.0};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    v[0] += y[2 * (i0 + i)];
    v[1] += y[2 * (i0 + i) + 1];
  }
  block_sums<2>(v, red);
  const double2 c = cmk2(v[0] / n, v[1] / n);
  // argmax and argmin of the distance (value, then index)
  double best[2] = {-1.0, INFINITY};
  int bi[2] = {0x7fffffff, 0x7fffffff};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double r = hypot(y[2 * (i0 + i)] - c.x, y[2 * (i0 + i) + 1] - c.y);
    if (r > best[0] || (r == best[0] && i < bi[0])) { best[0] = r; bi[0] = i; }
    if (r < best[1] || (r == best[1] && i < bi[1])) { best[1] = r; bi[1] = i; }
  }
  int res_i[2];
  double res_v[2];
  for (int q = 0; q < 2; ++q) {
    double bv = best[q];
    int ii = bi[q];
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, ii, o);
      const bool take = q == 0 ? (ov > bv || (ov == bv && oi < ii)) : (ov < bv || (ov == bv && oi < ii));
      if (take) { bv = ov; ii = oi; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) { s_v[w] = bv; s_i[w] = ii; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k2 = 1; k2 < nw; ++k2) {
        const bool take = q == 0 ? (s_v[k2] > bv || (s_v[k2] == bv && s_i[k2] < ii))
                                 : (s_v[k2] < bv || (s_v[k2] == bv && s_i[k2] < ii));
        if (take) { bv = s_v[k2]; ii = s_i[k2]; }
      }
      s_v[0] = bv;
      s_i[0] = ii;
    }
    __syncthreads();
    res_v[q] = s_v[0];
    res_i[q] = s_i[0];
    __syncthreads();
  }
  const double L = res_v[0], B = res_v[1];
  if (threadIdx.x == 0) part[b] = (L - B) / (L + B);
  if (!ybar) return;
  const double gL = 2.0 * B / ((L + B) * (L + B)), gB = -2.0 * L / ((L + B) * (L + B));
  const int p = res_i[0], q = res_i[1];
  const double2 ep = cmk2((y[2 * (i0 + p)] - c.x) / L, (y[2 * (i0 + p) + 1] - c.y) / L);
  const double2 eq = cmk2((y[2 * (i0 + q)] - c.x) / B, (y[2 * (i0 + q) + 1] - c.y) / B);
  const double2 all = (-1.0 / n) * (gL * ep + gB * eq);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 g = all;
    if (i == p) g += gL * ep;
    if (i == q) g += gB * eq;
    ybar[2 * (i0 + i)] = g.x;
    ybar[2 * (i0 + i) + 1] = g.y;
  }
}

// ---------------------------------------------------------------------------------
// The pair sums in double-float arithmetic (eb_opts.adj_df): the same sums as the FP64
// kernels above, each pair's terms in about 48 bits on the FP32 pipes (GB300 issues some
// 60 times more FP32 than FP64 operations), positions relative to the first node (the
// nearest pairs then keep ~1e-11 relative), compensated accumulators; the sums are
// finished in FP64 as above.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ cdf c4(float4 v) { return cdf{{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ cdf cdf_sub(cdf a, cdf b) { return cdf{dfl_sub(a.x, b.x), dfl_sub(a.y, b.y)}; }
__device__ __forceinline__ cdf cdf_conj(cdf a) { return cdf{a.x, dfl_neg(a.y)}; }
__device__ __forceinline__ cdf cdf_inv(cdf a) {
  const dfl r = dfl_rcp(dfl_add(dfl_sqr(a.x), dfl_sqr(a.y)));
  return cdf{dfl_mul(a.x, r), dfl_neg(dfl_mul(a.y, r))};
}
__device__ __forceinline__ cdf cdf_scale(dfl s, cdf a) { return cdf{dfl_mul(s, a.x), dfl_mul(s, a.y)}; }
struct cacc {
  dfacc x, y;
};
__device__ __forceinline__ void cacc_add(cacc& a, cdf v) {
  acc_dfl(a.x, v.x);
  acc_dfl(a.y, v.y);
}
__device__ __forceinline__ void cacc_put(const cacc& a, double* v) {
  v[0] = (double)a.x.s + (double)a.x.c;
  v[1] = (double)a.y.s + (double)a.y.c;
}

// out_i = the double-float form of in[i stride] - *shift (shift may be null)
__global__ void k_df4(int n, const double2* __restrict__ in, int stride, const double2* __restrict__ shift,
                      float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 v = in[(size_t)i * stride];
  if (shift) {
    v.x -= shift->x;
    v.y -= shift->y;
  }
  const dfl a = dfl_from_double(v.x), b = dfl_from_double(v.y);
  out[i] = make_float4(a.hi, a.lo, b.hi, b.lo);
}

__global__ void k_df2(int n, const double* __restrict__ in, float2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const dfl a = dfl_from_double(in[i]);
  out[i] = make_float2(a.hi, a.lo);
}

// k_aj_stokes_tgt in double-float (Ta = conj(Tb) is not summed separately)
__global__ void __launch_bounds__(PBS) k_aj_stokes_tgt_df(int nbk, const float4* __restrict__ zd,
                                                          const float4* __restrict__ qad,
                                                          const float4* __restrict__ qbd,
                                                          const double2* __restrict__ G1,
                                                          const double2* __restrict__ G2,
                                                          double2* __restrict__ zb) {
  __shared__ double red[6 * 32];
  const int t = blockIdx.x;
  const cdf zt = c4(zd[t]);
  cacc Tb{}, Tc{}, Td{};
  for (int j = threadIdx.x; j < nbk; j += blockDim.x) {
    if (j == t) continue;
    const cdf D = cdf_sub(c4(zd[j]), zt);
    const cdf iv = cdf_inv(D), iv2 = cdf_mul(iv, iv);
    const cdf qa = c4(qad[j]);
    cacc_add(Tb, cdf_mul(qa, iv2));
    cacc_add(Td, cdf_conj(cdf_mul(c4(qbd[j]), iv2)));
    cacc_add(Tc, cdf_mul(cdf_mul(cdf_conj(qa), D), cdf_conj(cdf_mul(iv2, iv))));
  }
  double v[6];
  cacc_put(Tb, v);
  cacc_put(Tc, v + 2);
  cacc_put(Td, v + 4);
  block_sums<6>(v, red);
  if (threadIdx.x == 0) {
    const double2 Tbv = cmk2(v[0], v[1]), Tcv = cmk2(v[2], v[3]), Tdv = cmk2(v[4], v[5]), Tav = cj(Tbv);
    const double2 g1 = G1[t], g2 = -G2[t];
    const double2 r1 = g1 * (-Tav - Tbv) + cj(g1) * (2.0 * Tcv - Tdv);
    const double2 r2 = g2 * (Tbv - Tav) + cj(g2) * (Tdv - 2.0 * Tcv);
    zb[t] = zb[t] - r1 - r2;
  }
}

// k_aj_stokes_src in double-float; Gd = the double-float form of the cotangent, scaled
// by gs in the FP64 finish
template <int SIG, bool DENS>
__global__ void __launch_bounds__(PBS) k_aj_stokes_src_df(int nbk, const float4* __restrict__ zd,
                                                          const float4* __restrict__ Gd, double gs,
                                                          const double2* __restrict__ dz,
                                                          const double* __restrict__ hpt,
                                                          const double2* __restrict__ dens,
                                                          const double2* __restrict__ qa,
                                                          const double2* __restrict__ qb,
                                                          double2* __restrict__ zb, double2* __restrict__ dzb,
                                                          double2* __restrict__ uB) {
  __shared__ double red[12 * 32];
  const int j = blockIdx.x;
  const cdf zj = c4(zd[j]);
  cacc Sa{}, Sb{}, Sc{}, Sq1{}, Sq2{}, Sd{};
  for (int t = threadIdx.x; t < nbk; t += blockDim.x) {
    if (t == j) continue;
    const cdf D = cdf_sub(zj, c4(zd[t]));
    const cdf iv = cdf_inv(D), iv2 = cdf_mul(iv, iv);
    const cdf g = c4(Gd[t]);
    const cdf ci2 = cdf_conj(iv2);
    cacc_add(Sa, cdf_mul(g, ci2));
    cacc_add(Sb, cdf_mul(g, iv2));
    const cdf Dg = cdf_mul(D, cdf_conj(g));
    cacc_add(Sc, cdf_mul(Dg, cdf_conj(cdf_mul(iv2, iv))));
    cacc_add(Sq1, cdf_mul(g, cdf_conj(iv)));
    cacc_add(Sq2, cdf_mul(Dg, ci2));
    cacc_add(Sd, cdf_mul(g, iv));
  }
  double v[12];
  cacc_put(Sa, v);
  cacc_put(Sb, v + 2);
  cacc_put(Sc, v + 4);
  cacc_put(Sq1, v + 6);
  cacc_put(Sq2, v + 8);
  cacc_put(Sd, v + 10);
  block_sums<12>(v, red);
  if (threadIdx.x == 0) {
    const double s = (double)SIG;
    const double2 Sav = gs * cmk2(v[0], v[1]), Sbv = gs * cmk2(v[2], v[3]), Scv = gs * cmk2(v[4], v[5]);
    const double2 Sq1v = gs * cmk2(v[6], v[7]), Sq2v = gs * cmk2(v[8], v[9]), Sdv = gs * cmk2(v[10], v[11]);
    const double2 a = qa[j], bq = qb[j];
    zb[j] = zb[j] + (-(cj(a) * Sav) - s * (a * Sbv) + (2.0 * s) * (cj(a) * Scv) - s * (cj(bq) * cj(Sbv)));
    const double2 qab = Sq1v - s * Sq2v, qbb = s * cj(Sdv);
    const double2 c0 = cmk2(0.0, -hpt[j] / (2.0 * EB_PI));
    const double2 u = dens[j], d = dz[j];
    dzb[j] = dzb[j] + (cj(c0 * u) * qab - (cj(c0) * u) * qbb + (c0 * u) * cj(qbb));
    if (DENS) uB[j] = uB[j] + (cj(c0 * d) * qab + (cj(c0) * d) * qbb - (c0 * d) * cj(qbb));
  }
}

// k_aj_cauchy_tgt in double-float
template <bool SELF, bool ADD>
__global__ void __launch_bounds__(PBS) k_aj_cauchy_tgt_df(int nt, const float4* __restrict__ ztd, int ns,
                                                          const float4* __restrict__ zsd,
                                                          const float4* __restrict__ qd,
                                                          const double* __restrict__ x, double2 coef,
                                                          double2* __restrict__ zb) {
  __shared__ double red[2 * 32];
  const int t = blockIdx.x;
  const cdf z = c4(ztd[t]);
  cacc A{};
  for (int j = threadIdx.x; j < ns; j += blockDim.x) {
    if (SELF && j == t) continue;
    const cdf iv = cdf_inv(cdf_sub(z, c4(zsd[j])));
    cacc_add(A, cdf_mul(c4(qd[j]), cdf_mul(iv, iv)));
  }
  double v[2];
  cacc_put(A, v);
  block_sums<2>(v, red);
  if (threadIdx.x == 0) {
    const double2 r = cj(-cmk2(v[0], v[1])) * (x[t] * coef);
    zb[t] = ADD ? zb[t] + r : r;
  }
}

// k_aj_cauchy_src in double-float (xd: the double-float form of x)
template <bool SELF, bool LAP>
__global__ void __launch_bounds__(PBS) k_aj_cauchy_src_df(int nt, const float4* __restrict__ ztd, int ns,
                                                          const float4* __restrict__ zsd,
                                                          const float2* __restrict__ xd, double2 coef,
                                                          const double2* __restrict__ q, int qs,
                                                          const double* __restrict__ ul,
                                                          const double* __restrict__ hpt,
                                                          double2* __restrict__ zb, double2* __restrict__ dzb,
                                                          double2* __restrict__ qsb, double2* __restrict__ zsb) {
  __shared__ double red[4 * 32];
  const int j = blockIdx.x;
  const cdf zj = c4(zsd[j]);
  cacc S1{}, S2{};
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    if (SELF && t == j) continue;
    const cdf iv = cdf_conj(cdf_inv(cdf_sub(c4(ztd[t]), zj)));
    const dfl xt = dfl{xd[t].x, xd[t].y};
    cacc_add(S1, cdf_scale(xt, iv));
    cacc_add(S2, cdf_scale(xt, cdf_mul(iv, iv)));
  }
  double v[4];
  cacc_put(S1, v);
  cacc_put(S2, v + 2);
  block_sums<4>(v, red);
  if (threadIdx.x == 0) {
    const double2 qb = cmk2(v[0], v[1]) * coef;
    const double2 zsbar = cj(q[(size_t)j * qs]) * (cmk2(v[2], v[3]) * coef);
    if (LAP) {
      zb[j] = zb[j] + zsbar;
      dzb[j] = dzb[j] + (ul[j] * hpt[j]) * qb;
    } else {
      qsb[j] = qb;
      zsb[j] = zsbar;
    }
  }
}

__global__ void k_axpby(int n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                        double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a * x[i] + b * y[i];
}

// RK2 as eb_rk2_step forms it: phi0 = dt d0, y1 = y + phi0; y_next = y + phi0/2 + (dt d1)/2
__global__ void k_rk_pred(int n, double dt, const double* __restrict__ y, const double* __restrict__ d0,
                          double* __restrict__ phi0, double* __restrict__ y1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double p = dt * d0[i];
  phi0[i] = p;
  y1[i] = y[i] + p;
}

__global__ void k_rk_corr(int n, double dt, const double* __restrict__ y, const double* __restrict__ phi0,
                          const double* __restrict__ d1, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = y[i] + 0.5 * phi0[i] + 0.5 * (dt * d1[i]);
}

__global__ void k_sum3(int n, const double* __restrict__ x, const double* __restrict__ y,
                       const double* __restrict__ z, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = x[i] + y[i] + z[i];
}

int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024)
    EB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return EB_OK;
}

// Cotangent buffers of one reverse pass over nbk nodes (carved from ctx->aj).
struct AjBufs {
  double2 *zb, *dzb, *uB, *gwb, *lam, *qsb, *zsb, *ztb, *gw, *qa, *qb, *ql, *f;
  double *sb, *kb, *thb, *ckb, *unb, *dphib, *psib, *ulb, *laml;
  double2* zkb;
};

int aj_bufs(eb_ctx* ctx, int nbk, int nk, AjBufs& B) {
  const size_t n = (size_t)nbk, k = (size_t)nk;
  const size_t nd2 = 13 * n + k, nd1 = 9 * n;
  EB_TRY(ctx->aj.ensure(sizeof(double2) * nd2 + sizeof(double) * nd1));
  EB_TRY(ctx->aj_part.ensure(sizeof(double) * 4 * k));
  double2* p2 = ctx->aj.as<double2>();
  double2** c2[] = {&B.zb, &B.dzb, &B.uB, &B.gwb, &B.lam, &B.qsb, &B.zsb, &B.ztb, &B.gw, &B.qa, &B.qb, &B.ql, &B.f};
  for (double2** q : c2) {
    *q = p2;
    p2 += n;
  }
  B.zkb = p2;
  p2 += k;
  double* p1 = reinterpret_cast<double*>(p2);
  double** c1[] = {&B.sb, &B.kb, &B.thb, &B.ckb, &B.unb, &B.dphib, &B.psib, &B.ulb, &B.laml};
  for (double** q : c1) {
    *q = p1;
    p1 += n;
  }
  return EB_OK;
}

int check_adjoint_model(eb_ctx* ctx, const eb_model* m) {
  if (!m) return EB_ERR_ARG;
  if (m->zbond[0] != 0.0 || m->zbond[1] != 0.0) {
    eb_set_last_error_msg("the adjoint of F covers free space (zbond = 0)");
    return EB_ERR_ARG;
  }
  if (ctx->nsim > 0) {
    eb_set_last_error_msg("the adjoint of F covers one simulation (no batch)");
    return EB_ERR_ARG;
  }
  if (m->mode != EB_SOLVE_FP64 && m->mode != EB_SOLVE_FP32_REFINED) return EB_ERR_ARG;
  return EB_OK;
}

void note_ierr(eb_adjoint_info* info, int ierr) {
  if (info && info->ierr == 0 && ierr != 0) info->ierr = ierr;
}

// v^T dF at y (device arrays, 2 nbk each) into yb_out (device); param_bar (host, 2) += the
// E0 and cap parts.
// ul_in / u_in (device, optional): the stage's solutions kept from its forward run, which
// the stage's rerun then replays instead of solving
int f_vjp_dev(eb_ctx* ctx, int k, const int* nd, const double* y, const double* v, const eb_model* m,
              double* yb_out, double* param_bar, eb_adjoint_info* info, const double* ul_in = nullptr,
              const double* u_in = nullptr) {
  cudaStream_t s = ctx->stream;
  int nbk = 0, nmax = 0;
  for (int b = 0; b < k; ++b) {
    nbk += nd[b];
    nmax = std::max(nmax, nd[b]);
  }
  // the forward stage at y, its intermediates kept (the stage installs the geometry)
  AjBufs B;
  EB_TRY(aj_bufs(ctx, nbk, k, B));
  eb_stage_info si{};
  EB_TRY(eb_stage_f_keep(ctx, k, nd, y, reinterpret_cast<double*>(B.f), m, &si, B.gw, ul_in, u_in));
  if (info) {
    info->lap_iters += si.lap_iters;
    info->stokes_iters += si.stokes_iters;
  }
  note_ierr(info, si.lap_ierr);
  note_ierr(info, si.stokes_ierr);
  const int* st = ctx->start.as<int>();
  const double2 *z = ctx->z.as<double2>(), *dz = ctx->dz.as<double2>(), *zk = ctx->zk.as<double2>();
  const double *ds = ctx->dsda.as<double>(), *ka = ctx->kappa.as<double>(), *hp = ctx->hpt.as<double>();
  const double* tha = ctx->tha.as<double>();
  const double2* ck = ctx->ckern.as<double2>();
  const double* lap = ctx->st_lap.as<double>();
  const double *un = lap, *ul = lap + nbk, *dphi = lap + 4 * (size_t)nbk;
  const double2* u = ctx->st_u.as<double2>();
  double* part = ctx->aj_part.as<double>();
  const size_t sm1 = sizeof(double2) * ((size_t)nmax + (size_t)nmax / 2);
  const size_t sm2 = sizeof(double2) * (2 * (size_t)nmax + (size_t)nmax / 2);
  const size_t smf = sizeof(double2) * 3 * (size_t)nmax;
  EB_TRY(set_smem((const void*)k_aj_rkup, sm2));
  EB_TRY(set_smem((const void*)k_aj_vel_local, sm1));
  EB_TRY(set_smem((const void*)k_aj_setvelf, sm1));
  EB_TRY(set_smem((const void*)k_aj_dtn, sm1));
  EB_TRY(set_smem((const void*)k_aj_pv_fine, smf));
  EB_TRY(set_smem((const void*)k_aj_extract, sm2));
  // node velocity, FILTER, EQUIT
  k_aj_rkup<<<k, SBS, sm2, s>>>(st, tha, un, dz, ds, reinterpret_cast<const double2*>(v), B.dzb, B.sb, B.thb,
                                B.unb, nmax);
  // INTERFACENEW
  k_aj_vel_local<<<k, SBS, sm1, s>>>(st, z, dz, ds, ka, hp, ck, u, un, B.gw, B.unb, m->cap, B.gwb, B.uB, B.kb,
                                     B.ckb, B.zb, B.dzb, B.sb, part, nmax);
  k_aj_charges<<<nblk(nbk, 256), 256, 0, s>>>(nbk, u, dz, hp, B.qa, B.qb);
  // double-float pair sums: positions relative to the first node, charges and cotangents
  const bool dfp = ctx->opts.adj_df > 0;
  float4 *zd = nullptr, *qad = nullptr, *qbd = nullptr, *g1d = nullptr, *g2d = nullptr, *ptd = nullptr,
         *psd = nullptr, *pqd = nullptr, *qld = nullptr;
  float2* xd = nullptr;
  const int nb = nblk(nbk, 256);
  if (dfp) {
    EB_TRY(ctx->aj_df.ensure(sizeof(float4) * 9 * (size_t)nbk + sizeof(float2) * (size_t)nbk));
    float4* p4 = ctx->aj_df.as<float4>();
    float4** c4s[] = {&zd, &qad, &qbd, &g1d, &g2d, &ptd, &psd, &pqd, &qld};
    for (float4** q : c4s) {
      *q = p4;
      p4 += nbk;
    }
    xd = reinterpret_cast<float2*>(p4);
    k_df4<<<nb, 256, 0, s>>>(nbk, z, 1, z, zd);
    k_df4<<<nb, 256, 0, s>>>(nbk, B.qa, 1, nullptr, qad);
    k_df4<<<nb, 256, 0, s>>>(nbk, B.qb, 1, nullptr, qbd);
    k_df4<<<nb, 256, 0, s>>>(nbk, B.gwb, 1, nullptr, g1d);
    k_aj_stokes_src_df<1, true><<<nbk, PBS, 0, s>>>(nbk, zd, g1d, 1.0, dz, hp, u, B.qa, B.qb, B.zb, B.dzb, B.uB);
    ctx->launches += 4;
  } else {
    k_aj_stokes_src<1, true><<<nbk, PBS, 0, s>>>(nbk, z, dz, hp, u, B.qa, B.qb, B.gwb, 1.0, B.zb, B.dzb, B.uB);
  }
  ctx->launches += 4;
  EB_TRY(eb_check_launch(ctx, "adjoint: velocity"));
  // Stokes solve: lambda = A_S^-T ubar
  eb_solve_info ai{};
  EB_TRY(eb_stokes_solve_adjoint(ctx, 2 * nbk, reinterpret_cast<const double*>(B.uB), reinterpret_cast<double*>(B.lam),
                                 m->mode, &ai, EB_DEVICE));
  if (info) info->stokes_adj_iters += ai.iters;
  note_ierr(info, ai.ierr);
  k_aj_op_local<<<k, SBS, 0, s>>>(st, z, dz, ds, ka, hp, zk, u, B.lam, B.zb, B.dzb, B.sb, B.kb, B.zkb);
  // the target side of both Stokes sums (INTERFACENEW's and FASMVP's) in one pass
  if (dfp) {
    k_df4<<<nb, 256, 0, s>>>(nbk, B.lam, 1, nullptr, g2d);
    k_aj_stokes_tgt_df<<<nbk, PBS, 0, s>>>(nbk, zd, qad, qbd, B.gwb, B.lam, B.zb);
    k_aj_stokes_src_df<-1, false><<<nbk, PBS, 0, s>>>(nbk, zd, g2d, -1.0, dz, hp, u, B.qa, B.qb, B.zb, B.dzb,
                                                      nullptr);
    eb_count_launch(ctx);
  } else {
    k_aj_stokes_tgt<<<nbk, PBS, 0, s>>>(nbk, z, B.qa, B.qb, B.gwb, B.lam, B.zb);
    k_aj_stokes_src<-1, false><<<nbk, PBS, 0, s>>>(nbk, z, dz, hp, u, B.qa, B.qb, B.lam, -1.0, B.zb, B.dzb, nullptr);
  }
  const double alpha_c = 2.0 * EB_PI * (double)(nd[k - 1] - 1) / (double)nd[k - 1];
  k_aj_setvelf<<<k, SBS, sm1, s>>>(st, z, dz, ds, dphi, B.lam, m->e0, m->cap, alpha_c, B.dzb, B.sb, B.zb, B.dphib,
                                   part, nmax);
  k_aj_dtn<<<k, SBS, sm1, s>>>(st, ds, dphi, B.dphib, B.sb, B.zb, B.psib, nmax);
  ctx->launches += 5;
  EB_TRY(eb_check_launch(ctx, "adjoint: Stokes operator"));
  // PVINTEV's Cauchy sum and its interpolation
  EB_TRY(eb_pv_fine(ctx, ul));
  const double2* pvz = ctx->pvz.as<double2>();
  const double2* pvq = ctx->pvq.as<double2>();
  const double2 cpv = make_double2(-1.0 / (2.0 * EB_PI), 0.0);
  // (evaluation points: the even fine nodes; sources and charges: the odd ones)
  if (dfp) {
    k_df4<<<nb, 256, 0, s>>>(nbk, pvz, 2, z, ptd);
    k_df4<<<nb, 256, 0, s>>>(nbk, pvz + 1, 2, z, psd);
    k_df4<<<nb, 256, 0, s>>>(nbk, pvq + 1, 2, nullptr, pqd);
    k_df2<<<nb, 256, 0, s>>>(nbk, B.psib, xd);
    k_aj_cauchy_tgt_df<false, false><<<nbk, PBS, 0, s>>>(nbk, ptd, nbk, psd, pqd, B.psib, cpv, B.ztb);
    k_aj_cauchy_src_df<false, false><<<nbk, PBS, 0, s>>>(nbk, ptd, nbk, psd, xd, cpv, pvq + 1, 2, nullptr, nullptr,
                                                         nullptr, nullptr, B.qsb, B.zsb);
    ctx->launches += 4;
  } else {
    k_aj_cauchy_tgt<false, false><<<nbk, PBS, 0, s>>>(nbk, pvz, 2, nbk, pvz + 1, 2, pvq + 1, 2, B.psib, cpv, B.ztb);
    k_aj_cauchy_src<false, false><<<nbk, PBS, 0, s>>>(nbk, pvz, 2, nbk, pvz + 1, 2, pvq + 1, 2, B.psib, cpv, nullptr,
                                                      nullptr, nullptr, nullptr, B.qsb, B.zsb);
  }
  k_aj_pv_fine<<<dim3(k, 3), SBS, smf, s>>>(st, dz, ul, hp, B.qsb, B.zsb, B.ztb, B.ulb, B.dzb, B.zb, nmax);
  ctx->launches += 3;
  EB_TRY(eb_check_launch(ctx, "adjoint: PV integral"));
  // Laplace solve: lambda_L = A_L^-T ulbar
  EB_TRY(eb_laplace_solve_adjoint(ctx, nbk, B.ulb, B.laml, m->mode, &ai, EB_DEVICE));
  if (info) info->lap_adj_iters += ai.iters;
  note_ierr(info, ai.ierr);
  k_aj_lap_local<<<nblk(nbk, 256), 256, 0, s>>>(nbk, dz, ds, ka, hp, ul, B.laml, B.zb, B.kb, B.sb, B.ql);
  const double2 clp = make_double2(0.0, 1.0 / EB_PI);
  if (dfp) {
    k_df4<<<nb, 256, 0, s>>>(nbk, B.ql, 1, nullptr, qld);
    k_df2<<<nb, 256, 0, s>>>(nbk, B.laml, xd);
    k_aj_cauchy_tgt_df<true, true><<<nbk, PBS, 0, s>>>(nbk, zd, nbk, zd, qld, B.laml, clp, B.zb);
    k_aj_cauchy_src_df<true, true><<<nbk, PBS, 0, s>>>(nbk, zd, nbk, zd, xd, clp, B.ql, 1, ul, hp, B.zb, B.dzb,
                                                       nullptr, nullptr);
    ctx->launches += 2;
  } else {
    k_aj_cauchy_tgt<true, true><<<nbk, PBS, 0, s>>>(nbk, z, 1, nbk, z, 1, B.ql, 1, B.laml, clp, B.zb);
    k_aj_cauchy_src<true, true><<<nbk, PBS, 0, s>>>(nbk, z, 1, nbk, z, 1, B.ql, 1, B.laml, clp, ul, hp, B.zb, B.dzb,
                                                    nullptr, nullptr);
  }
  k_aj_extract<<<k, SBS, sm2, s>>>(st, z, B.zb, B.dzb, B.sb, B.kb, B.thb, B.ckb, B.zkb, yb_out, nmax);
  ctx->launches += 4;
  EB_TRY(eb_check_launch(ctx, "adjoint: Laplace operator and EXTRACTDAT"));
  if (param_bar) {
    std::vector<double> h(4 * (size_t)k);
    EB_CUDA_TRY(cudaMemcpyAsync(h.data(), part, sizeof(double) * 4 * k, cudaMemcpyDeviceToHost, s));
    EB_CUDA_TRY(cudaStreamSynchronize(s));
    for (int b = 0; b < k; ++b) {
      param_bar[0] += h[4 * b];
      param_bar[1] += h[4 * b + 1] + h[4 * b + 2];
    }
  }
  return EB_OK;
}

int check_drops(int k, const int* nd) {
  for (int b = 0; b < k; ++b)
    if (nd[b] < 4 || (nd[b] & (nd[b] - 1)) != 0) {
      eb_set_last_error_msg("the adjoint of F needs power-of-two drop sizes >= 4");
      return EB_ERR_ARG;
    }
  return EB_OK;
}

}  // namespace

int eb_rk_f_vjp(eb_ctx* ctx, int k, const int* nd, const double* rku, const double* v, const eb_model* model,
                double* rku_bar, double* param_bar, eb_adjoint_info* info, int mem) {
  if (!ctx || k <= 0 || !nd || !rku || !v || !rku_bar) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  EB_TRY(check_adjoint_model(ctx, model));
  EB_TRY(check_drops(k, nd));
  cudaSetDevice(ctx->device);
  if (info) *info = eb_adjoint_info{};
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  const size_t bytes = sizeof(double) * 2 * (size_t)nbk;
  cudaStream_t s = ctx->stream;
  if (mem == EB_DEVICE) {
    EB_TRY(f_vjp_dev(ctx, k, nd, rku, v, model, rku_bar, param_bar, info));
    EB_CUDA_TRY(cudaStreamSynchronize(s));
    return EB_OK;
  }
  EB_TRY(ctx->aj_rk.ensure(3 * bytes));
  double* yd = ctx->aj_rk.as<double>();
  double* vd = yd + 2 * (size_t)nbk;
  double* od = vd + 2 * (size_t)nbk;
  EB_CUDA_TRY(cudaMemcpyAsync(yd, rku, bytes, cudaMemcpyHostToDevice, s));
  EB_CUDA_TRY(cudaMemcpyAsync(vd, v, bytes, cudaMemcpyHostToDevice, s));
  EB_TRY(f_vjp_dev(ctx, k, nd, yd, vd, model, od, param_bar, info));
  EB_CUDA_TRY(cudaMemcpyAsync(rku_bar, od, bytes, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

namespace {

// Kept solutions of one RK2 step's two stages (device, nbk + 2 nbk doubles each), or null.
struct StepSolutions {
  const double *ul0, *u0, *ul1, *u1;
};

// The transpose of one RK2 step on device arrays: rb (2 nbk, in: dJ/dy after the step,
// out: before it) from the step's start state y (2 nbk).
int step_vjp_dev(eb_ctx* ctx, int k, const int* nd, double dt, const double* y, double* rb_io,
                 const eb_model* model, double* param_bar, eb_adjoint_info* info, const StepSolutions& ss) {
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  const int neq = 2 * nbk;
  const size_t bytes = sizeof(double) * (size_t)neq;
  cudaStream_t s = ctx->stream;
  // y0, y1 (= y0 + dt k1, k1 in place), rbar, v, g2, g1
  EB_TRY(ctx->aj_rk.ensure(6 * bytes));
  double* y0 = ctx->aj_rk.as<double>();
  double* y1 = y0 + neq;
  double* rb = y1 + neq;
  double* vv = rb + neq;
  double* g2 = vv + neq;
  double* g1 = g2 + neq;
  EB_CUDA_TRY(cudaMemcpyAsync(y0, y, bytes, cudaMemcpyDeviceToDevice, s));
  EB_CUDA_TRY(cudaMemcpyAsync(rb, rb_io, bytes, cudaMemcpyDeviceToDevice, s));
  // the predictor y1 = y0 + dt F(y0)
  eb_stage_info si{};
  EB_TRY(eb_stage_f_keep(ctx, k, nd, y0, y1, model, &si, nullptr, ss.ul0, ss.u0));
  if (info) {
    info->lap_iters += si.lap_iters;
    info->stokes_iters += si.stokes_iters;
  }
  note_ierr(info, si.lap_ierr);
  note_ierr(info, si.stokes_ierr);
  const int nb = nblk(neq, 256);
  k_axpby<<<nb, 256, 0, s>>>(neq, 1.0, y0, dt, y1, y1);
  // y_next = y0 + dt/2 F(y0) + dt/2 F(y1): g2 = J(y1)^T (dt/2 rbar),
  // g1 = J(y0)^T (dt/2 rbar + dt g2), rbar_out = rbar + g2 + g1
  k_axpby<<<nb, 256, 0, s>>>(neq, 0.5 * dt, rb, 0.0, rb, vv);
  ctx->launches += 2;
  EB_TRY(f_vjp_dev(ctx, k, nd, y1, vv, model, g2, param_bar, info, ss.ul1, ss.u1));
  k_axpby<<<nb, 256, 0, s>>>(neq, 0.5 * dt, rb, dt, g2, vv);
  eb_count_launch(ctx);
  EB_TRY(f_vjp_dev(ctx, k, nd, y0, vv, model, g1, param_bar, info, ss.ul0, ss.u0));
  k_sum3<<<nb, 256, 0, s>>>(neq, rb, g2, g1, rb);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "rk2 step adjoint"));
  EB_CUDA_TRY(cudaMemcpyAsync(rb_io, rb, bytes, cudaMemcpyDeviceToDevice, s));
  return EB_OK;
}

}  // namespace

int eb_rk2_step_vjp(eb_ctx* ctx, int k, const int* nd, double dt, const double* ybar, double* rbar,
                    const eb_model* model, double* param_bar, eb_adjoint_info* info, int mem) {
  if (!ctx || k <= 0 || !nd || !ybar || !rbar) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  EB_TRY(check_adjoint_model(ctx, model));
  EB_TRY(check_drops(k, nd));
  cudaSetDevice(ctx->device);
  if (info) *info = eb_adjoint_info{};
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  const size_t bytes = sizeof(double) * 2 * (size_t)nbk;
  cudaStream_t s = ctx->stream;
  const double* y = ybar;
  double* r = rbar;
  if (mem == EB_HOST) {  // staged through the checkpoint buffer
    EB_TRY(ctx->aj_ck.ensure(2 * bytes));
    double* yd = ctx->aj_ck.as<double>();
    double* rd = yd + 2 * (size_t)nbk;
    EB_CUDA_TRY(cudaMemcpyAsync(yd, ybar, bytes, cudaMemcpyHostToDevice, s));
    EB_CUDA_TRY(cudaMemcpyAsync(rd, rbar, bytes, cudaMemcpyHostToDevice, s));
    y = yd;
    r = rd;
  }
  EB_TRY(step_vjp_dev(ctx, k, nd, dt, y, r, model, param_bar, info, StepSolutions{}));
  if (mem == EB_HOST) EB_CUDA_TRY(cudaMemcpyAsync(rbar, r, bytes, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

int eb_deformation(eb_ctx* ctx, int k, const int* nd, const double* rku, double* value, double* rku_bar, int mem) {
  if (!ctx || k <= 0 || !nd || !rku || !value) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int nbk = 0;
  std::vector<int> st(k + 1, 0);
  for (int b = 0; b < k; ++b) {
    if (nd[b] < 3) return EB_ERR_ARG;
    st[b + 1] = st[b] + nd[b];
  }
  nbk = st[k];
  const size_t bytes = sizeof(double) * 2 * (size_t)nbk;
  cudaStream_t s = ctx->stream;
  // starts, the part sums, and (host memory) the state and its gradient
  EB_TRY(ctx->aj_part.ensure(sizeof(double) * 4 * (size_t)k));
  EB_TRY(ctx->aj_rk.ensure(2 * bytes + sizeof(int) * (size_t)(k + 1)));
  double* yd = ctx->aj_rk.as<double>();
  double* gd = yd + 2 * (size_t)nbk;
  int* sd = reinterpret_cast<int*>(gd + 2 * (size_t)nbk);
  EB_CUDA_TRY(cudaMemcpyAsync(sd, st.data(), sizeof(int) * (k + 1), cudaMemcpyHostToDevice, s));
  const double* y = rku;
  double* g = rku_bar;
  if (mem == EB_HOST) {
    EB_CUDA_TRY(cudaMemcpyAsync(yd, rku, bytes, cudaMemcpyHostToDevice, s));
    y = yd;
    g = rku_bar ? gd : nullptr;
  }
  k_deformation<<<k, 256, 0, s>>>(sd, y, ctx->aj_part.as<double>(), g);
  eb_count_launch(ctx);
  EB_TRY(eb_check_launch(ctx, "deformation"));
  std::vector<double> part(k);
  EB_CUDA_TRY(cudaMemcpyAsync(part.data(), ctx->aj_part.p, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  if (mem == EB_HOST && rku_bar) EB_CUDA_TRY(cudaMemcpyAsync(rku_bar, gd, bytes, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  double J = 0.0;
  for (double p : part) J += p;
  *value = J;
  return EB_OK;
}

int eb_rk2_gradient(eb_ctx* ctx, int k, const int* nd, double dt, int nsteps, const double* y0,
                    const eb_model* model, double* value, double* y0_bar, double* param_bar,
                    eb_adjoint_info* info, int mem) {
  if (!ctx || k <= 0 || !nd || !y0 || !value || !y0_bar || nsteps < 0) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  EB_TRY(check_adjoint_model(ctx, model));
  EB_TRY(check_drops(k, nd));
  cudaSetDevice(ctx->device);
  if (info) *info = eb_adjoint_info{};
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  const size_t n = (size_t)nbk, neq = 2 * n, bytes = sizeof(double) * neq;
  cudaStream_t s = ctx->stream;
  // per step: its start state and its two stages' Laplace (nbk) and Stokes (2 nbk)
  // solutions; then the final state, the cotangent and two stage derivatives
  const size_t per_step = neq + 2 * (n + neq);
  EB_TRY(ctx->aj_ck.ensure(sizeof(double) * (per_step * (size_t)nsteps + 4 * neq)));
  double* ck = ctx->aj_ck.as<double>();
  auto state = [&](int st) { return ck + per_step * (size_t)st; };
  auto sol = [&](int st, int which) { return ck + per_step * (size_t)st + neq + (size_t)which * (n + neq); };
  double* yfin = ck + per_step * (size_t)nsteps;
  double* rb = yfin + neq;
  double* d0 = rb + neq;
  double* d1 = d0 + neq;
  EB_CUDA_TRY(cudaMemcpyAsync(nsteps > 0 ? state(0) : yfin, y0, bytes,
                              mem == EB_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
  const int nb = nblk((long long)neq, 256);
  auto add_info = [&](const eb_stage_info& si) {
    if (info) {
      info->lap_iters += si.lap_iters;
      info->stokes_iters += si.stokes_iters;
    }
    note_ierr(info, si.lap_ierr);
    note_ierr(info, si.stokes_ierr);
  };
  // forward: the RK2 steps (electric.f:762-786), each stage's solutions kept
  for (int st = 0; st < nsteps; ++st) {
    double* y = state(st);
    double* ynext = st + 1 < nsteps ? state(st + 1) : yfin;
    eb_stage_info si{};
    EB_TRY(eb_stage_f_keep(ctx, k, nd, y, d0, model, &si, nullptr, nullptr, nullptr, sol(st, 0), sol(st, 0) + n));
    add_info(si);
    k_rk_pred<<<nb, 256, 0, s>>>((int)neq, dt, y, d0, d0, ynext);  // phi0 in d0, the predictor in ynext
    eb_count_launch(ctx);
    si = eb_stage_info{};
    EB_TRY(eb_stage_f_keep(ctx, k, nd, ynext, d1, model, &si, nullptr, nullptr, nullptr, sol(st, 1),
                           sol(st, 1) + n));
    add_info(si);
    k_rk_corr<<<nb, 256, 0, s>>>((int)neq, dt, y, d0, d1, ynext);
    eb_count_launch(ctx);
  }
  EB_TRY(eb_deformation(ctx, k, nd, yfin, value, rb, EB_DEVICE));
  // reverse: each step's stages replayed with their kept solutions
  for (int st = nsteps - 1; st >= 0; --st) {
    const StepSolutions ss{sol(st, 0), sol(st, 0) + n, sol(st, 1), sol(st, 1) + n};
    EB_TRY(step_vjp_dev(ctx, k, nd, dt, state(st), rb, model, param_bar, info, ss));
  }
  EB_CUDA_TRY(cudaMemcpyAsync(y0_bar, rb, bytes, mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}
