/*
 * CPU oracle for the ElectricBubbles boundary-integral hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker and the timed CPU baseline. The GPU
 * product never links, loads or calls this file. See eb_oracle.h for how the
 * restatement is pinned (analytic known answers from the reference; end-to-end
 * parity against the Fortran binary itself is unpinned because no Fortran
 * compiler is available).
 *
 * Citations are file:line into the reference project (mcetal/ElectricBubbles).
 */
#include "eb_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef eb_or_cplx cplx;
#define EB_PI 3.14159265358979323846264338327950288

int eb_or_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static int clamp_threads(int nt) {
  if (nt <= 0) return eb_or_max_threads();
  return nt;
}

/* ======================================================================
 * Spectral toolkit
 * ====================================================================== */

/* Unnormalised complex DFT with DCFFTF (dir = -1, kernel exp(-i...)) and DCFFTB
 * (dir = +1, kernel exp(+i...)) semantics, dcfft.f:1-77 and :715-790. Written from
 * the DFT definition (radix-2 Cooley-Tukey for powers of two, direct sum otherwise);
 * FFTPACK's mixed-radix passes are not restated. */
void eb_or_fft(int n, cplx* c, int dir) {
  if (n <= 1) return;
  if ((n & (n - 1)) == 0) {
    for (int i = 1, j = 0; i < n; ++i) {
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) { cplx t = c[i]; c[i] = c[j]; c[j] = t; }
    }
    cplx* w = (cplx*)malloc(sizeof(cplx) * (size_t)(n / 2));
    for (int j = 0; j < n / 2; ++j) {
      double a = 2.0 * EB_PI * (double)j / (double)n;
      w[j] = cos(a) + (double)dir * sin(a) * I;
    }
    for (int len = 2; len <= n; len <<= 1) {
      int half = len / 2, step = n / len;
      for (int i = 0; i < n; i += len)
        for (int j = 0; j < half; ++j) {
          cplx u = c[i + j], v = c[i + j + half] * w[j * step];
          c[i + j] = u + v;
          c[i + j + half] = u - v;
        }
    }
    free(w);
    return;
  }
  cplx* out = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  for (int k = 0; k < n; ++k) {
    cplx s = 0;
    for (int j = 0; j < n; ++j) {
      long m = ((long)j * k) % n;
      double a = 2.0 * EB_PI * (double)m / (double)n;
      s += c[j] * (cos(a) + (double)dir * sin(a) * I);
    }
    out[k] = s;
  }
  memcpy(c, out, sizeof(cplx) * (size_t)n);
  free(out);
}

/* FDIFFF, dcfft.f:1371-1428: spectral derivative d/dalpha of a periodic sample
 * on alpha_j = 2 pi j / n; the Nyquist mode of an even-length sample is zeroed. */
void eb_or_fdifff(int n, const cplx* f, cplx* df) {
  cplx* c = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  memcpy(c, f, sizeof(cplx) * (size_t)n);
  eb_or_fft(n, c, -1);
  for (int i = 0; i < n; ++i) c[i] /= (double)n;
  int nsc, nscr;
  if (n % 2 == 0) { nsc = (n - 2) / 2; nscr = nsc + 1; }
  else { nsc = (n - 1) / 2; nscr = nsc; }
  for (int k = -nsc; k <= -1; ++k) df[n + k] = (double)k * I * c[n + k];
  df[0] = 0;
  for (int k = 1; k <= nscr; ++k) df[k] = (double)k * I * c[k];
  if (n % 2 == 0) df[nscr] = 0;
  eb_or_fft(n, df, +1);
  free(c);
}

/* FOURINT, electric.f:1307-1331: Fourier coefficients of the antiderivative
 * (mean and Nyquist modes dropped). */
void eb_or_fourint(int n, const cplx* zf, cplx* zfi) {
  int h = n / 2;
  zfi[0] = 0;
  for (int i = 1; i <= h - 1; ++i) zfi[i] = zf[i] / ((double)i * I);
  zfi[h] = 0;
  for (int i = 1; i <= h - 1; ++i) zfi[n - i] = -zf[n - i] / ((double)i * I);
}

static double powi_d(double x, int e) {
  double r = 1.0;
  while (e > 0) {
    if (e & 1) r *= x;
    x *= x;
    e >>= 1;
  }
  return r;
}

/* FILTER, electric.f:1152-1187: exp(-10 (k/n)^25) filter plus zeroing of real or
 * imaginary parts below 1e-13 and of the Nyquist mode. The ratio k/n is formed in
 * single precision as the reference does (FLOAT(i)/FLOAT(n), electric.f:1163). */
void eb_or_filter(int nd, cplx* cn) {
  int n = nd / 2;
  const double eps = 1e-13;
  for (int i = 0; i <= n; ++i) {
    double ratio = (double)((float)i / (float)n);
    double ffilt = exp(-10.0 * powi_d(ratio, 25));
    cplx v = ffilt * cn[i];
    if (fabs(creal(v)) < eps) v = 0.0 + cimag(v) * I;
    if (fabs(cimag(v)) < eps) v = creal(v);
    cn[i] = v;
  }
  cn[n] = 0;
  for (int i = 1; i <= n - 1; ++i) {
    double ratio = (double)((float)i / (float)n);
    double ffilt = exp(-10.0 * powi_d(ratio, 25));
    cplx v = ffilt * cn[nd - i];
    if (fabs(creal(v)) < eps) v = 0.0 + cimag(v) * I;
    if (fabs(cimag(v)) < eps) v = creal(v);
    cn[nd - i] = v;
  }
}

/* FINTERC, pv_integral.f:276-328: trigonometric interpolation of a complex periodic
 * sample from nd to 2 nd points (Nyquist mode dropped; even fine nodes coincide
 * with the coarse nodes). */
void eb_or_finterc(int nd, const cplx* f, cplx* f2) {
  int nf = 2 * nd;
  cplx* c = (cplx*)malloc(sizeof(cplx) * (size_t)nd);
  memcpy(c, f, sizeof(cplx) * (size_t)nd);
  eb_or_fft(nd, c, -1);
  c[nd / 2] = 0;
  for (int i = 0; i < nf; ++i) f2[i] = 0;
  for (int i = 0; i <= nd / 2; ++i) f2[i] = c[i] / (double)nd;
  for (int i = 0; i <= nd / 2 - 2; ++i) f2[nf - 1 - i] = c[nd - 1 - i] / (double)nd;
  eb_or_fft(nf, f2, +1);
  free(c);
}

/* FINTER, pv_integral.f:206-260: the real-valued version. The reference zeroes
 * WORK(IPT+2*NYK-1) and WORK(IPT+2*NYK) (:235-236), which are the imaginary part of
 * mode nd/2-1 and the real part of mode nd/2 in its interleaved layout; this is
 * restated as written. */
void eb_or_finter(int nd, const double* f, double* f2) {
  int nf = 2 * nd;
  cplx* c = (cplx*)malloc(sizeof(cplx) * (size_t)nd);
  cplx* w = (cplx*)malloc(sizeof(cplx) * (size_t)nf);
  for (int i = 0; i < nd; ++i) c[i] = f[i];
  eb_or_fft(nd, c, -1);
  int nyk = nd / 2;
  c[nyk - 1] = creal(c[nyk - 1]);
  c[nyk] = cimag(c[nyk]) * I;
  for (int i = 0; i < nf; ++i) w[i] = 0;
  for (int i = 0; i <= nyk; ++i) w[i] = c[i] / (double)nd;
  for (int m = nyk + 1; m <= nd - 1; ++m) w[nf - nd + m] = c[m] / (double)nd;
  eb_or_fft(nf, w, +1);
  for (int i = 0; i < nf; ++i) f2[i] = creal(w[i]);
  free(c);
  free(w);
}

/* ======================================================================
 * Geometry
 * ====================================================================== */

/* EXTRACTDAT, electric.f:636-716 (per-drop centroid zk, z', z'', curvature kappa,
 * ckern = -z''/z', tha = -kappa |z'|, dz = -z', dsda = |dz|, area). The wall data
 * xleft/slength and zc = i zbond area/(8 pi) are left to the caller. */
void eb_or_extractdat(int k, const int* nd, const double* rku, cplx* z, cplx* zk,
                      cplx* dz, double* tha, double* dsda, double* kappa, cplx* ckern,
                      double* area) {
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  for (int i = 0; i < nbk; ++i) z[i] = rku[2 * i] + rku[2 * i + 1] * I;
  int ndmax = 0;
  for (int b = 0; b < k; ++b) ndmax = nd[b] > ndmax ? nd[b] : ndmax;
  cplx* za = (cplx*)malloc(sizeof(cplx) * (size_t)ndmax);
  cplx* zai = (cplx*)malloc(sizeof(cplx) * (size_t)ndmax);
  int ist = 0;
  for (int b = 0; b < k; ++b) {
    int n = nd[b];
    memcpy(za, z + ist, sizeof(cplx) * (size_t)n);
    eb_or_fft(n, za, -1);
    zk[b] = za[0] / (double)n;
    eb_or_fdifff(n, z + ist, za);
    eb_or_fdifff(n, za, zai);
    for (int i = 0; i < n; ++i) {
      double xd = creal(za[i]), yd = cimag(za[i]);
      double xdd = creal(zai[i]), ydd = cimag(zai[i]);
      double dsdt = sqrt(xd * xd + yd * yd);
      kappa[ist + i] = -(xd * ydd - yd * xdd) / (dsdt * dsdt * dsdt);
      ckern[ist + i] = -(xdd + ydd * I) / (xd + yd * I);
      tha[ist + i] = -kappa[ist + i] * dsdt;
      dz[ist + i] = -(xd + yd * I);
      dsda[ist + i] = cabs(dz[ist + i]);
    }
    for (int i = 0; i < n; ++i) za[i] = cimag(z[ist + i]) * creal(dz[ist + i]);
    eb_or_fft(n, za, -1);
    area[b] = 2.0 * EB_PI * creal(za[0] / (double)n);
    ist += n;
  }
  free(za);
  free(zai);
}

/* ======================================================================
 * Stokes (Sherman-Lauricella) sums
 * ====================================================================== */

/* Charges of CADAPDR/CADAPMOD, cadapdrop.f:214-222 (the "fudged" signs, which are
 * also those of cadapmod.f:215-219): qa = dens dz h/(2 pi i),
 * qb = (-conj(dens) dz + dens conj(dz)) h/(2 pi i); qc = -conj(z) qa is implied. */
static void stokes_charges(int n, const cplx* dz, const double* hpt, const cplx* dens,
                           cplx* qa, cplx* qb) {
  const cplx z2pi = 1.0 / (2.0 * EB_PI * I);
  for (int j = 0; j < n; ++j) {
    qa[j] = z2pi * dens[j] * dz[j] * hpt[j];
    qb[j] = (-conj(dens[j]) * dz[j] + dens[j] * conj(dz[j])) * z2pi * hpt[j];
  }
}

/* Exact O(N^2) evaluation of the sum CADAPDR (sign = -1, cadapdrop2.f:564-620 and
 * :724-769) or CADAPMOD (sign = +1, cadap2.f:1090-1146 and :1319-1364) approximates:
 *   gradw_t = sum_{j != t} qa/D + s [ conj(qb/D) - D conj(qa) conj(1/D^2) ],
 * D = z_j - z_t. The combination z_t conj(qa) + conj(qc) of the reference equals
 * -D conj(qa) and is formed that way here to avoid cancellation. */
void eb_or_stokes_direct(int n, const cplx* z, const cplx* dz, const double* hpt,
                         const cplx* dens, int sign, cplx* gradw, int nthreads) {
  cplx* qa = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* qb = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  stokes_charges(n, dz, hpt, dens, qa, qb);
  const double s = (double)sign;
  int nt = clamp_threads(nthreads);
  (void)nt;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 16)
  for (int t = 0; t < n; ++t) {
    cplx acc = 0;
    cplx zt = z[t];
    for (int j = 0; j < n; ++j) {
      if (j == t) continue;
      cplx d = z[j] - zt;
      cplx zinv = 1.0 / d;
      cplx zinv2c = conj(zinv * zinv);
      acc += qa[j] * zinv + s * (conj(qb[j] * zinv) - d * conj(qa[j]) * zinv2c);
    }
    gradw[t] = acc;
  }
  free(qa);
  free(qb);
}

/* The same direct sum evaluated only at the nodes tidx[0..nt) (self excluded); used to
 * check large layer-potential sums on a sample of targets. */
void eb_or_stokes_direct_at(int n, const cplx* z, const cplx* dz, const double* hpt,
                            const cplx* dens, int sign, int nt_, const int* tidx, cplx* out,
                            int nthreads) {
  cplx* qa = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* qb = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  stokes_charges(n, dz, hpt, dens, qa, qb);
  const double s = (double)sign;
  int nt = clamp_threads(nthreads);
  (void)nt;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
  for (int ii = 0; ii < nt_; ++ii) {
    int t = tidx[ii];
    cplx acc = 0;
    cplx zt = z[t];
    for (int j = 0; j < n; ++j) {
      if (j == t) continue;
      cplx d = z[j] - zt;
      cplx zinv = 1.0 / d;
      cplx zinv2c = conj(zinv * zinv);
      acc += qa[j] * zinv + s * (conj(qb[j] * zinv) - d * conj(qa[j]) * zinv2c);
    }
    out[ii] = acc;
  }
  free(qa);
  free(qb);
}

/* ---- restatement of the per-level uniform-grid FMM CADAPDR/CADAPMOD ---- */

/* SLMKXP, cadap2.f:412-468 (P2M, 1-based coefficients m1[1..p], m2[1..p]). */
static void slmkxp(cplx zc, int nin, const int* idx, const cplx* zs, const cplx* qa,
                   const cplx* qb, const cplx* qc, cplx* m1, cplx* m2, int p) {
  for (int j = 1; j <= p; ++j) { m1[j] = 0; m2[j] = 0; }
  for (int ii = 0; ii < nin; ++ii) {
    int i = idx[ii];
    cplx zsh = zs[i] - zc;
    cplx z0phi = -qa[i], z0psi = -qb[i];
    for (int j = 1; j <= p; ++j) {
      m1[j] += z0phi;
      m2[j] += z0psi;
      z0phi *= zsh;
      z0psi *= zsh;
    }
    z0psi = qc[i];
    for (int j = 2; j <= p; ++j) {
      m2[j] += z0psi * (double)(j - 1);
      z0psi *= zsh;
    }
  }
}

/* SLMVALDR / SLMVAL, cadapdrop2.f:251-301 and cadap2.f:470-520 (M2P). */
static void slmval(const cplx* m1, const cplx* m2, cplx zc, int p, cplx zt, double s,
                   cplx* gw) {
  cplx zsinv = 1.0 / (zt - zc);
  cplx phi = m1[p] * zsinv;
  cplx phip = (double)p * m1[p] * zsinv;
  cplx psi = m2[p] * zsinv;
  for (int j = p - 1; j >= 1; --j) {
    phi = (phi + m1[j]) * zsinv;
    psi = (psi + m2[j]) * zsinv;
    phip = (phip + (double)j * m1[j]) * zsinv;
  }
  phip = -phip * zsinv;
  *gw += phi + s * (zt * conj(phip) + conj(psi));
}

/* SLLVALDR / SLLVAL, cadapdrop2.f:304-350 and cadap2.f:575-621 (L2P). */
static void sllval(const cplx* l1, const cplx* l2, int p, cplx zc, cplx zt, double s,
                   cplx* gw) {
  cplx zsh = zt - zc;
  cplx phi = 0, psi = 0, phip = 0;
  for (int j = p; j >= 0; --j) {
    phi = l1[j] + zsh * phi;
    psi = l2[j] + zsh * psi;
  }
  for (int j = p; j >= 1; --j) phip = (double)j * l1[j] + zsh * phip;
  *gw += phi + s * (zt * conj(phip) + conj(psi));
}

/* SLSHIFT + ADDEXP, cadap2.f:1149-1215 and :1452-1465 (M2L; binomial table
 * C(i,j) = binom(i-1, j-1) of DOINT0DR, cadapdrop2.f:53-63). */
static void slshift_add(const cplx* m1, const cplx* m2, cplx zc, int p, cplx zc2,
                        const double* binom, int ldb, cplx* l1, cplx* l2) {
  cplx z0p[64], a1[64], a2[64];
  cplx cd = 1.0 / (zc2 - zc), cdd = cd;
  z0p[0] = 1.0;
  for (int i = 1; i <= p; ++i) { z0p[i] = cdd; cdd *= cd; }
  for (int i = 1; i <= p; ++i) { a1[i] = m1[i] * z0p[i]; a2[i] = m2[i] * z0p[i]; }
  for (int m = 0; m <= p - 1; ++m) {
    cplx b1 = 0, b2 = 0;
    for (int k = 1; k <= p; ++k) {
      double c = binom[(m + k - 1) * ldb + (k - 1)];
      b1 += a1[k] * c;
      b2 += a2[k] * c;
    }
    if (m % 2 == 0) { b1 *= z0p[m]; b2 *= z0p[m]; }
    else { b1 = -b1 * z0p[m]; b2 = -b2 * z0p[m]; }
    l1[m] += b1;
    l2[m] += b2;
  }
}

/* MKINTL, cadap2.f:780-828: children of the parent's neighbours that are not
 * adjacent; returned in increasing box order (row-major), which is the order in
 * which the reference's source-box loop delivers their contributions. */
static int mkintl(int nside, int ix, int iy, int* out) {
  int imin, imax, jmin, jmax, n = 0;
  int col = ix + 1, row = iy + 1;
  if (col % 2 == 0) { imin = col - 3 > 1 ? col - 3 : 1; imax = col + 2 < nside ? col + 2 : nside; }
  else { imin = col - 2 > 1 ? col - 2 : 1; imax = col + 3 < nside ? col + 3 : nside; }
  if (row % 2 == 0) { jmin = row - 3 > 1 ? row - 3 : 1; jmax = row + 2 < nside ? row + 2 : nside; }
  else { jmin = row - 2 > 1 ? row - 2 : 1; jmax = row + 3 < nside ? row + 3 : nside; }
  for (int j = jmin; j <= jmax; ++j)
    for (int i = imin; i <= imax; ++i) {
      if (abs(col - i) <= 1 && abs(row - j) <= 1) continue;
      out[n++] = (j - 1) * nside + (i - 1);
    }
  return n;
}

/* CADAPDR (sign -1, cadapdrop.f:3-387) / CADAPMOD (sign +1, cadapmod.f:3-386) with
 * IFLAG1 = 0, IFLAG2 = 0 (free space, fields at the sources, self excluded).
 * Each level re-bins the sources (ASSIGN1, cadap2.f:252-409), forms multipoles from
 * the sources, and for every interaction-list pair evaluates the multipole directly
 * (target box with <= NTERMS/2 points) or converts it to a local expansion; the
 * near field is summed directly at the finest level (DONN0DR, cadapdrop2.f:623-722).
 * The loops are arranged per target box so that they can run on several threads;
 * every target still receives its contributions in the reference's order.
 * The reference's workspace caps (cadapdrop.f:176-185, 240-249) are lifted. */
int eb_or_cadap_fmm(int n, const cplx* zin, const cplx* dzin, const double* hpt,
                    const cplx* dens, int sign, int levmax, double tol, cplx* gradw,
                    int nthreads) {
  return eb_or_cadap_fmm_w(n, zin, dzin, hpt, dens, sign, levmax, tol, 0, 0.0, 0.0, gradw, nthreads);
}

/* MPREFLECT, cadap2.f:1468-1507: the expansions of PHI and PSI (1-based m1, m2 about
 * zc, absolute PSI) reflected across the wall y = 0, about conj(zc). */
static void mpreflect(cplx zc, const cplx* m1, const cplx* m2, int p, cplx* r1, cplx* r2) {
  r1[1] = conj(m1[1] - m2[1]);
  r2[1] = r1[1] - conj(m1[1]);
  for (int k = 2; k <= p; ++k) {
    r1[k] = conj(-m2[k] + (double)k * m1[k] + (double)(k - 1) * m1[k - 1] * zc);
    r2[k] = -conj(m1[k]) + (double)k * r1[k] + (double)(k - 1) * r1[k - 1] * conj(zc);
  }
}

/* The column range of MKINTL / MKINTR (cadap2.f:780-877), 0-based: the children of the
 * parent columns next to the parent of column c. */
static void mk_colrange(int nside, int c, int* lo, int* hi) {
  int col = c + 1;
  if (col % 2 == 0) { *lo = col - 3 > 1 ? col - 3 : 1; *hi = col + 2 < nside ? col + 2 : nside; }
  else { *lo = col - 2 > 1 ? col - 2 : 1; *hi = col + 3 < nside ? col + 3 : nside; }
  *lo -= 1;
  *hi -= 1;
}

/* The image sources of target box (tx, ty): the source boxes of the first two rows whose
 * MKINTR list (cadap2.f:830-877) holds the target, in increasing box order. MKINTR of a
 * source in row IROWB takes the columns of its parent's neighbours in rows 1 and 2, and
 * row 1 only when IROWB = 2 or the columns differ by more than one; the relation is
 * symmetric in the two boxes' columns. */
static int mkintr_sources(int nside, int tx, int ty, int* out) {
  int n = 0, lo, hi;
  if (ty > 1) return 0;
  mk_colrange(nside, tx, &lo, &hi);
  for (int sy = 0; sy <= 1 && sy < nside; ++sy)
    for (int sx = lo; sx <= hi; ++sx) {
      if (ty == 0 && sy == 0 && abs(sx - tx) <= 1) continue;
      out[n++] = sy * nside + sx;
    }
  return n;
}

/* SLDREFDR (cadapdrop2.f:857-934, sign -1) / SLDREF (cadap2.f:1509-1586, sign +1) with
 * I1 = 0: the reflected sources of one box at one target. */
static cplx sldref(cplx zt, int nin, const int* idx, const cplx* zs, const cplx* qa,
                   const cplx* qb, const cplx* qc, double s) {
  cplx phil = 0, phipl = 0, psil = 0;
  for (int jj = 0; jj < nin; ++jj) {
    int j = idx[jj];
    cplx zd = conj(zs[j]) - zt, zd2 = zd * zd, zd3 = zd2 * zd;
    cplx g1 = -conj(qb[j]) + conj(qa[j]);
    cplx d1 = -conj(qb[j]);
    cplx g2 = -conj(qc[j]) - conj(qa[j] * zs[j]);
    cplx d2 = 2.0 * g2 - conj(zs[j]) * g1;
    cplx d3 = -2.0 * conj(zs[j]) * g2;
    phil += g1 / zd;
    phil += g2 / zd2;
    phipl += g1 / zd2;
    phipl += 2.0 * g2 / zd3;
    psil += d1 / zd;
    psil += d2 / zd2;
    psil += d3 / zd3;
  }
  return phil + s * (zt * conj(phipl) + conj(psil));
}

/* CADAPDR / CADAPMOD with IFLAG2 = 1 (wall-bounded, iwall != 0): the sources are scaled
 * into the square [xleft, xleft + slength] x [0, slength] (cadapdrop.f:142-145), whose
 * bottom edge is the wall; every level adds the reflected multipoles of the first two
 * rows (MPREFLECT + MKINTR, cadapdrop2.f:159-197), and the finest level the reflected
 * near field of the first row (MKNBRRFL + SLDREFDR, cadapdrop2.f:690-721). */
int eb_or_cadap_fmm_w(int n, const cplx* zin, const cplx* dzin, const double* hpt,
                      const cplx* dens, int sign, int levmax, double tol, int iwall,
                      double xleft, double slength, cplx* gradw, int nthreads) {
  int nterms = -(int)lround(log(tol) / log(2.0));
  if (nterms > 60) return 4;
  const int p = nterms, nlmax = nterms / 2;
  const double s = (double)sign;
  int nt = clamp_threads(nthreads);
  (void)nt;
  double rminx, rminy, rscal;
  if (iwall) {
    rscal = 64.0 / slength;
    rminx = xleft;
    rminy = 0.0;
  } else {
    rminx = creal(zin[0]);
    double rmaxx = creal(zin[0]);
    rminy = cimag(zin[0]);
    double rmaxy = cimag(zin[n > 1 ? 1 : 0]);
    for (int i = 0; i < n; ++i) {
      double x = creal(zin[i]), y = cimag(zin[i]);
      if (x > rmaxx) rmaxx = x;
      if (y > rmaxy) rmaxy = y;
      if (x < rminx) rminx = x;
      if (y < rminy) rminy = y;
    }
    double rsx = rmaxx - rminx, rsy = rmaxy - rminy;
    rscal = 64.0 / (rsx > rsy ? rsx : rsy);
  }
  const cplx z2pi = 1.0 / (2.0 * 4.0 * atan(1.0) * I);
  cplx* zs = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* qa = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* qb = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* qc = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  for (int j = 0; j < n; ++j) {
    zs[j] = ((creal(zin[j]) - rminx) + (cimag(zin[j]) - rminy) * I) * rscal;
    qa[j] = z2pi * dens[j] * dzin[j] * hpt[j];
    qb[j] = (-conj(dens[j]) * dzin[j] + dens[j] * conj(dzin[j])) * z2pi * hpt[j];
    qc[j] = -z2pi * conj(zs[j]) * dens[j] * dzin[j] * hpt[j];
  }
  for (int j = 0; j < n; ++j) gradw[j] = 0;
  const int ldb = 120;
  double* binom = (double*)malloc(sizeof(double) * ldb * ldb);
  for (int i = 0; i < ldb; ++i)
    for (int j = 0; j < ldb; ++j) binom[i * ldb + j] = 0;
  binom[0] = 1.0;
  for (int i = 1; i < ldb; ++i) binom[i * ldb] = 1.0;
  for (int i = 1; i < ldb; ++i)
    for (int j = 1; j < ldb; ++j) binom[i * ldb + j] = binom[(i - 1) * ldb + j - 1] + binom[(i - 1) * ldb + j];

  int* ibox = (int*)malloc(sizeof(int) * (size_t)n);
  int* iatadr = (int*)malloc(sizeof(int) * (size_t)n);
  int nsidemax = 1 << levmax;
  size_t nbmax = (size_t)nsidemax * nsidemax;
  int* ioffst = (int*)malloc(sizeof(int) * (nbmax + 1));
  int* icnt = (int*)malloc(sizeof(int) * nbmax);
  cplx* mp1 = (cplx*)malloc(sizeof(cplx) * nbmax * (size_t)(p + 1));
  cplx* mp2 = (cplx*)malloc(sizeof(cplx) * nbmax * (size_t)(p + 1));
  /* reflected multipoles of the first two rows (wall) */
  cplx* mr1 = (cplx*)malloc(sizeof(cplx) * 2 * (size_t)nsidemax * (size_t)(p + 1));
  cplx* mr2 = (cplx*)malloc(sizeof(cplx) * 2 * (size_t)nsidemax * (size_t)(p + 1));

  for (int ilev = 1; ilev <= levmax; ++ilev) {
    int nside = 1 << ilev;
    int nboxes = nside * nside;
    double hbox = 64.0 / nside;
    /* ASSIGN1: counting sort of the sources into the level's boxes. */
    for (int b = 0; b < nboxes; ++b) icnt[b] = 0;
    for (int j = 0; j < n; ++j) {
      int ixh = (int)(creal(zs[j]) / hbox), iyh = (int)(cimag(zs[j]) / hbox);
      if (ixh >= nside) ixh = nside - 1;
      if (iyh >= nside) iyh = nside - 1;
      if (ixh < 0) ixh = 0;
      if (iyh < 0) iyh = 0;
      ibox[j] = iyh * nside + ixh;
      icnt[ibox[j]]++;
    }
    ioffst[0] = 0;
    for (int b = 0; b < nboxes; ++b) ioffst[b + 1] = ioffst[b] + icnt[b];
    for (int b = 0; b < nboxes; ++b) icnt[b] = 0;
    for (int j = 0; j < n; ++j) {
      int b = ibox[j];
      iatadr[ioffst[b] + icnt[b]++] = j;
    }
    /* Multipoles of every non-empty box (SLMKXP). */
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
    for (int b = 0; b < nboxes; ++b) {
      int nin = ioffst[b + 1] - ioffst[b];
      if (nin <= 0) continue;
      cplx zc = ((b % nside) + 0.5) * hbox + ((b / nside) + 0.5) * hbox * I;
      slmkxp(zc, nin, iatadr + ioffst[b], zs, qa, qb, qc, mp1 + (size_t)b * (p + 1),
             mp2 + (size_t)b * (p + 1), p);
      if (iwall && b < 2 * nside)
        mpreflect(zc, mp1 + (size_t)b * (p + 1), mp2 + (size_t)b * (p + 1), p,
                  mr1 + (size_t)b * (p + 1), mr2 + (size_t)b * (p + 1));
    }
    /* Interaction lists, per target box (DOINT0DR, cadapdrop2.f:84-197) and the
     * local-expansion evaluation (:200-234). */
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
    for (int t = 0; t < nboxes; ++t) {
      int ntin = ioffst[t + 1] - ioffst[t];
      if (ntin <= 0) continue;
      int tx = t % nside, ty = t / nside;
      int list[40], rlist[16];
      int nl = mkintl(nside, tx, ty, list);
      int nr = iwall ? mkintr_sources(nside, tx, ty, rlist) : 0;
      cplx zct = (tx + 0.5) * hbox + (ty + 0.5) * hbox * I;
      cplx l1[64], l2[64];
      for (int j = 0; j <= p; ++j) { l1[j] = 0; l2[j] = 0; }
      /* source boxes in increasing order, each with its direct then its reflected part
       * (the order of DOINT0DR's source loop, cadapdrop2.f:84-197) */
      for (int q = 0, qr = 0; q < nl || qr < nr;) {
        int refl = q >= nl || (qr < nr && rlist[qr] < list[q]);
        int sb = refl ? rlist[qr++] : list[q++];
        int nsin = ioffst[sb + 1] - ioffst[sb];
        if (nsin <= 0) continue;
        cplx zcs = ((sb % nside) + 0.5) * hbox + ((sb / nside) + 0.5) * hbox * I;
        const cplx* m1 = mp1 + (size_t)sb * (p + 1);
        const cplx* m2 = mp2 + (size_t)sb * (p + 1);
        if (refl) {
          zcs = conj(zcs);
          m1 = mr1 + (size_t)sb * (p + 1);
          m2 = mr2 + (size_t)sb * (p + 1);
        }
        if (ntin <= nlmax) {
          for (int kk = 0; kk < ntin; ++kk) {
            int jt = iatadr[ioffst[t] + kk];
            slmval(m1, m2, zcs, p, zs[jt], s, &gradw[jt]);
          }
        } else {
          slshift_add(m1, m2, zcs, p, zct, binom, ldb, l1, l2);
        }
      }
      if (ntin > nlmax) {
        for (int kk = 0; kk < ntin; ++kk) {
          int jt = iatadr[ioffst[t] + kk];
          sllval(l1, l2, p, zct, zs[jt], s, &gradw[jt]);
        }
      }
    }
  }
  /* Near field at the finest level: DONN0DR with SLSELFDR/SLDIRDR (sign -1) or
   * DONN0 with SLSELF/SLDIR (sign +1). */
  {
    int nside = 1 << levmax;
    int nboxes = nside * nside;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
    for (int t = 0; t < nboxes; ++t) {
      int ntin = ioffst[t + 1] - ioffst[t];
      if (ntin <= 0) continue;
      int tx = t % nside, ty = t / nside;
      for (int jy = ty - 1; jy <= ty + 1; ++jy) {
        if (jy < 0 || jy >= nside) continue;
        for (int jx = tx - 1; jx <= tx + 1; ++jx) {
          if (jx < 0 || jx >= nside) continue;
          int sb = jy * nside + jx;
          int s0 = ioffst[sb], nsin = ioffst[sb + 1] - s0;
          if (nsin <= 0) continue;
          for (int kk = 0; kk < ntin; ++kk) {
            int it = iatadr[ioffst[t] + kk];
            cplx zt = zs[it];
            if (sb == t) {
              cplx phil = 0, phip = 0, psil = 0;
              for (int jj = 0; jj < nsin; ++jj) {
                if (jj == kk) continue;
                int j = iatadr[s0 + jj];
                cplx zd = zs[j] - zt, zd2 = zd * zd;
                phil += qa[j] / zd;
                phip += qa[j] / zd2;
                psil += qb[j] / zd;
                psil += qc[j] / zd2;
              }
              gradw[it] += phil + s * (zt * conj(phip) + conj(psil));
            } else {
              for (int jj = 0; jj < nsin; ++jj) {
                int j = iatadr[s0 + jj];
                cplx zinv = 1.0 / (zs[j] - zt);
                cplx zinv2c = conj(zinv * zinv);
                gradw[it] += qa[j] * zinv + s * (conj(qb[j] * zinv) + (zt * conj(qa[j]) + conj(qc[j])) * zinv2c);
              }
            }
          }
        }
      }
      /* reflected near field of the first row (DONN0DR's IFLAG2 loop, after the direct
       * near field of every box): the first-row source boxes next to the target box */
      if (iwall && ty == 0) {
        for (int sx = tx - 1; sx <= tx + 1; ++sx) {
          if (sx < 0 || sx >= nside) continue;
          int s0 = ioffst[sx], nsin = ioffst[sx + 1] - s0;
          if (nsin <= 0) continue;
          for (int kk = 0; kk < ntin; ++kk) {
            int it = iatadr[ioffst[t] + kk];
            gradw[it] += sldref(zs[it], nsin, iatadr + s0, zs, qa, qb, qc, s);
          }
        }
      }
    }
  }
  for (int j = 0; j < n; ++j) gradw[j] *= rscal;
  free(zs); free(qa); free(qb); free(qc); free(binom); free(ibox); free(iatadr);
  free(ioffst); free(icnt); free(mp1); free(mp2); free(mr1); free(mr2);
  return 0;
}

/* Exact value of the reflected part of the wall-bounded sum (IFLAG2 = 1): the images of
 * all sources across y = 0, the target's own image included, with the pair terms of
 * SLDREFDR (sign -1) / SLDREF (sign +1) in physical coordinates. With qc = -conj(z) qa,
 *   gamma1 = conj(qa) - conj(qb), gamma2 = 2 i y_j conj(qa), delta1 = -conj(qb),
 *   Phi = gamma1/zeta + gamma2/zeta^2,  zeta = conj(z_j) - z_t,
 * and z_t conj(Phi') + conj(Psi) = (z_t - z_j) conj(gamma1/zeta^2 + 2 gamma2/zeta^3)
 * + 2 conj(gamma2/zeta^2) + conj(delta1/zeta) (no terms of size |z|). */
void eb_or_stokes_image_direct(int n, const cplx* z, const cplx* dz, const double* hpt,
                               const cplx* dens, int sign, cplx* gimg, int nthreads) {
  cplx* qa = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  cplx* qb = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  stokes_charges(n, dz, hpt, dens, qa, qb);
  const double s = (double)sign;
  int nt = clamp_threads(nthreads);
  (void)nt;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 16)
  for (int t = 0; t < n; ++t) {
    cplx acc = 0, zt = z[t];
    for (int j = 0; j < n; ++j) {
      cplx g1 = conj(qa[j]) - conj(qb[j]), d1 = -conj(qb[j]);
      cplx g2 = 2.0 * I * cimag(z[j]) * conj(qa[j]);
      cplx tz = 1.0 / (conj(z[j]) - zt), t2 = tz * tz, dd = zt - z[j];
      acc += g1 * tz + g2 * t2 +
             s * (dd * conj(g1 * t2 + 2.0 * g2 * t2 * tz) + 2.0 * conj(g2 * t2) + conj(d1 * tz));
    }
    gimg[t] = acc;
  }
  free(qa);
  free(qb);
}

/* REFSING, reflect.f:28-86: the images across y = 0 of the log sources zc at the drop
 * centres zk and of the poles zb, added to phi, phi' and psi at ztarg. */
void eb_or_refsing(cplx zt, int k, const cplx* zk, const cplx* zc, const cplx* zb, cplx* phi,
                   cplx* phip, cplx* psi) {
  for (int j = 0; j < k; ++j) {
    cplx zdis = zt - conj(zk[j]), zdis2 = zdis * zdis;
    cplx gamma1 = -conj(zb[j]), delta1 = gamma1, delta2 = conj(zk[j]) * gamma1;
    *phi += gamma1 / zdis;
    *phip -= gamma1 / zdis2;
    *psi += delta1 / zdis;
    *psi += delta2 / zdis2;
    *phi -= zc[j] * clog(zdis);
    *phip -= zc[j] / zdis;
    *psi -= conj(zc[j]) * clog(zdis);
    cplx alpha1 = conj(zc[j]) * (zk[j] - conj(zk[j]));
    cplx beta1 = zc[j] * conj(zk[j]) + alpha1, beta2 = alpha1 * conj(zk[j]);
    *phi += alpha1 / zdis;
    *phip -= alpha1 / zdis2;
    *psi += beta1 / zdis;
    *psi += beta2 / zdis2;
  }
}

/* The wall data of EXTRACTDAT (electric.f:657-711): xleft = min x, slength =
 * max(max x - min x, max y) over all nodes. */
void eb_or_wallinfo(int nbk, const cplx* z, double* xleft, double* slength) {
  double xmin = 1e10, xmax = -1e10, ymax = -1e10;
  for (int i = 0; i < nbk; ++i) {
    double x = creal(z[i]), y = cimag(z[i]);
    xmin = x < xmin ? x : xmin;
    xmax = x > xmax ? x : xmax;
    ymax = y > ymax ? y : ymax;
  }
  *xleft = xmin;
  *slength = xmax - xmin > ymax ? xmax - xmin : ymax;
}

/* ======================================================================
 * Cauchy (Laplace) sums
 * ====================================================================== */

/* Exact value of DAPIF2 with IFLAG7 = 3 (dapif1.f:552-558, 1071-1074; the pair
 * kernel of DABARR, dapif3.f:460-545): field_t = sum_j q_j / (z_t - z_j), skipping
 * j == t when `self` is set (sources and targets are then the same points). */
void eb_or_cauchy_direct(int nt, const cplx* zt, int ns, const cplx* zsrc, const cplx* q,
                         int self, cplx* field, int nthreads) {
  int nth = clamp_threads(nthreads);
  (void)nth;
#pragma omp parallel for num_threads(nth) schedule(dynamic, 16)
  for (int t = 0; t < nt; ++t) {
    cplx acc = 0, z = zt[t];
    for (int j = 0; j < ns; ++j) {
      if (self && j == t) continue;
      acc += q[j] / (z - zsrc[j]);
    }
    field[t] = acc;
  }
}

/* ======================================================================
 * Operators
 * ====================================================================== */

static double* per_point_h(const eb_or_geom* g) {
  double* h = (double*)malloc(sizeof(double) * (size_t)g->nbk);
  int ist = 0;
  for (int b = 0; b < g->k; ++b) {
    for (int i = 0; i < g->nd[b]; ++i) h[ist + i] = 2.0 * EB_PI / g->nd[b];
    ist += g->nd[b];
  }
  return h;
}

/* gw += the exact reflected part of the wall-bounded sum */
static void add_images(const eb_or_geom* g, const double* h, const cplx* dens, int sign, cplx* gw,
                       int nthreads) {
  cplx* gi = (cplx*)malloc(sizeof(cplx) * (size_t)g->nbk);
  eb_or_stokes_image_direct(g->nbk, g->z, g->dz, h, dens, sign, gi, nthreads);
  for (int i = 0; i < g->nbk; ++i) gw[i] += gi[i];
  free(gi);
}

/* FASMVP, stokesbubb.f:496-614 (the Stokes matvec behind MATVEC,
 * stokesbubb.f:419-465): u is the interleaved real vector of length 2 nbk. */
void eb_or_fasmvp(const eb_or_geom* g, const double* u, double* w, int mode,
                  int nthreads) {
  int nbk = g->nbk, k = g->k;
  cplx* dens = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* stress = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* za = (cplx*)malloc(sizeof(cplx) * (size_t)k);
  double* pk = (double*)malloc(sizeof(double) * (size_t)k);
  double* h = per_point_h(g);
  for (int i = 0; i < nbk; ++i) dens[i] = u[2 * i] + u[2 * i + 1] * I;
  int ist = 0;
  for (int b = 0; b < k; ++b) {
    double hb = 2.0 * EB_PI / g->nd[b];
    za[b] = 0;
    pk[b] = 0;
    for (int i = 0; i < g->nd[b]; ++i) {
      cplx zdis = g->z[ist + i] - g->zk[b];
      double zx = creal(dens[ist + i] * g->dz[ist + i] / (zdis * zdis));
      pk[b] += 2.0 * hb * zx / EB_PI;
      za[b] += hb * dens[ist + i];
    }
    ist += g->nd[b];
  }
  double pinf = -pk[0];
  for (int b = 0; b < k; ++b) pk[b] += pinf;
  /* CADAPDR with IFLAG2 = iwall (stokesbubb.f:553-563) */
  if (mode == EB_OR_CADAP) {
    eb_or_cadap_fmm_w(nbk, g->z, g->dz, h, dens, -1, 7, 1e-13, g->iwall, g->xleft, g->slength, stress,
                      nthreads);
  } else {
    eb_or_stokes_direct(nbk, g->z, g->dz, h, dens, -1, stress, nthreads);
    if (g->iwall) add_images(g, h, dens, -1, stress, nthreads);
  }
  ist = 0;
  for (int b = 0; b < k; ++b) {
    double qwi = 2.0 * EB_PI / g->nd[b];
    for (int i = 0; i < g->nd[b]; ++i) {
      int t = ist + i;
      cplx zu = dens[t], z = g->z[t];
      cplx zn = -I * g->dz[t] / g->dsda[t];
      cplx zself = zu * qwi * g->dsda[t] * 0.5 * g->kappa[t] / EB_PI;
      zself = zself - conj(zu) * qwi * g->dsda[t] * 0.5 * g->kappa[t] * zn * zn / EB_PI;
      stress[t] = stress[t] + zself - 0.5 * I * (pinf - pk[b]) * z;
      cplx wt = dens[t] + za[b] + stress[t];
      w[2 * t] = creal(wt);
      w[2 * t + 1] = cimag(wt);
    }
    ist += g->nd[b];
  }
  free(dens); free(stress); free(za); free(pk); free(h);
}

/* ======================================================================
 * DAPIF2 with IFLAG7 = 3 (dapif1.f:458-1077): the Cauchy sum
 *   field_i = sum_{j != i} q_j / (z_i - z_j)
 * by the Carrier-Greengard-Rokhlin adaptive FMM the reference cites (dapif1.f:468-471).
 * Restated: the points scaled into the root square with factor 0.99 (dapif1.f:743-767);
 * a box with more than napb points split into four (DAASSI, dapif1.f:1165-1255);
 * NTERMS = -nint(log2 tol) + 3 expansion terms (dapif1.f:688); the lists of DALI12 /
 * DALI34 (dapif2.f:3-356): list 1 the adjacent leaves (direct sum, DABARR's pair loop,
 * dapif3.f:460-545), list 2 the children of the parent's colleagues that are not
 * adjacent (M2L, DAFLEX), list 3 the descendants of the colleagues that are not adjacent
 * while their parents are (M2P, DSLOR1, dapif3.f:1724-1749) and its dual list 4 (P2L,
 * DSLOT3, dapif3.f:1387-1410); upward pass P2M + M2M (DAUPWD, dapif2.f:478-595),
 * downward pass L2L + L2P (DADNWD, dapif3.f:553-680). Expansions are scaled by the box
 * side r: field = (1/r) sum_k a_k / u^(k+1) (multipole), (1/r) sum_m L_m v^m (local),
 * u, v the offsets from the centre in units of r. The reference's 90-degree symmetry
 * shortcut of M2L (DAINSY/DASYME) and its per-distance reduced orders are not restated:
 * they change the cost, not the sums.
 * ====================================================================== */
typedef struct {
  cplx c;           /* centre */
  double r;         /* side */
  int level, parent, child[4], nchild, start, count, ix, iy;
  int *ul, nu, *vl, nv, *wl, nw, *xl, nx; /* lists 1-4 */
  int cu, cv, cw, cx;                     /* capacities */
} dbox;

static void dl_push(int** a, int* n, int* cap, int v) {
  if (*n == *cap) {
    *cap = *cap ? 2 * *cap : 8;
    *a = (int*)realloc(*a, sizeof(int) * (size_t)*cap);
  }
  (*a)[(*n)++] = v;
}

static int dbox_adjacent(const dbox* a, const dbox* b) {
  /* boxes of levels la <= lb touch (or coincide) iff b's grid cell, seen at a's level
   * with one cell of margin, overlaps a */
  const dbox* s = a->level <= b->level ? a : b;
  const dbox* t = a->level <= b->level ? b : a;
  int f = t->level - s->level;
  long x0 = (long)s->ix << f, x1 = ((long)(s->ix + 1) << f) - 1;
  long y0 = (long)s->iy << f, y1 = ((long)(s->iy + 1) << f) - 1;
  return t->ix >= x0 - 1 && t->ix <= x1 + 1 && t->iy >= y0 - 1 && t->iy <= y1 + 1;
}

void eb_or_dapif2(int n, const cplx* z, const cplx* q, double tol, int napb, cplx* field,
                  int nthreads) {
  nthreads = clamp_threads(nthreads);
  int p = -(int)lround(log(tol) / log(2.0)) + 3;
  if (p < 4) p = 4;
  if (p > 60) p = 60;
  double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  for (int i = 0; i < n; ++i) {
    xmin = fmin(xmin, creal(z[i])); xmax = fmax(xmax, creal(z[i]));
    ymin = fmin(ymin, cimag(z[i])); ymax = fmax(ymax, cimag(z[i]));
  }
  double side = fmax(xmax - xmin, ymax - ymin) / 0.99;
  if (!(side > 0)) side = 1.0;
  int* perm = (int*)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  int nb = 1, capb = 1024;
  dbox* B = (dbox*)calloc((size_t)capb, sizeof(dbox));
  B[0].c = 0.5 * (xmin + xmax) + 0.5 * (ymin + ymax) * I;
  B[0].r = side;
  B[0].parent = -1;
  B[0].count = n;
  /* DAASSI: split boxes with more than napb points, level by level */
  int* tmp = (int*)malloc(sizeof(int) * (size_t)n);
  for (int b = 0; b < nb; ++b) {
    if (B[b].count <= napb || B[b].level >= 40) continue;
    int cnt[4] = {0, 0, 0, 0};
    const int s0 = B[b].start, m = B[b].count;
    for (int t = 0; t < m; ++t) {
      cplx w = z[perm[s0 + t]] - B[b].c;
      int qd = (creal(w) >= 0 ? 1 : 0) + (cimag(w) >= 0 ? 2 : 0);
      cnt[qd]++;
    }
    int off[4] = {0, cnt[0], cnt[0] + cnt[1], cnt[0] + cnt[1] + cnt[2]};
    int pos[4] = {off[0], off[1], off[2], off[3]};
    for (int t = 0; t < m; ++t) {
      cplx w = z[perm[s0 + t]] - B[b].c;
      int qd = (creal(w) >= 0 ? 1 : 0) + (cimag(w) >= 0 ? 2 : 0);
      tmp[pos[qd]++] = perm[s0 + t];
    }
    memcpy(perm + s0, tmp, sizeof(int) * (size_t)m);
    for (int qd = 0; qd < 4; ++qd) {
      if (!cnt[qd]) continue;
      if (nb == capb) {
        capb *= 2;
        B = (dbox*)realloc(B, sizeof(dbox) * (size_t)capb);
      }
      dbox* c = &B[nb];
      memset(c, 0, sizeof(dbox));
      double h = 0.25 * B[b].r;
      c->c = B[b].c + ((qd & 1) ? h : -h) + ((qd & 2) ? h : -h) * I;
      c->r = 0.5 * B[b].r;
      c->level = B[b].level + 1;
      c->parent = b;
      c->start = s0 + off[qd];
      c->count = cnt[qd];
      c->ix = 2 * B[b].ix + (qd & 1);
      c->iy = 2 * B[b].iy + ((qd >> 1) & 1);
      B[b].child[B[b].nchild++] = nb;
      nb++;
    }
  }
  free(tmp);
  int L = 0;
  for (int b = 0; b < nb; ++b) L = B[b].level > L ? B[b].level : L;
  /* colleagues (same level, adjacent, self included), then the lists */
  int** col = (int**)calloc((size_t)nb, sizeof(int*));
  int* ncol = (int*)calloc((size_t)nb, sizeof(int));
  for (int b = 0; b < nb; ++b) {
    col[b] = (int*)malloc(sizeof(int) * 9);
    if (B[b].parent < 0) {
      col[b][ncol[b]++] = b;
      continue;
    }
    int P = B[b].parent;
    for (int a = 0; a < ncol[P]; ++a) {
      int Q = col[P][a];
      for (int cc = 0; cc < B[Q].nchild; ++cc) {
        int C = B[Q].child[cc];
        if (abs(B[C].ix - B[b].ix) <= 1 && abs(B[C].iy - B[b].iy) <= 1 && ncol[b] < 9) col[b][ncol[b]++] = C;
      }
    }
  }
  for (int b = 0; b < nb; ++b) {
    dbox* X = &B[b];
    int P = X->parent;
    if (P >= 0) /* list 2 */
      for (int a = 0; a < ncol[P]; ++a) {
        int Q = col[P][a];
        for (int cc = 0; cc < B[Q].nchild; ++cc) {
          int C = B[Q].child[cc];
          if (!(abs(B[C].ix - X->ix) <= 1 && abs(B[C].iy - X->iy) <= 1)) dl_push(&X->vl, &X->nv, &X->cv, C);
        }
      }
    if (X->nchild) continue;
    /* lists 1 and 3 of a leaf: colleagues, and below the split ones */
    int stack[256], sp = 0;
    for (int a = 0; a < ncol[b]; ++a) {
      int C = col[b][a];
      if (!B[C].nchild) {
        dl_push(&X->ul, &X->nu, &X->cu, C);
        continue;
      }
      for (int cc = 0; cc < B[C].nchild; ++cc) stack[sp++] = B[C].child[cc];
      while (sp > 0) {
        int D = stack[--sp];
        if (!dbox_adjacent(X, &B[D])) {
          dl_push(&X->wl, &X->nw, &X->cw, D);                 /* list 3 */
          dl_push(&B[D].xl, &B[D].nx, &B[D].cx, b);           /* its dual, list 4 */
        } else if (!B[D].nchild) {
          dl_push(&X->ul, &X->nu, &X->cu, D);                 /* finer adjacent leaf */
          dl_push(&B[D].ul, &B[D].nu, &B[D].cu, b);           /* and the converse */
        } else {
          for (int cc = 0; cc < B[D].nchild && sp < 250; ++cc) stack[sp++] = B[D].child[cc];
        }
      }
    }
  }
  /* binomials C(i, j), i, j < 2p + 2 */
  const int lb = 2 * p + 2;
  double* bin = (double*)calloc((size_t)lb * lb, sizeof(double));
  for (int i = 0; i < lb; ++i) {
    bin[i * lb] = 1.0;
    for (int j = 1; j <= i; ++j) bin[i * lb + j] = bin[(i - 1) * lb + j - 1] + bin[(i - 1) * lb + j];
  }
  cplx* M = (cplx*)calloc((size_t)nb * p, sizeof(cplx));
  cplx* Lc = (cplx*)calloc((size_t)nb * p, sizeof(cplx));
  /* upward pass: P2M at leaves, M2M level by level */
  for (int l = L; l >= 0; --l) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
    for (int b = 0; b < nb; ++b) {
      if (B[b].level != l) continue;
      cplx* mb = M + (size_t)b * p;
      if (!B[b].nchild) {
        for (int t = 0; t < B[b].count; ++t) {
          int j = perm[B[b].start + t];
          cplx w = (z[j] - B[b].c) / B[b].r, pw = 1.0;
          for (int k = 0; k < p; ++k) { mb[k] += q[j] * pw; pw *= w; }
        }
      } else {
        for (int cc = 0; cc < B[b].nchild; ++cc) {
          int C = B[b].child[cc];
          cplx e = (B[C].c - B[b].c) / B[b].r, ep[64], hp = 1.0;
          ep[0] = 1.0;
          for (int k = 1; k < p; ++k) ep[k] = ep[k - 1] * e;
          cplx a[64];
          for (int k = 0; k < p; ++k) { a[k] = M[(size_t)C * p + k] * hp; hp *= 0.5; }
          for (int k = 0; k < p; ++k) {
            cplx s = 0;
            for (int l2 = 0; l2 <= k; ++l2) s += bin[k * lb + l2] * ep[k - l2] * a[l2];
            mb[k] += s;
          }
        }
      }
    }
  }
  /* list 2 (M2L) and list 4 (P2L) into every box's local expansion */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (int b = 0; b < nb; ++b) {
    cplx* lbx = Lc + (size_t)b * p;
    for (int a = 0; a < B[b].nv; ++a) {
      int S = B[b].vl[a];
      cplx d = (B[b].c - B[S].c) / B[b].r, dinv = 1.0 / d, dp[130];
      dp[0] = dinv;
      for (int k = 1; k < 2 * p + 1; ++k) dp[k] = dp[k - 1] * dinv;
      const cplx* ms = M + (size_t)S * p;
      for (int m = 0; m < p; ++m) {
        cplx s = 0;
        for (int k = 0; k < p; ++k) s += ms[k] * bin[(m + k) * lb + k] * dp[m + k];
        lbx[m] += (m & 1) ? -s : s;
      }
    }
    for (int a = 0; a < B[b].nx; ++a) {
      int S = B[b].xl[a];
      for (int t = 0; t < B[S].count; ++t) {
        int j = perm[B[S].start + t];
        cplx ws = (z[j] - B[b].c) / B[b].r, wi = 1.0 / ws, pw = wi;
        for (int m = 0; m < p; ++m) { lbx[m] -= q[j] * pw; pw *= wi; }
      }
    }
  }
  /* L2L level by level */
  for (int l = 1; l <= L; ++l) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
    for (int b = 0; b < nb; ++b) {
      if (B[b].level != l) continue;
      int P = B[b].parent;
      cplx e = (B[b].c - B[P].c) / B[P].r, ep[64];
      ep[0] = 1.0;
      for (int k = 1; k < p; ++k) ep[k] = ep[k - 1] * e;
      const cplx* lp = Lc + (size_t)P * p;
      cplx* lc = Lc + (size_t)b * p;
      double hj = 0.5;  /* (r_c / r_p) 2^-j */
      for (int j = 0; j < p; ++j) {
        cplx s = 0;
        for (int m = j; m < p; ++m) s += lp[m] * bin[m * lb + j] * ep[m - j];
        lc[j] += hj * s;
        hj *= 0.5;
      }
    }
  }
  /* leaves: L2P, list 3 (M2P) and list 1 (direct) */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
  for (int b = 0; b < nb; ++b) {
    if (B[b].nchild) continue;
    const dbox* X = &B[b];
    for (int t = 0; t < X->count; ++t) {
      int i = perm[X->start + t];
      cplx v = (z[i] - X->c) / X->r, s = 0, pw = 1.0;
      const cplx* lbx = Lc + (size_t)b * p;
      for (int m = 0; m < p; ++m) { s += lbx[m] * pw; pw *= v; }
      cplx f = s / X->r;
      for (int a = 0; a < X->nw; ++a) {
        int W = X->wl[a];
        cplx u = (z[i] - B[W].c) / B[W].r, ui = 1.0 / u, pu = ui, sm = 0;
        const cplx* mw = M + (size_t)W * p;
        for (int k = 0; k < p; ++k) { sm += mw[k] * pu; pu *= ui; }
        f += sm / B[W].r;
      }
      for (int a = 0; a < X->nu; ++a) {
        int S = X->ul[a];
        for (int tt = 0; tt < B[S].count; ++tt) {
          int j = perm[B[S].start + tt];
          if (j != i) f += q[j] / (z[i] - z[j]);
        }
      }
      field[i] = f;
    }
  }
  for (int b = 0; b < nb; ++b) { free(B[b].ul); free(B[b].vl); free(B[b].wl); free(B[b].xl); free(col[b]); }
  free(col); free(ncol); free(B); free(perm); free(bin); free(M); free(Lc);
}

/* FASMVP_LAP, laplace.f:159-262 (the Laplace matvec behind MATVEC_LAPL,
 * laplace.f:429-465). Only the first nbk entries of w are written; the reference
 * also accumulates k constraint sums past the end (:252-259). */
void eb_or_fasmvp_lap2(const eb_or_geom* g, const double* u, double* w, int mode, int nthreads) {
  int nbk = g->nbk;
  cplx* q = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* cf = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  const cplx z2pii = 1.0 / (2.0 * EB_PI * I);
  int ist = 0;
  for (int b = 0; b < g->k; ++b) {
    double hb = 2.0 * EB_PI / g->nd[b];
    for (int i = 0; i < g->nd[b]; ++i) q[ist + i] = u[ist + i] * g->dz[ist + i] * hb;
    ist += g->nd[b];
  }
  if (mode == EB_OR_CADAP)
    eb_or_dapif2(nbk, g->z, q, 1e-11, 30, cf, nthreads);  /* laplace.f:211: TOL 1e-11, NAPB 30 */
  else
    eb_or_cauchy_direct(nbk, g->z, nbk, g->z, q, 1, cf, nthreads);
  ist = 0;
  for (int b = 0; b < g->k; ++b) {
    double hs = 2.0 * EB_PI / g->nd[b];
    for (int i = 0; i < g->nd[b]; ++i) {
      int t = ist + i;
      double self = 0.25 * hs * g->kappa[t] * g->dsda[t] / EB_PI;
      double zc = self * u[t] - creal(z2pii * cf[t]);
      double wt = u[t] + 2.0 * zc;
      double du = hs * u[t] * g->dsda[t];
      w[t] = wt - 2.0 * du;
    }
    ist += g->nd[b];
  }
  free(q);
  free(cf);
}

void eb_or_fasmvp_lap(const eb_or_geom* g, const double* u, double* w, int nthreads) {
  eb_or_fasmvp_lap2(g, u, w, EB_OR_DIRECT, nthreads);
}

/* PVINTEV, pv_integral.f:53-204: principal-value Cauchy integral by the alternating
 * point rule on the 2x Fourier-interpolated curve (charges on the odd fine nodes,
 * evaluation at the even fine nodes, which are the original nodes). */
static void pvintev_impl(int k, const int* nd, const cplx* z, const cplx* ucmplx,
                         cplx* phicmplx, int mode, int nthreads) {
  int nbk = 0, ndmax = 0;
  for (int b = 0; b < k; ++b) { nbk += nd[b]; ndmax = nd[b] > ndmax ? nd[b] : ndmax; }
  cplx* zsrc = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* ztgt = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* qs = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* u2 = (cplx*)malloc(sizeof(cplx) * 2 * (size_t)ndmax);
  double* xc = (double*)malloc(sizeof(double) * (size_t)ndmax);
  double* yc = (double*)malloc(sizeof(double) * (size_t)ndmax);
  double* x2 = (double*)malloc(sizeof(double) * 2 * (size_t)ndmax);
  double* y2 = (double*)malloc(sizeof(double) * 2 * (size_t)ndmax);
  cplx* cf = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  int ist = 0;
  for (int b = 0; b < k; ++b) {
    int n = nd[b];
    double hb = 2.0 * EB_PI / n;
    eb_or_finterc(n, ucmplx + ist, u2);
    for (int i = 0; i < n; ++i) { xc[i] = creal(z[ist + i]); yc[i] = cimag(z[ist + i]); }
    eb_or_finter(n, xc, x2);
    eb_or_finter(n, yc, y2);
    for (int i = 0; i < n; ++i) {
      zsrc[ist + i] = x2[2 * i + 1] + y2[2 * i + 1] * I;
      ztgt[ist + i] = x2[2 * i] + y2[2 * i] * I;
      qs[ist + i] = u2[2 * i + 1] * hb;
    }
    ist += n;
  }
  /* DAPIF2 runs on all 2N fine points X2, Y2 (pv_integral.f:174-176); the even ones
   * carry zero charge and the odd ones are never read, so only odd-source -> even-node
   * pairs contribute. The field is read at the even fine nodes (CFIELD(2I-1),
   * :192-201), FINTER's interpolated positions: they differ from the original nodes by
   * FINTER's zeroed parts of modes nd/2-1 and nd/2 (pv_integral.f:235-236). */
  if (mode == EB_OR_CADAP) {
    /* DAPIF2 on all 2N fine points, TOL 1e-10 (pv_integral.f:176): charges on the odd
     * fine nodes, the field read at the even ones (the original nodes) */
    cplx* zall = (cplx*)malloc(sizeof(cplx) * 2 * (size_t)nbk);
    cplx* qall = (cplx*)calloc(2 * (size_t)nbk, sizeof(cplx));
    cplx* fall = (cplx*)malloc(sizeof(cplx) * 2 * (size_t)nbk);
    for (int i = 0; i < nbk; ++i) {
      zall[2 * i] = ztgt[i];
      zall[2 * i + 1] = zsrc[i];
      qall[2 * i + 1] = qs[i];
    }
    eb_or_dapif2(2 * nbk, zall, qall, 1e-10, 30, fall, nthreads);
    for (int i = 0; i < nbk; ++i) cf[i] = fall[2 * i];
    free(zall); free(qall); free(fall);
  } else {
    eb_or_cauchy_direct(nbk, ztgt, nbk, zsrc, qs, 0, cf, nthreads);
  }
  const cplx z2pii = 1.0 / (2.0 * EB_PI * I);
  for (int i = 0; i < nbk; ++i) phicmplx[i] = -z2pii * cf[i];
  free(zsrc); free(ztgt); free(qs); free(u2); free(xc); free(yc); free(x2); free(y2); free(cf);
}

void eb_or_pvintev(int k, const int* nd, const cplx* z, const cplx* ucmplx, cplx* phicmplx,
                   int nthreads) {
  pvintev_impl(k, nd, z, ucmplx, phicmplx, EB_OR_DIRECT, nthreads);
}

/* DIRICH_NEU_MAP, laplace.f:266-331. */
static void dirich_neu_map_impl(const eb_or_geom* g, const double* u, double* phi,
                                double* psi, double* dphi_dn, int mode, int nthreads) {
  int nbk = g->nbk;
  cplx* uc = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* ph = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  for (int i = 0; i < nbk; ++i) uc[i] = u[i] * g->dz[i];
  pvintev_impl(g->k, g->nd, g->z, uc, ph, mode, nthreads);
  int ndmax = 0;
  for (int b = 0; b < g->k; ++b) ndmax = g->nd[b] > ndmax ? g->nd[b] : ndmax;
  cplx* zf = (cplx*)malloc(sizeof(cplx) * (size_t)ndmax);
  cplx* zfi = (cplx*)malloc(sizeof(cplx) * (size_t)ndmax);
  int ist = 0;
  for (int b = 0; b < g->k; ++b) {
    int n = g->nd[b];
    for (int i = 0; i < n; ++i) {
      cplx zphi = -0.5 * u[ist + i] - ph[ist + i] - g->z[ist + i];
      phi[ist + i] = creal(zphi);
      psi[ist + i] = cimag(zphi);
      zf[i] = psi[ist + i];
    }
    eb_or_fdifff(n, zf, zfi);
    for (int i = 0; i < n; ++i) dphi_dn[ist + i] = -creal(zfi[i]) / g->dsda[ist + i];
    ist += n;
  }
  free(uc); free(ph); free(zf); free(zfi);
}

void eb_or_dirich_neu_map(const eb_or_geom* g, const double* u, double* phi, double* psi,
                          double* dphi_dn, int nthreads) {
  dirich_neu_map_impl(g, u, phi, psi, dphi_dn, EB_OR_DIRECT, nthreads);
}

/* INTERFACENEW, electric.f:791-912 (free space, iwall = 0): interface normal
 * velocity Un from the Stokes density u. */
void eb_or_interfacenew(const eb_or_geom* g, const cplx* ckern, const cplx* zc,
                        double cap, const cplx* u, double* un, double* flux, int mode,
                        int nthreads) {
  int nbk = g->nbk, k = g->k;
  cplx* udot = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  cplx* gw = (cplx*)malloc(sizeof(cplx) * (size_t)nbk);
  double* h = per_point_h(g);
  int ist = 0;
  for (int b = 0; b < k; ++b) {
    eb_or_fdifff(g->nd[b], u + ist, udot + ist);
    ist += g->nd[b];
  }
  /* CADAPMOD with IFLAG2 = iwall (electric.f:828-837) */
  if (mode == EB_OR_CADAP) {
    eb_or_cadap_fmm_w(nbk, g->z, g->dz, h, u, +1, 7, 1e-13, g->iwall, g->xleft, g->slength, gw, nthreads);
  } else {
    eb_or_stokes_direct(nbk, g->z, g->dz, h, u, +1, gw, nthreads);
    if (g->iwall) add_images(g, h, u, +1, gw, nthreads);
  }
  cplx* zb = (cplx*)calloc((size_t)(k > 0 ? k : 1), sizeof(cplx)); /* zb = 0 (electric.f:823) */
  const cplx z2pii = 1.0 / (2.0 * EB_PI * I);
  double fl = 0.0;
  ist = 0;
  for (int b = 0; b < k; ++b) {
    double hb = 2.0 * EB_PI / g->nd[b];
    for (int i = 0; i < g->nd[b]; ++i) {
      int t = ist + i;
      cplx zn = -I * g->dz[t] / g->dsda[t];
      cplx z = g->z[t];
      cplx zcorr = 0.5 * hb * 2.0 * creal(ckern[t]) * u[t] - 2.0 * hb * udot[t];
      zcorr = zcorr * z2pii;
      cplx zself = conj(u[t]) * hb * cabs(g->dz[t]) * 0.5 * g->kappa[t] * zn * zn / EB_PI;
      gw[t] = gw[t] + zself + zcorr;
      cplx zck = 0;
      for (int nb = 0; nb < k; ++nb) {
        cplx zdis = z - g->zk[nb];
        zck = zck + 2.0 * zc[nb] * log(cabs(zdis)) + conj(zc[nb]) * zdis / conj(zdis);
      }
      cplx zphi = 0, zphip = 0, zpsi = -I * 0.5 * cap * z;
      if (g->iwall) eb_or_refsing(z, k, g->zk, zc, zb, &zphi, &zphip, &zpsi);
      cplx gwr = zphi + z * conj(zphip) + conj(zpsi);
      gw[t] = gw[t] + gwr + zck;
      cplx zvel = -I * gw[t];
      un[t] = creal(zvel * conj(zn));
      fl += hb * un[t] * g->dsda[t];
    }
    ist += g->nd[b];
  }
  if (flux) *flux = fl;
  free(udot); free(gw); free(h); free(zb);
}

/* SETVELF, stokesbubb.f:4-135: right-hand side of the Stokes equation, with iwall = 1
 * when zbond != 0 (READINI, electric.f:321-326). Restated as written, including the
 * electric-stress loop's use of `alpha` left over from the previous loops (:125; its
 * last value is 2 pi (nd_k - 1)/nd_k of the last drop). The C_k loop (:73-102)
 * contributes exactly zero when every zc is zero, and is skipped then. The wall branch
 * (:53-60) subtracts the reflected log sources (REFSING with zb = 0) and then `zstr`,
 * which that branch never assigns (:67): it is taken here as the capillary term of the
 * free-space branch, -conj(-i cap z / 2), the term INTERFACENEW keeps in both cases
 * (electric.f:868-871); the two readings agree when cap = 0. */
void eb_or_setvelf(const eb_or_geom* g, const cplx* zc, cplx zbond, double cap,
                   double e0, const double* dphi_dn, double* rhs) {
  int k = g->k, ndmax = 0;
  for (int b = 0; b < k; ++b) ndmax = g->nd[b] > ndmax ? g->nd[b] : ndmax;
  cplx* zf = (cplx*)malloc(sizeof(cplx) * (size_t)ndmax);
  cplx* zfi = (cplx*)malloc(sizeof(cplx) * (size_t)ndmax);
  int anyzc = 0;
  for (int b = 0; b < k; ++b) if (zc[b] != 0) anyzc = 1;
  cplx* zb0 = (cplx*)calloc((size_t)(k > 0 ? k : 1), sizeof(cplx)); /* zb = 0 (stokesbubb.f:26-28) */
  double alpha = 0.0;
  int ist = 0;
  for (int b = 0; b < k; ++b) {
    int n = g->nd[b];
    for (int i = 0; i < n; ++i)
      zfi[i] = zbond * conj(g->z[ist + i]) * g->dz[ist + i] + conj(zbond) * g->z[ist + i] * g->dz[ist + i];
    eb_or_fft(n, zfi, -1);
    for (int i = 0; i < n; ++i) zfi[i] /= (double)n;
    eb_or_fourint(n, zfi, zf);
    eb_or_fft(n, zf, +1);
    for (int i = 0; i < n; ++i) {
      alpha = 2.0 * EB_PI * (double)i / n;
      cplx zn = -0.5 * g->dz[ist + i] / g->dsda[ist + i];
      cplx zgrav = -I * 0.25 * (alpha * zfi[0] + zf[i]);
      cplx r = zn + zgrav;
      if (zbond != 0) {
        cplx zphi = 0, zphip = 0, zpsi0 = 0, zz = g->z[ist + i];
        eb_or_refsing(zz, k, g->zk, zc, zb0, &zphi, &zphip, &zpsi0);
        r -= zphi - zz * conj(zphip) - conj(zpsi0);
      }
      cplx zpsi = -I * 0.5 * cap * g->z[ist + i];
      cplx zstr = -conj(zpsi);
      r -= zstr;
      rhs[2 * (ist + i)] = creal(r);
      rhs[2 * (ist + i) + 1] = cimag(r);
    }
    if (anyzc) {
      for (int nb = 0; nb < k; ++nb) {
        for (int i = 0; i < n; ++i) zf[i] = (g->z[ist + i] - g->zk[nb]) / cabs(g->z[ist + i] - g->zk[nb]);
        eb_or_fdifff(n, zf, zfi);
        for (int i = 0; i < n; ++i) zf[i] = -I * zfi[i] / zf[i];
        eb_or_fft(n, zf, -1);
        for (int i = 0; i < n; ++i) zf[i] /= (double)n;
        double zf1 = creal(zf[0]);
        eb_or_fourint(n, zf, zfi);
        eb_or_fft(n, zfi, +1);
        cplx d0 = g->z[ist] - g->zk[nb];
        double rad = cabs(d0);
        double arg0 = asin(cimag(d0) / rad);
        if (creal(d0) < 0.0) arg0 = EB_PI - arg0;
        for (int i = 0; i < n; ++i) {
          alpha = 2.0 * EB_PI * (double)i / n;
          double arg = arg0 + alpha * zf1 + creal(zfi[i] - zfi[0]);
          cplx zck = 2.0 * I * zc[nb] * arg - conj(zc[nb]) * cexp(2.0 * I * arg);
          rhs[2 * (ist + i)] -= creal(zck);
          rhs[2 * (ist + i) + 1] -= cimag(zck);
        }
      }
    }
    ist += n;
  }
  ist = 0;
  for (int b = 0; b < k; ++b) {
    int n = g->nd[b];
    for (int i = 0; i < n; ++i) zfi[i] = g->dz[ist + i] * dphi_dn[ist + i] * dphi_dn[ist + i];
    eb_or_fft(n, zfi, -1);
    for (int i = 0; i < n; ++i) zfi[i] /= (double)n;
    cplx zf1 = zfi[0];
    eb_or_fourint(n, zfi, zf);
    eb_or_fft(n, zf, +1);
    for (int i = 0; i < n; ++i) {
      cplx zstr = alpha * zf1 + zf[i] - zf[0];
      zstr = 0.25 * I * e0 * zstr;
      rhs[2 * (ist + i)] += creal(zstr);
      rhs[2 * (ist + i) + 1] += cimag(zstr);
    }
    ist += n;
  }
  free(zf);
  free(zfi);
  free(zb0);
}

/* EQUIT, electric.f:1270-1302: tangential velocity keeping nodes equi-arclength. */
void eb_or_equit(int nd, const double* tha, const double* un, double* t) {
  cplx* zf = (cplx*)malloc(sizeof(cplx) * (size_t)nd);
  cplx* zfi = (cplx*)malloc(sizeof(cplx) * (size_t)nd);
  double dalph = 2.0 * EB_PI / nd;
  for (int i = 0; i < nd; ++i) zf[i] = -tha[i] * un[i];
  eb_or_fft(nd, zf, -1);
  for (int i = 0; i < nd; ++i) zf[i] /= (double)nd;
  zf[nd / 2] = 0;
  double dadt = creal(zf[0]);
  eb_or_fourint(nd, zf, zfi);
  eb_or_fft(nd, zfi, +1);
  for (int i = 0; i < nd; ++i) {
    double alpha = dalph * i;
    t[i] = -creal(zf[0] * alpha + zfi[i]) + alpha * dadt;
  }
  free(zf);
  free(zfi);
}

/* ======================================================================
 * GMRES: SLATEC DGMRES (dgmres.f:413-553) -> DPIGMR (dpigmr.f:242-439) with the
 * settings of SOLVEI / SOLVE_LAPL (stokesbubb.f:330-350, laplace.f:361-382):
 * ITOL = 0, no preconditioner, no scaling, KMP = MAXL, no restart.
 * ====================================================================== */

static double dnrm2(int n, const double* x) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[i] * x[i];
  return sqrt(s);
}
static double ddot(int n, const double* x, const double* y) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}

/* DORTH, dorth.f:90-123: modified Gram-Schmidt with the conditional
 * reorthogonalisation test. hcol receives HES(1..ll, ll). */
static void dorth(int n, double* vnew, const double* v, double* hcol, int ll,
                  double* snormw) {
  double vnrm = dnrm2(n, vnew);
  for (int i = 0; i < ll; ++i) {
    hcol[i] = ddot(n, v + (size_t)i * n, vnew);
    double tem = -hcol[i];
    for (int r = 0; r < n; ++r) vnew[r] += tem * v[(size_t)i * n + r];
  }
  *snormw = dnrm2(n, vnew);
  if (vnrm + 0.001 * (*snormw) != vnrm) return;
  double sumdsq = 0.0;
  for (int i = 0; i < ll; ++i) {
    double tem = -ddot(n, v + (size_t)i * n, vnew);
    if (hcol[i] + 0.001 * tem == hcol[i]) continue;
    hcol[i] -= tem;
    for (int r = 0; r < n; ++r) vnew[r] += tem * v[(size_t)i * n + r];
    sumdsq += tem * tem;
  }
  if (sumdsq == 0.0) return;
  double arg = (*snormw) * (*snormw) - sumdsq;
  *snormw = sqrt(arg > 0.0 ? arg : 0.0);
}

/* DHEQR, dheqr.f:82-176, column update (IJOB > 1; for ll = 1 identical to IJOB = 1). */
static int dheqr_col(double* hes, int ldh, int ll, double* q) {
  double* a = hes + (size_t)(ll - 1) * ldh;
  for (int kk = 0; kk < ll - 1; ++kk) {
    double c = q[2 * kk], s = q[2 * kk + 1];
    double t1 = a[kk], t2 = a[kk + 1];
    a[kk] = c * t1 - s * t2;
    a[kk + 1] = s * t1 + c * t2;
  }
  double t1 = a[ll - 1], t2 = a[ll], c, s;
  if (t2 == 0.0) { c = 1.0; s = 0.0; }
  else if (fabs(t2) >= fabs(t1)) { double t = t1 / t2; s = -1.0 / sqrt(1.0 + t * t); c = -s * t; }
  else { double t = t2 / t1; c = 1.0 / sqrt(1.0 + t * t); s = -c * t; }
  q[2 * (ll - 1)] = c;
  q[2 * (ll - 1) + 1] = s;
  a[ll - 1] = c * t1 - s * t2;
  return a[ll - 1] == 0.0 ? ll : 0;
}

/* DHELS, dhels.f:77-96. */
static void dhels(const double* hes, int ldh, int ll, const double* q, double* b) {
  for (int kk = 0; kk < ll; ++kk) {
    double c = q[2 * kk], s = q[2 * kk + 1];
    double t1 = b[kk], t2 = b[kk + 1];
    b[kk] = c * t1 - s * t2;
    b[kk + 1] = s * t1 + c * t2;
  }
  for (int kb = 0; kb < ll; ++kb) {
    int kk = ll - 1 - kb;
    b[kk] /= hes[(size_t)kk * ldh + kk];
    double t = -b[kk];
    for (int r = 0; r < kk; ++r) b[r] += t * hes[(size_t)kk * ldh + r];
  }
}

int eb_or_gmres(int n, const double* b, double* x, eb_or_matvec_fn mv, void* ud,
                int maxl, double tol, int* iter, double* err) {
  if (maxl > n) maxl = n;
  int ldh = maxl + 1;
  double* v = (double*)malloc(sizeof(double) * (size_t)n * (size_t)(maxl + 1));
  double* hes = (double*)calloc((size_t)ldh * (size_t)maxl, sizeof(double));
  double* q = (double*)calloc(2 * (size_t)maxl, sizeof(double));
  double* y = (double*)calloc((size_t)maxl + 1, sizeof(double));
  double bnrm = dnrm2(n, b);
  mv(n, x, v, ud);
  for (int i = 0; i < n; ++i) v[i] = b[i] - v[i];
  double r0nrm = dnrm2(n, v);
  *iter = 0;
  *err = r0nrm / bnrm;
  int ierr = 0;
  if (*err <= tol) goto done;
  {
    double tem = 1.0 / r0nrm;
    for (int i = 0; i < n; ++i) v[i] *= tem;
    double prod = 1.0, rho = r0nrm, snormw = 0.0;
    int ll, iflag = 1, lgmr = 0;
    for (ll = 1; ll <= maxl; ++ll) {
      lgmr = ll;
      double* vn = v + (size_t)ll * n;
      mv(n, v + (size_t)(ll - 1) * n, vn, ud);
      dorth(n, vn, v, hes + (size_t)(ll - 1) * ldh, ll, &snormw);
      hes[(size_t)(ll - 1) * ldh + ll] = snormw;
      if (dheqr_col(hes, ldh, ll, q) == ll) { iflag = 2; break; }
      prod *= q[2 * (ll - 1) + 1];
      rho = fabs(prod * r0nrm);
      *iter = ll;
      *err = rho / bnrm;
      if (*err <= tol) { iflag = 0; break; }
      if (ll == maxl) break;
      tem = 1.0 / snormw;
      for (int i = 0; i < n; ++i) vn[i] *= tem;
    }
    if (iflag != 0 && iflag != 2) iflag = (rho < r0nrm) ? 1 : 2;
    if (iflag != 2) {
      for (int i = 0; i <= lgmr; ++i) y[i] = 0.0;
      y[0] = r0nrm;
      dhels(hes, ldh, lgmr, q, y);
      for (int i = 0; i < lgmr; ++i)
        for (int r = 0; r < n; ++r) x[r] += y[i] * v[(size_t)i * n + r];
    }
    ierr = iflag;
  }
done:
  free(v); free(hes); free(q); free(y);
  return ierr;
}

/* ======================================================================
 * One stage F and the RK2 (Heun) step
 * ====================================================================== */

typedef struct {
  const eb_or_geom* g;
  int mode, nthreads;
} mv_ud;

static void mv_stokes(int n, const double* x, double* y, void* ud) {
  (void)n;
  mv_ud* m = (mv_ud*)ud;
  eb_or_fasmvp(m->g, x, y, m->mode, m->nthreads);
}
static void mv_lapl(int n, const double* x, double* y, void* ud) {
  (void)n;
  mv_ud* m = (mv_ud*)ud;
  eb_or_fasmvp_lap2(m->g, x, y, m->mode, m->nthreads);
}

/* F, electric.f:968-1109, free space (zbond = 0 keeps iwall = 0). */
void eb_or_f(eb_or_model* m, int k, const int* nd, const double* rku, double* rkup) {
  int nbk = 0, ndmax = 0;
  for (int b = 0; b < k; ++b) { nbk += nd[b]; ndmax = nd[b] > ndmax ? nd[b] : ndmax; }
  size_t nc = (size_t)nbk;
  cplx* z = (cplx*)malloc(sizeof(cplx) * nc);
  cplx* dz = (cplx*)malloc(sizeof(cplx) * nc);
  cplx* ckern = (cplx*)malloc(sizeof(cplx) * nc);
  cplx* zk = (cplx*)malloc(sizeof(cplx) * (size_t)k);
  cplx* zc = (cplx*)malloc(sizeof(cplx) * (size_t)k);
  double* area = (double*)malloc(sizeof(double) * (size_t)k);
  double* tha = (double*)malloc(sizeof(double) * nc);
  double* dsda = (double*)malloc(sizeof(double) * nc);
  double* kappa = (double*)malloc(sizeof(double) * nc);
  double* rhs = (double*)malloc(sizeof(double) * 2 * nc);
  double* soln = (double*)malloc(sizeof(double) * 2 * nc);
  double* ulap = (double*)malloc(sizeof(double) * nc);
  double* phi = (double*)malloc(sizeof(double) * nc);
  double* psi = (double*)malloc(sizeof(double) * nc);
  double* dphi = (double*)malloc(sizeof(double) * nc);
  double* un = (double*)malloc(sizeof(double) * nc);
  double* tt = (double*)malloc(sizeof(double) * (size_t)ndmax);
  cplx* u = (cplx*)malloc(sizeof(cplx) * nc);
  cplx* zf = (cplx*)malloc(sizeof(cplx) * (size_t)ndmax);
  eb_or_extractdat(k, nd, rku, z, zk, dz, tha, dsda, kappa, ckern, area);
  for (int b = 0; b < k; ++b) zc[b] = I * m->zbond * area[b] / (8.0 * EB_PI);
  eb_or_geom g = {k, nd, nbk, z, dz, dsda, kappa, zk, 0, 0.0, 0.0};
  if (m->zbond != 0) { /* wall-bounded (READINI, electric.f:321-326) */
    g.iwall = 1;
    eb_or_wallinfo(nbk, z, &g.xleft, &g.slength);
  }
  mv_ud ud = {&g, m->mode, m->nthreads};
  /* Laplace solve: GETBCs (laplace.f:5-25) then SOLVE_LAPL (x0 = rhs). */
  for (int i = 0; i < nbk; ++i) rhs[i] = -2.0 * creal(z[i]);
  for (int i = 0; i < nbk; ++i) ulap[i] = rhs[i];
  eb_or_gmres(nbk, rhs, ulap, mv_lapl, &ud, m->maxl, m->gmres_tol, &m->lap_iter, &m->lap_err);
  dirich_neu_map_impl(&g, ulap, phi, psi, dphi, m->mode, m->nthreads);
  /* Stokes solve: SETVELF then SOLVEI (x0 = rhs). */
  eb_or_setvelf(&g, zc, m->zbond, m->cap, m->e0, dphi, rhs);
  for (int i = 0; i < 2 * nbk; ++i) soln[i] = rhs[i];
  eb_or_gmres(2 * nbk, rhs, soln, mv_stokes, &ud, m->maxl, m->gmres_tol, &m->stokes_iter,
              &m->stokes_err);
  for (int i = 0; i < nbk; ++i) u[i] = soln[2 * i] + soln[2 * i + 1] * I;
  eb_or_interfacenew(&g, ckern, zc, m->cap, u, un, &m->flux, m->mode, m->nthreads);
  int ist = 0;
  for (int b = 0; b < k; ++b) {
    int n = nd[b];
    eb_or_equit(n, tha + ist, un + ist, tt);
    for (int i = 0; i < n; ++i) {
      zf[i] = -un[ist + i] * I * dz[ist + i] - tt[i] * dz[ist + i];
      zf[i] = zf[i] / dsda[ist + i];
    }
    eb_or_fft(n, zf, -1);
    for (int i = 0; i < n; ++i) zf[i] /= (double)n;
    eb_or_filter(n, zf);
    eb_or_fft(n, zf, +1);
    for (int i = 0; i < n; ++i) {
      rkup[2 * (ist + i)] = creal(zf[i]);
      rkup[2 * (ist + i) + 1] = cimag(zf[i]);
    }
    ist += n;
  }
  free(z); free(dz); free(ckern); free(zk); free(zc); free(area); free(tha); free(dsda);
  free(kappa); free(rhs); free(soln); free(ulap); free(phi); free(psi); free(dphi);
  free(un); free(tt); free(u); free(zf);
}

/* RK2 (modified Euler / Heun), electric.f:762-786. */
void eb_or_rk2(eb_or_model* m, int k, const int* nd, double dt, double* ybar) {
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  int neq = 2 * nbk;
  double* dy = (double*)malloc(sizeof(double) * (size_t)neq);
  double* y = (double*)malloc(sizeof(double) * (size_t)neq);
  double* phi0 = (double*)malloc(sizeof(double) * (size_t)neq);
  eb_or_f(m, k, nd, ybar, dy);
  for (int i = 0; i < neq; ++i) { phi0[i] = dt * dy[i]; y[i] = ybar[i] + phi0[i]; }
  eb_or_f(m, k, nd, y, dy);
  for (int i = 0; i < neq; ++i) ybar[i] = ybar[i] + 0.5 * phi0[i] + 0.5 * (dt * dy[i]);
  free(dy); free(y); free(phi0);
}
