// Complex-variable FMM for the two layer-potential sums of the hot path.
//
//  Stokes (Sherman-Lauricella), what CADAPDR / CADAPMOD compute (cadapdrop2.f,
//  cadap2.f):   GW(z) = phi(z) + s [ z conj(phi'(z)) + conj(psi(z)) ],  s = -1 / +1,
//      phi(z) = sum qa_j/(z_j - z),   psi(z) = sum qb_j/(z_j - z) + qc_j/(z_j - z)^2,
//      qc_j = -conj(z_j) qa_j   (charges of cadapdrop.f:214-222).
//  Cauchy, what DAPIF2 computes with IFLAG7 = 3 (dapif1.f:552-558):
//      F(z_i) = sum_{j != i} q_j/(z_i - z_j) = -phi(z_i).
//
// Differences from the reference's per-level uniform FMM (CADAPDR, which forms
// multipoles from the sources at every level and has no M2M/L2L):
//  * a sparse quadtree with an upward pass (P2M at leaves, M2M) and a downward pass
//    (M2L over the same interaction lists, L2L, L2P);
//  * expansions are stored scaled by the box side r (M_k / r^k, L_m r^m), so every
//    translation operator depends only on the box offset in box units;
//  * psi is kept relative to the expansion centre c: psi_c = psi + conj(c) phi', so
//    that GW = phi + s[(z - c) conj(phi') + conj(psi_c)] involves no cancellation
//    between terms of size |z|. Moving an expansion from centre c to c' adds
//    conj(c' - c) phi' to psi;
//  * M2L uses the scale / binomial / scale factorisation of SLSHIFT
//    (cadap2.f:1149-1215) with the order truncated per offset to what the offset's
//    separation ratio needs for the requested tolerance.
#include <algorithm>
#include <cmath>
#include <vector>

#include "eb_internal.h"

namespace {

__device__ __forceinline__ unsigned int compact2d(unsigned long long x) {
  x &= 0x5555555555555555ull;
  x = (x | (x >> 1)) & 0x3333333333333333ull;
  x = (x | (x >> 2)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x >> 4)) & 0x00FF00FF00FF00FFull;
  x = (x | (x >> 8)) & 0x0000FFFF0000FFFFull;
  x = (x | (x >> 16)) & 0x00000000FFFFFFFFull;
  return (unsigned int)x;
}

__device__ __forceinline__ double2 box_center(unsigned long long key, double x0, double y0,
                                              double r) {
  unsigned int ix = compact2d(key), iy = compact2d(key >> 1);
  return make_double2(x0 + ((double)ix + 0.5) * r, y0 + ((double)iy + 0.5) * r);
}

__device__ __forceinline__ int quadrant(unsigned long long key) {
  return (int)(key & 3ull);  // bit 0: ix & 1, bit 1: iy & 1
}

// ---------------------------------------------------------------------------------
// Charges (sorted order). Stokes: qa, qb of cadapdrop.f:214-222 plus the near-field
// combinations P = qa + s qb, Q = qa - s qb, A = -s conj(qa).
// ---------------------------------------------------------------------------------
template <typename T>
__global__ void k_charges_stokes(int n, const int* __restrict__ perm,
                                 const double2* __restrict__ dens, const double2* __restrict__ dz,
                                 const double* __restrict__ hpt, double s,
                                 c_t<T>* __restrict__ qa, c_t<T>* __restrict__ qb,
                                 c_t<T>* __restrict__ pq, c_t<T>* __restrict__ aa) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int o = perm[i];
  double2 u = dens[o], d = dz[o];
  double h = hpt[o] * (1.0 / (2.0 * EB_PI));
  // 1/(2 pi i) = -i/(2 pi)
  double2 w = cmul<double>(u, d);
  double2 a = make_double2(w.y * h, -w.x * h);
  double2 v = csub<double>(cmul<double>(u, cconj<double>(d)), cmul<double>(cconj<double>(u), d));
  double2 b = make_double2(v.y * h, -v.x * h);
  qa[i] = cmk<T>((T)a.x, (T)a.y);
  qb[i] = cmk<T>((T)b.x, (T)b.y);
  pq[2 * i] = cmk<T>((T)(a.x + s * b.x), (T)(a.y + s * b.y));
  pq[2 * i + 1] = cmk<T>((T)(a.x - s * b.x), (T)(a.y - s * b.y));
  aa[i] = cmk<T>((T)(-s * a.x), (T)(s * a.y));
}

template <typename T>
__global__ void k_charges_cauchy(int n, const int* __restrict__ perm,
                                 const double2* __restrict__ q, c_t<T>* __restrict__ qa) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 v = q[perm[i]];
  qa[i] = cmk<T>((T)v.x, (T)v.y);
}

// ---------------------------------------------------------------------------------
// P2M at the leaves: one warp per leaf, lanes over the leaf's points, one warp
// reduction per coefficient (SLMKXP, cadap2.f:412-468, with scaled coefficients
// and psi relative to the box centre).
// ---------------------------------------------------------------------------------
template <typename T, int E>
__global__ void k_p2m(int off, int nleaf, const unsigned long long* __restrict__ bkey,
                      const int* __restrict__ pt0, const int* __restrict__ pt1,
                      const double2* __restrict__ zs, const c_t<T>* __restrict__ qa,
                      const c_t<T>* __restrict__ qb, double x0, double y0, double r, int p,
                      c_t<T>* __restrict__ mpole) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= nleaf) return;
  int b = off + warp;
  double2 c = box_center(bkey[b], x0, y0, r);
  const T rinv = (T)(1.0 / r);
  c_t<T> acc[2][2];
#pragma unroll
  for (int e = 0; e < 2; ++e)
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) acc[e][sl] = cmk<T>(0, 0);
  int i0 = pt0[b], i1 = pt1[b];
  for (int base = i0; base < i1; base += 32) {
    int i = base + lane;
    c_t<T> w = cmk<T>(0, 0), ah = cmk<T>(0, 0), bh = cmk<T>(0, 0);
    if (i < i1) {
      double2 zi = zs[i];
      w = cmk<T>((T)((zi.x - c.x) / r), (T)((zi.y - c.y) / r));
      ah = cscale<T>(qa[i], rinv);
      if (E == 2) bh = cscale<T>(qb[i], rinv);
    }
    c_t<T> cw = cconj<T>(w);
    c_t<T> cwa = cmul<T>(cw, ah);  // conj(w) a / r
    c_t<T> pw = cmk<T>(1, 0), pwm = cmk<T>(0, 0);
    for (int k = 1; k <= p; ++k) {
      c_t<T> tphi = cmul<T>(ah, pw);
      T s0 = warp_sum<T>(-tphi.x), s1 = warp_sum<T>(-tphi.y);
      int slot = (k - 1) >> 5;
      bool own = ((k - 1) & 31) == lane;
      if (own) {
        if (slot == 0) { acc[0][0].x += s0; acc[0][0].y += s1; }
        else { acc[0][1].x += s0; acc[0][1].y += s1; }
      }
      if (E == 2) {
        c_t<T> tpsi = cmul<T>(bh, pw);
        cfma<T>(tpsi, cscale<T>(cwa, (T)(k - 1)), pwm);
        T s2 = warp_sum<T>(-tpsi.x), s3 = warp_sum<T>(-tpsi.y);
        if (own) {
          if (slot == 0) { acc[1][0].x += s2; acc[1][0].y += s3; }
          else { acc[1][1].x += s2; acc[1][1].y += s3; }
        }
      }
      pwm = pw;
      pw = cmul<T>(pw, w);
    }
  }
#pragma unroll
  for (int sl = 0; sl < 2; ++sl) {
    int kk = lane + 32 * sl;
    if (kk < p) {
#pragma unroll
      for (int e = 0; e < E; ++e) mpole[((size_t)b * E + e) * p + kk] = acc[e][sl];
    }
  }
}

// ---------------------------------------------------------------------------------
// M2M: one warp per parent box, children processed in turn. With e the child centre
// offset in child units and a_k = e^-k M_k:   M'_n = (e/2)^n sum_{k<=n} C(n-1,k-1) a_k.
// psi is first moved to the parent centre: psi_k += conj(e) (k-1) phi_{k-1}.
// ---------------------------------------------------------------------------------
template <typename T, int E>
__global__ void k_m2m(int offp, int nbp, const unsigned long long* __restrict__ bkey,
                      const int* __restrict__ child0, const int* __restrict__ nchild, int p,
                      const T* __restrict__ binom, int ldb, const c_t<T>* __restrict__ epow2,
                      const c_t<T>* __restrict__ einv, c_t<T>* __restrict__ mpole) {
  extern __shared__ unsigned char smem_raw[];
  c_t<T>* sa = reinterpret_cast<c_t<T>*>(smem_raw);
  int wib = threadIdx.x >> 5;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= nbp) return;
  c_t<T>* a = sa + (size_t)wib * E * p;
  int P = offp + warp;
  const int ld = p + 2;
  c_t<T> acc[2][2];
#pragma unroll
  for (int e = 0; e < 2; ++e)
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) acc[e][sl] = cmk<T>(0, 0);
  int c0 = child0[P], nc = nchild[P];
  for (int ci = 0; ci < nc; ++ci) {
    int c = c0 + ci;
    int q = quadrant(bkey[c]);
    c_t<T> ec = epow2[q * ld + 1];
    ec = cscale<T>(ec, (T)2);  // e = 2 (e/2)
    const c_t<T>* mc = mpole + (size_t)c * E * p;
    for (int kk = lane; kk < p; kk += 32) {
      int k = kk + 1;
      c_t<T> sc = einv[q * ld + k];
      a[kk] = cmul<T>(mc[kk], sc);
      if (E == 2) {
        c_t<T> mpsi = mc[p + kk];
        if (k >= 2) cfma<T>(mpsi, cscale<T>(cconj<T>(ec), (T)(k - 1)), mc[kk - 1]);
        a[p + kk] = cmul<T>(mpsi, sc);
      }
    }
    __syncwarp();
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {
      int nn = lane + 32 * sl;
      if (nn < p) {
        int n = nn + 1;
        c_t<T> s0 = cmk<T>(0, 0), s1 = cmk<T>(0, 0);
        const T* brow = binom + (size_t)(n - 1) * ldb;
        for (int k = 1; k <= n; ++k) {
          T cb = brow[k - 1];
          crfma<T>(s0, cb, a[k - 1]);
          if (E == 2) crfma<T>(s1, cb, a[p + k - 1]);
        }
        c_t<T> post = epow2[q * ld + n];
        cfma<T>(acc[0][sl], post, s0);
        if (E == 2) cfma<T>(acc[1][sl], post, s1);
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int sl = 0; sl < 2; ++sl) {
    int nn = lane + 32 * sl;
    if (nn < p) {
#pragma unroll
      for (int e = 0; e < E; ++e) mpole[((size_t)P * E + e) * p + nn] = acc[e][sl];
    }
  }
}

// ---------------------------------------------------------------------------------
// M2L over the interaction lists of every box of levels >= 2 (one launch for all
// levels): one warp per target box. For offset d = (c_t - c_s)/r,
//   a_k = M_k d^-k,  L_m += (-1)^m d^-m sum_k C(m+k-1, m) a_k,
// with k, m <= pd(d). psi is first moved to the target centre:
//   psi_k -= conj(d) (k-1) phi_{k-1}.
// ---------------------------------------------------------------------------------
template <typename T, int E>
__global__ void __launch_bounds__(128) k_m2l(int first, int ntarget, const int* __restrict__ vlist,
                      const unsigned char* __restrict__ vcode, const int* __restrict__ vcount,
                      int p, const T* __restrict__ binom, int ldb,
                      const c_t<T>* __restrict__ dinv, const int* __restrict__ pdv,
                      const c_t<T>* __restrict__ mpole, c_t<T>* __restrict__ local) {
  extern __shared__ unsigned char smem_raw[];
  // C2[(k-1)*(p+1) + m] = C(m+k-1, m), k = 1..p, m = 0..p
  T* C2 = reinterpret_cast<T*>(smem_raw);
  const int ldc = p + 1;
  c_t<T>* sa = reinterpret_cast<c_t<T>*>(smem_raw + ((sizeof(T) * (size_t)p * ldc + 15) & ~(size_t)15));
  for (int idx = threadIdx.x; idx < p * ldc; idx += blockDim.x) {
    int k = idx / ldc + 1, m = idx % ldc;
    C2[idx] = binom[(size_t)(m + k - 1) * ldb + m];
  }
  __syncthreads();
  int wib = threadIdx.x >> 5;
  int lane = threadIdx.x & 31;
  int t = blockIdx.x * (blockDim.x >> 5) + wib;
  if (t >= ntarget) return;
  int gid = first + t;
  c_t<T>* a = sa + (size_t)wib * E * p;
  const int ldd = p + 2;
  c_t<T> acc[2][2];
#pragma unroll
  for (int e = 0; e < 2; ++e)
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) acc[e][sl] = cmk<T>(0, 0);
  int nv = vcount[gid];
  for (int j = 0; j < nv; ++j) {
    int s = vlist[(size_t)gid * EB_VMAX + j];
    int code = vcode[(size_t)gid * EB_VMAX + j];
    int pd = pdv[code];
    const c_t<T>* dv = dinv + (size_t)code * ldd;
    const c_t<T>* ms = mpole + (size_t)s * E * p;
    T dxr = (T)(code % 7 - 3), dyr = (T)(code / 7 - 3);
    for (int kk = lane; kk < pd; kk += 32) {
      int k = kk + 1;
      c_t<T> sc = dv[k];
      a[kk] = cmul<T>(ms[kk], sc);
      if (E == 2) {
        c_t<T> mpsi = ms[p + kk];
        // psi_k -= conj(d) (k-1) phi_{k-1}
        if (k >= 2) cfma<T>(mpsi, cmk<T>(-dxr * (T)(k - 1), dyr * (T)(k - 1)), ms[kk - 1]);
        a[p + kk] = cmul<T>(mpsi, sc);
      }
    }
    __syncwarp();
#pragma unroll
    for (int sl = 0; sl < 2; ++sl) {
      int m = lane + 32 * sl;
      if (m <= pd) {
        c_t<T> b0 = cmk<T>(0, 0), b1 = cmk<T>(0, 0);
        const T* col = C2 + m;
#pragma unroll 4
        for (int k = 1; k <= pd; ++k) {
          T cb = col[(k - 1) * ldc];
          crfma<T>(b0, cb, a[k - 1]);
          if (E == 2) crfma<T>(b1, cb, a[p + k - 1]);
        }
        c_t<T> post = dv[m];
        if (m & 1) post = cmk<T>(-post.x, -post.y);
        cfma<T>(acc[0][sl], post, b0);
        if (E == 2) cfma<T>(acc[1][sl], post, b1);
      }
    }
    __syncwarp();
  }
  const int ldl = p + 1;
#pragma unroll
  for (int sl = 0; sl < 2; ++sl) {
    int m = lane + 32 * sl;
    if (m <= p) {
#pragma unroll
      for (int e = 0; e < E; ++e) local[((size_t)gid * E + e) * ldl + m] = acc[e][sl];
    }
  }
}

// ---------------------------------------------------------------------------------
// L2L: one warp per child box. With e the child offset in child units and
// a_m = (e/2)^m L_m:   L'_j += e^-j sum_{m>=j} C(m, j) a_m.
// psi is first moved to the child centre: psi_m += conj(e/2) (m+1) phi_{m+1}.
// ---------------------------------------------------------------------------------
template <typename T, int E>
__global__ void k_l2l(int offc, int nbc, const unsigned long long* __restrict__ bkey,
                      const int* __restrict__ parent, int p, const T* __restrict__ binom,
                      int ldb, const c_t<T>* __restrict__ epow2, const c_t<T>* __restrict__ einv,
                      c_t<T>* __restrict__ local) {
  extern __shared__ unsigned char smem_raw[];
  c_t<T>* sa = reinterpret_cast<c_t<T>*>(smem_raw);
  int wib = threadIdx.x >> 5;
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= nbc) return;
  const int ldl = p + 1, ld = p + 2;
  c_t<T>* a = sa + (size_t)wib * E * ldl;
  int c = offc + warp;
  int P = parent[c];
  int q = quadrant(bkey[c]);
  c_t<T> eh = epow2[q * ld + 1];  // e/2
  const c_t<T>* lp = local + (size_t)P * E * ldl;
  for (int m = lane; m <= p; m += 32) {
    c_t<T> sc = epow2[q * ld + m];
    a[m] = cmul<T>(lp[m], sc);
    if (E == 2) {
      c_t<T> lpsi = lp[ldl + m];
      if (m < p) cfma<T>(lpsi, cscale<T>(cconj<T>(eh), (T)(m + 1)), lp[m + 1]);
      a[ldl + m] = cmul<T>(lpsi, sc);
    }
  }
  __syncwarp();
  c_t<T>* lc = local + (size_t)c * E * ldl;
  for (int j = lane; j <= p; j += 32) {
    c_t<T> s0 = cmk<T>(0, 0), s1 = cmk<T>(0, 0);
    for (int m = j; m <= p; ++m) {
      T cb = binom[(size_t)m * ldb + j];
      crfma<T>(s0, cb, a[m]);
      if (E == 2) crfma<T>(s1, cb, a[ldl + m]);
    }
    c_t<T> post = einv[q * ld + j];
    c_t<T> v0 = lc[j];
    cfma<T>(v0, post, s0);
    lc[j] = v0;
    if (E == 2) {
      c_t<T> v1 = lc[ldl + j];
      cfma<T>(v1, post, s1);
      lc[ldl + j] = v1;
    }
  }
}

// ---------------------------------------------------------------------------------
// Leaf evaluation, FP64: L2P plus the near field over the U list (SLSELFDR/SLDIRDR,
// cadapdrop2.f:564-620, 724-769; DABARR's pair loop, dapif3.f:460-545).
// One warp per leaf, one lane per target point; source data are broadcast loads.
// ---------------------------------------------------------------------------------
template <int E>
__global__ void __launch_bounds__(128) k_leaf64(int off, int nleaf, int has_far,
                         const unsigned long long* __restrict__ bkey,
                         const int* __restrict__ pt0, const int* __restrict__ pt1,
                         const int* __restrict__ ulist, const int* __restrict__ ucount,
                         const int* __restrict__ perm, const double2* __restrict__ zs,
                         const double2* __restrict__ pq, const double2* __restrict__ aa,
                         const double2* __restrict__ qa, double x0, double y0, double r,
                         int p, double s, const double2* __restrict__ local,
                         double2* __restrict__ out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= nleaf) return;
  int b = off + warp;
  double2 c = box_center(bkey[b], x0, y0, r);
  int i0 = pt0[b], i1 = pt1[b];
  int nu = ucount[warp];
  const int ldl = p + 1;
  const double2* lb = local + (size_t)b * E * ldl;
  for (int base = i0; base < i1; base += 32) {
    int i = base + lane;
    bool act = i < i1;
    int ii = act ? i : i0;
    double2 zi = zs[ii];
    double gx = 0.0, gy = 0.0;
    if (has_far) {
      double2 u = make_double2((zi.x - c.x) / r, (zi.y - c.y) / r);
      double2 phi = lb[p], dphi = make_double2(0.0, 0.0);
      for (int m = p - 1; m >= 0; --m) {
        dphi = cmul<double>(dphi, u);
        dphi = cadd<double>(dphi, phi);
        phi = cmul<double>(phi, u);
        phi = cadd<double>(phi, lb[m]);
      }
      if (E == 2) {
        double2 psi = lb[ldl + p];
        for (int m = p - 1; m >= 0; --m) {
          psi = cmul<double>(psi, u);
          psi = cadd<double>(psi, lb[ldl + m]);
        }
        // GW = phi + s [ u conj(dphi) + conj(psi) ]
        double2 t = cmulc<double>(u, dphi);
        gx = phi.x + s * (t.x + psi.x);
        gy = phi.y + s * (t.y - psi.y);
      } else {
        gx = -phi.x;
        gy = -phi.y;
      }
    }
    for (int jl = 0; jl < nu; ++jl) {
      int sb = ulist[(size_t)warp * EB_UMAX + jl];
      int j0 = pt0[sb], j1 = pt1[sb];
      for (int j = j0; j < j1; ++j) {
        double2 zj = zs[j];
        double dx = zj.x - zi.x, dy = zj.y - zi.y;
        double d2 = fma(dx, dx, dy * dy);
        if (j == ii) continue;
        double rr = 1.0 / d2;
        double ix = dx * rr, iy = -dy * rr;  // 1/D
        if (E == 2) {
          double2 P = pq[2 * j], Q = pq[2 * j + 1], A = aa[j];
          // qa/D + s conj(qb/D)
          gx = fma(P.x, ix, fma(-P.y, iy, gx));
          gy = fma(Q.x, iy, fma(Q.y, ix, gy));
          // - s D conj(qa) conj(1/D)^2 = A * D * w^2, w = conj(1/D)
          double w2x = fma(ix, ix, -iy * iy), w2y = -2.0 * ix * iy;
          double tx = fma(dx, w2x, -dy * w2y), ty = fma(dx, w2y, dy * w2x);
          gx = fma(A.x, tx, fma(-A.y, ty, gx));
          gy = fma(A.x, ty, fma(A.y, tx, gy));
        } else {
          double2 q = qa[j];
          // F += q/(z_i - z_j) = -q/D
          gx = fma(-q.x, ix, fma(q.y, iy, gx));
          gy = fma(-q.x, iy, fma(-q.y, ix, gy));
        }
      }
    }
    if (act) out[perm[i]] = make_double2(gx, gy);
  }
}

// Leaf evaluation, FP32: positions as float hi + lo so that differences are exact to
// float precision, Kahan-compensated accumulation of the near-field sum.
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  float y = v - c;
  float t = s + y;
  c = (t - s) - y;
  s = t;
}

template <int E>
__global__ void __launch_bounds__(128) k_leaf32(int off, int nleaf, int has_far,
                         const unsigned long long* __restrict__ bkey,
                         const int* __restrict__ pt0, const int* __restrict__ pt1,
                         const int* __restrict__ ulist, const int* __restrict__ ucount,
                         const int* __restrict__ perm, const double2* __restrict__ zs,
                         const float2* __restrict__ zhi, const float2* __restrict__ zlo,
                         const float2* __restrict__ pq, const float2* __restrict__ aa,
                         const float2* __restrict__ qa, double x0, double y0, double r,
                         int p, float s, const float2* __restrict__ local,
                         double2* __restrict__ out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= nleaf) return;
  int b = off + warp;
  double2 c = box_center(bkey[b], x0, y0, r);
  int i0 = pt0[b], i1 = pt1[b];
  int nu = ucount[warp];
  const int ldl = p + 1;
  const float2* lb = local + (size_t)b * E * ldl;
  for (int base = i0; base < i1; base += 32) {
    int i = base + lane;
    bool act = i < i1;
    int ii = act ? i : i0;
    float2 hi = zhi[ii], lo = zlo[ii];
    float gx = 0.f, gy = 0.f, cx = 0.f, cy = 0.f;
    if (has_far) {
      double2 zi = zs[ii];
      float2 u = make_float2((float)((zi.x - c.x) / r), (float)((zi.y - c.y) / r));
      float2 phi = lb[p], dphi = make_float2(0.f, 0.f);
      for (int m = p - 1; m >= 0; --m) {
        dphi = cadd<float>(cmul<float>(dphi, u), phi);
        phi = cadd<float>(cmul<float>(phi, u), lb[m]);
      }
      if (E == 2) {
        float2 psi = lb[ldl + p];
        for (int m = p - 1; m >= 0; --m) psi = cadd<float>(cmul<float>(psi, u), lb[ldl + m]);
        float2 t = cmulc<float>(u, dphi);
        gx = phi.x + s * (t.x + psi.x);
        gy = phi.y + s * (t.y - psi.y);
      } else {
        gx = -phi.x;
        gy = -phi.y;
      }
    }
    for (int jl = 0; jl < nu; ++jl) {
      int sb = ulist[(size_t)warp * EB_UMAX + jl];
      int j0 = pt0[sb], j1 = pt1[sb];
      for (int j = j0; j < j1; ++j) {
        float2 hj = zhi[j], lj = zlo[j];
        float dx = (hj.x - hi.x) + (lj.x - lo.x);
        float dy = (hj.y - hi.y) + (lj.y - lo.y);
        if (j == ii) continue;
        float d2 = fmaf(dx, dx, dy * dy);
        float rr = __fdividef(1.0f, d2);
        float ix = dx * rr, iy = -dy * rr;
        float tx_, ty_;
        if (E == 2) {
          float2 P = pq[2 * j], Q = pq[2 * j + 1], A = aa[j];
          float w2x = fmaf(ix, ix, -iy * iy), w2y = -2.0f * ix * iy;
          float tx = fmaf(dx, w2x, -dy * w2y), ty = fmaf(dx, w2y, dy * w2x);
          tx_ = fmaf(P.x, ix, fmaf(-P.y, iy, fmaf(A.x, tx, -A.y * ty)));
          ty_ = fmaf(Q.x, iy, fmaf(Q.y, ix, fmaf(A.x, ty, A.y * tx)));
        } else {
          float2 q = qa[j];
          tx_ = fmaf(-q.x, ix, q.y * iy);
          ty_ = fmaf(-q.x, iy, -q.y * ix);
        }
        kahan_add(gx, cx, tx_);
        kahan_add(gy, cy, ty_);
      }
    }
    if (act) out[perm[i]] = make_double2((double)gx, (double)gy);
  }
}

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

template <typename T>
int tables_build(EbTables& tb, int p, double tol) {
  tb.p = p;
  const int ldb = 2 * p + 2, ld = p + 2;
  std::vector<T> binom((size_t)ldb * ldb, (T)0);
  std::vector<double> bd((size_t)ldb * ldb, 0.0);
  for (int i = 0; i < ldb; ++i) {
    bd[(size_t)i * ldb] = 1.0;
    for (int j = 1; j <= i; ++j) bd[(size_t)i * ldb + j] = bd[(size_t)(i - 1) * ldb + j - 1] + (j <= i - 1 ? bd[(size_t)(i - 1) * ldb + j] : 0.0);
  }
  for (size_t i = 0; i < bd.size(); ++i) binom[i] = (T)bd[i];
  std::vector<c_t<T>> dinv((size_t)EB_NCODE * ld), epow2((size_t)4 * ld), einv((size_t)4 * ld);
  std::vector<int> pd(EB_NCODE, 0);
  const double rad = std::sqrt(0.5);
  for (int code = 0; code < EB_NCODE; ++code) {
    int dx = code % 7 - 3, dy = code / 7 - 3;
    bool valid = std::abs(dx) >= 2 || std::abs(dy) >= 2;
    double re = 1.0, im = 0.0;  // d^-j
    double dn = (double)dx * dx + (double)dy * dy;
    double ivr = valid ? dx / dn : 0.0, ivi = valid ? -dy / dn : 0.0;
    for (int j = 0; j < ld; ++j) {
      dinv[(size_t)code * ld + j] = cmk<T>((T)(valid ? re : 0.0), (T)(valid ? im : 0.0));
      double nr = re * ivr - im * ivi, ni = re * ivi + im * ivr;
      re = nr;
      im = ni;
    }
    if (valid) {
      double rho = rad / (std::sqrt(dn) - rad);
      int need = (int)std::ceil(std::log(tol) / std::log(rho));
      pd[code] = std::max(2, std::min(p, need));
    }
  }
  for (int q = 0; q < 4; ++q) {
    double er = (q & 1) - 0.5, ei = ((q >> 1) & 1) - 0.5;
    double pr = 1.0, pi = 0.0, vr = 1.0, vi = 0.0;
    double hr = 0.5 * er, hi = 0.5 * ei;
    double en = er * er + ei * ei, ir = er / en, ii = -ei / en;
    for (int j = 0; j < ld; ++j) {
      epow2[(size_t)q * ld + j] = cmk<T>((T)pr, (T)pi);
      einv[(size_t)q * ld + j] = cmk<T>((T)vr, (T)vi);
      double nr = pr * hr - pi * hi, ni = pr * hi + pi * hr;
      pr = nr; pi = ni;
      nr = vr * ir - vi * ii; ni = vr * ii + vi * ir;
      vr = nr; vi = ni;
    }
  }
  EB_TRY(tb.binom.ensure(sizeof(T) * binom.size()));
  EB_TRY(tb.dinv.ensure(sizeof(c_t<T>) * dinv.size()));
  EB_TRY(tb.pd.ensure(sizeof(int) * pd.size()));
  EB_TRY(tb.epow.ensure(sizeof(c_t<T>) * epow2.size()));
  EB_TRY(tb.einv.ensure(sizeof(c_t<T>) * einv.size()));
  EB_CUDA_TRY(cudaMemcpy(tb.binom.p, binom.data(), sizeof(T) * binom.size(), cudaMemcpyHostToDevice));
  EB_CUDA_TRY(cudaMemcpy(tb.dinv.p, dinv.data(), sizeof(c_t<T>) * dinv.size(), cudaMemcpyHostToDevice));
  EB_CUDA_TRY(cudaMemcpy(tb.pd.p, pd.data(), sizeof(int) * pd.size(), cudaMemcpyHostToDevice));
  EB_CUDA_TRY(cudaMemcpy(tb.epow.p, epow2.data(), sizeof(c_t<T>) * epow2.size(), cudaMemcpyHostToDevice));
  EB_CUDA_TRY(cudaMemcpy(tb.einv.p, einv.data(), sizeof(c_t<T>) * einv.size(), cudaMemcpyHostToDevice));
  return EB_OK;
}

struct ProfScope {
  eb_ctx* ctx;
  int cls;
  cudaStream_t st;
  ProfScope(eb_ctx* c, int k, cudaStream_t s) : ctx(c), cls(k), st(s) {
    if (ctx->profiling) cudaEventRecord(ctx->ev0, st);
  }
  void done() {
    if (!ctx->profiling) return;
    cudaEventRecord(ctx->ev1, st);
    cudaEventSynchronize(ctx->ev1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->prof_launch[cls]++;
    ctx->prof_ms[cls] += ms;
  }
};

// Upward pass, M2L and downward pass, shared by both kernels. Leaves the local
// expansions of every box in w.local.
template <typename T, int E>
int fmm_expansions(eb_ctx* ctx, EbTree& t, EbTables& tb, EbFmmWork& w) {
  cudaStream_t st = eb_stream(ctx);
  const int p = tb.p, L = t.L;
  const int ldb = 2 * p + 2;
  EB_TRY(w.mpole.ensure(sizeof(c_t<T>) * (size_t)t.nbox * E * p));
  EB_TRY(w.local.ensure(sizeof(c_t<T>) * (size_t)t.nbox * E * (p + 1)));
  double rleaf = t.W / (double)(1 << L);
  int offL = t.lev_off[L];
  k_p2m<T, E><<<nblk((long long)t.nleaf * 32, 128), 128, 0, st>>>(
      offL, t.nleaf, t.bkey.as<unsigned long long>(), t.pt0.as<int>(), t.pt1.as<int>(),
      t.zs.as<double2>(), w.qa.as<c_t<T>>(), w.qb.as<c_t<T>>(), t.x0, t.y0, rleaf, p,
      w.mpole.as<c_t<T>>());
  eb_count_launch(ctx);
  for (int l = L - 1; l >= 2; --l) {
    int nb = t.lev_off[l + 1] - t.lev_off[l];
    size_t sm = sizeof(c_t<T>) * 4 * E * p;
    k_m2m<T, E><<<nblk((long long)nb * 32, 128), 128, sm, st>>>(
        t.lev_off[l], nb, t.bkey.as<unsigned long long>(), t.child0.as<int>(), t.nchild.as<int>(), p,
        tb.binom.as<T>(), ldb, tb.epow.as<c_t<T>>(), tb.einv.as<c_t<T>>(), w.mpole.as<c_t<T>>());
    eb_count_launch(ctx);
  }
  {
    int first = t.lev_off[2], nt = t.nbox - first;
    size_t c2 = (sizeof(T) * (size_t)p * (p + 1) + 15) & ~(size_t)15;
    size_t sm = c2 + sizeof(c_t<T>) * 4 * E * p;
    if (sm > 48 * 1024)
      EB_CUDA_TRY(cudaFuncSetAttribute(k_m2l<T, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    ProfScope ps(ctx, 1, st);
    k_m2l<T, E><<<nblk(nt, 4), 128, sm, st>>>(first, nt, t.vlist.as<int>(), t.vcode.as<unsigned char>(),
                                              t.vcount.as<int>(), p, tb.binom.as<T>(), ldb,
                                              tb.dinv.as<c_t<T>>(), tb.pd.as<int>(),
                                              w.mpole.as<c_t<T>>(), w.local.as<c_t<T>>());
    eb_count_launch(ctx);
    ps.done();
  }
  for (int l = 3; l <= L; ++l) {
    int nb = t.lev_off[l + 1] - t.lev_off[l];
    size_t sm = sizeof(c_t<T>) * 4 * E * (p + 1);
    k_l2l<T, E><<<nblk((long long)nb * 32, 128), 128, sm, st>>>(
        t.lev_off[l], nb, t.bkey.as<unsigned long long>(), t.parent.as<int>(), p, tb.binom.as<T>(),
        ldb, tb.epow.as<c_t<T>>(), tb.einv.as<c_t<T>>(), w.local.as<c_t<T>>());
    eb_count_launch(ctx);
  }
  return EB_OK;
}

template <typename T, int E>
int fmm_run(eb_ctx* ctx, EbTree& t, int sign, const double2* dens, const double2* dz,
            const double* hpt, const double2* q, double2* out) {
  cudaStream_t st = eb_stream(ctx);
  const bool f64 = sizeof(T) == 8;
  EbTables& tb = f64 ? ctx->tab64 : ctx->tab32;
  EbFmmWork& w = f64 ? ctx->work64 : ctx->work32;
  const int n = t.n;
  EB_TRY(w.qa.ensure(sizeof(c_t<T>) * (size_t)n));
  EB_TRY(w.qb.ensure(sizeof(c_t<T>) * (size_t)n));
  EB_TRY(w.pq.ensure(sizeof(c_t<T>) * 2 * (size_t)n));
  EB_TRY(w.aa.ensure(sizeof(c_t<T>) * (size_t)n));
  if (E == 2) {
    k_charges_stokes<T><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), dens, dz, hpt, (double)sign,
                                                      w.qa.as<c_t<T>>(), w.qb.as<c_t<T>>(),
                                                      w.pq.as<c_t<T>>(), w.aa.as<c_t<T>>());
  } else {
    k_charges_cauchy<T><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), q, w.qa.as<c_t<T>>());
  }
  eb_count_launch(ctx);
  const int has_far = t.L >= 2;
  if (has_far) EB_TRY((fmm_expansions<T, E>(ctx, t, tb, w)));
  else EB_TRY(w.local.ensure(sizeof(c_t<T>) * (size_t)(E * (tb.p + 1))));
  double rleaf = t.W / (double)(1 << t.L);
  int offL = t.lev_off[t.L];
  ProfScope ps(ctx, 0, st);
  if (f64) {
    k_leaf64<E><<<nblk((long long)t.nleaf * 32, 128), 128, 0, st>>>(
        offL, t.nleaf, has_far, t.bkey.as<unsigned long long>(), t.pt0.as<int>(), t.pt1.as<int>(),
        t.ulist.as<int>(), t.ucount.as<int>(), t.perm.as<int>(), t.zs.as<double2>(),
        w.pq.as<double2>(), w.aa.as<double2>(), w.qa.as<double2>(), t.x0, t.y0, rleaf, tb.p,
        (double)sign, w.local.as<double2>(), out);
  } else {
    k_leaf32<E><<<nblk((long long)t.nleaf * 32, 128), 128, 0, st>>>(
        offL, t.nleaf, has_far, t.bkey.as<unsigned long long>(), t.pt0.as<int>(), t.pt1.as<int>(),
        t.ulist.as<int>(), t.ucount.as<int>(), t.perm.as<int>(), t.zs.as<double2>(),
        t.zhi.as<float2>(), t.zlo.as<float2>(), w.pq.as<float2>(), w.aa.as<float2>(),
        w.qa.as<float2>(), t.x0, t.y0, rleaf, tb.p, (float)sign, w.local.as<float2>(), out);
  }
  eb_count_launch(ctx);
  ps.done();
  ctx->last_p = tb.p;
  return eb_check_launch(ctx, "fmm apply");
}

}  // namespace

int eb_tables_init(eb_ctx* ctx) {
  int p64 = ctx->opts.p64, p32 = ctx->opts.p32;
  if (p64 < 2 || p64 > EB_MAX_P || p32 < 2 || p32 > EB_MAX_P) {
    eb_set_last_error_msg("expansion order outside [2, 60]");
    return EB_ERR_TOL;
  }
  EB_TRY(tables_build<double>(ctx->tab64, p64, ctx->opts.tol64));
  EB_TRY(tables_build<float>(ctx->tab32, p32, ctx->opts.tol32));
  return EB_OK;
}

int eb_fmm_apply(eb_ctx* ctx, EbTree& t, int kernel, int sign, int precision,
                 const double2* dens, const double2* dz, const double* hpt, double2* out) {
  if (!t.valid) return EB_ERR_NOGEOM;
  if (kernel != 0) return EB_ERR_ARG;
  if (precision == EB_FP64) return fmm_run<double, 2>(ctx, t, sign, dens, dz, hpt, nullptr, out);
  return fmm_run<float, 2>(ctx, t, sign, dens, dz, hpt, nullptr, out);
}

int eb_fmm_apply_cauchy(eb_ctx* ctx, EbTree& t, int precision, const double2* q, double2* out) {
  if (!t.valid) return EB_ERR_NOGEOM;
  if (precision == EB_FP64) return fmm_run<double, 1>(ctx, t, 0, nullptr, nullptr, nullptr, q, out);
  return fmm_run<float, 1>(ctx, t, 0, nullptr, nullptr, nullptr, q, out);
}
