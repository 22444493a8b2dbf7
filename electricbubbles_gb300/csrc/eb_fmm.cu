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

#include "eb_df.cuh"
#include "eb_internal.h"
#include "eb_post.cuh"

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

// Morton key of the box (x, y) of a level (the even bits hold x)
__device__ __forceinline__ unsigned long long morton_key(unsigned int x, unsigned int y) {
  unsigned long long r = 0;
  for (int b = 0; b < 32; ++b)
    r |= ((unsigned long long)((x >> b) & 1u) << (2 * b)) | ((unsigned long long)((y >> b) & 1u) << (2 * b + 1));
  return r;
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
// Computed in T: the FP32 operator forms its charges in FP32 (GB300's FP64 pipe is ~1/60
// of its FP32 rate). dz = null: the charges of the transposed operator's sum,
// qa = -dens, qb = conj(dens).
template <typename T>
__global__ void k_charges_stokes(int n, const int* __restrict__ perm,
                                 const double2* __restrict__ dens, const double2* __restrict__ dz,
                                 const double* __restrict__ hpt, double sd,
                                 c_t<T>* __restrict__ qa, c_t<T>* __restrict__ qb,
                                 c_t<T>* __restrict__ pq, c_t<T>* __restrict__ aa) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int o = perm[i];
  const double2 ud = dens[o];
  const c_t<T> u = cmk<T>((T)ud.x, (T)ud.y);
  const T s = (T)sd;
  c_t<T> a, b;
  if (dz) {
    const double2 dd = dz[o];
    const c_t<T> d = cmk<T>((T)dd.x, (T)dd.y);
    const T h = (T)hpt[o] * (T)(1.0 / (2.0 * EB_PI));
    // 1/(2 pi i) = -i/(2 pi)
    c_t<T> w = cmul<T>(u, d);
    a = cmk<T>(w.y * h, -w.x * h);
    c_t<T> v = csub<T>(cmul<T>(u, cconj<T>(d)), cmul<T>(cconj<T>(u), d));
    b = cmk<T>(v.y * h, -v.x * h);
  } else {
    a = cmk<T>(-u.x, -u.y);
    b = cconj<T>(u);
  }
  qa[i] = a;
  qb[i] = b;
  pq[2 * i] = cmk<T>(a.x + s * b.x, a.y + s * b.y);
  pq[2 * i + 1] = cmk<T>(a.x - s * b.x, a.y - s * b.y);
  aa[i] = cmk<T>(-s * a.x, s * a.y);
}

__device__ __forceinline__ float4 df4(double2 v) {
  float hx = __double2float_rn(v.x), hy = __double2float_rn(v.y);
  return make_float4(hx, __double2float_rn(v.x - (double)hx), hy, __double2float_rn(v.y - (double)hy));
}

// FP64 charges plus the double-float near-field data P, Q, A scaled by 1/r_leaf, the
// side of the point's own leaf (the near field works in leaf units): 2^lev / W.
__global__ void k_charges_stokes_df(int n, const int* __restrict__ perm, const double2* __restrict__ dens,
                                    const double2* __restrict__ dz, const double* __restrict__ hpt,
                                    double s, double winv, const unsigned char* __restrict__ plev,
                                    float4* __restrict__ qdf, float4* __restrict__ pq, float4* __restrict__ aa) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int o = perm[i];
  const double rinv = ldexp(winv, (int)plev[i]);
  double2 u = dens[o], a, b;
  if (dz) {
    double2 d = dz[o];
    double h = hpt[o] * (1.0 / (2.0 * EB_PI));
    double2 w = cmul<double>(u, d);
    a = make_double2(w.y * h, -w.x * h);
    double2 v = csub<double>(cmul<double>(u, cconj<double>(d)), cmul<double>(cconj<double>(u), d));
    b = make_double2(v.y * h, -v.x * h);
  } else {  // the transposed operator's charges
    a = make_double2(-u.x, -u.y);
    b = cconj<double>(u);
  }
  qdf[2 * i] = df4(make_double2(a.x * rinv, a.y * rinv));
  qdf[2 * i + 1] = df4(make_double2(b.x * rinv, b.y * rinv));
  pq[2 * i] = df4(make_double2((a.x + s * b.x) * rinv, (a.y + s * b.y) * rinv));
  pq[2 * i + 1] = df4(make_double2((a.x - s * b.x) * rinv, (a.y - s * b.y) * rinv));
  aa[i] = df4(make_double2(-s * a.x * rinv, s * a.y * rinv));
}

// Cauchy charge of node o: q[o], or u_o dz_o h_o (FASMVP_LAP, laplace.f:190-200) when
// q is null.
__device__ __forceinline__ double2 cauchy_charge(int o, const double2* q, const double* lu,
                                                 const double2* dz, const double* hpt) {
  if (q) return q[o];
  const double f = lu[o] * hpt[o];
  return make_double2(f * dz[o].x, f * dz[o].y);
}

__global__ void k_charges_cauchy_df(int n, const int* __restrict__ perm, const double2* __restrict__ q,
                                    const double* __restrict__ lu, const double2* __restrict__ dz,
                                    const double* __restrict__ hpt, double winv,
                                    const unsigned char* __restrict__ plev, float4* __restrict__ qdf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double rinv = ldexp(winv, (int)plev[i]);
  double2 v = cauchy_charge(perm[i], q, lu, dz, hpt);
  qdf[i] = df4(make_double2(v.x * rinv, v.y * rinv));
}

template <typename T>
__global__ void k_charges_cauchy(int n, const int* __restrict__ perm,
                                 const double2* __restrict__ q, const double* __restrict__ lu,
                                 const double2* __restrict__ dz, const double* __restrict__ hpt,
                                 c_t<T>* __restrict__ qa) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int o = perm[i];
  if (q) {
    qa[i] = cmk<T>((T)q[o].x, (T)q[o].y);
  } else {
    const T f = (T)lu[o] * (T)hpt[o];
    qa[i] = cmk<T>(f * (T)dz[o].x, f * (T)dz[o].y);
  }
}

// ---------------------------------------------------------------------------------
// 1/x in FP64 for the near field: the hardware reciprocal approximation refined by two
// Newton-Raphson steps r <- r + r (1 - x r), each of which squares the relative error.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ double rcp_nr(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

template <typename T>
__device__ __forceinline__ c_t<T> cpow_int(c_t<T> u, int n) {
  c_t<T> r = cmk<T>(1, 0), b = u;
  while (n > 0) {
    if (n & 1) r = cmul<T>(r, b);
    b = cmul<T>(b, b);
    n >>= 1;
  }
  return r;
}

// ---------------------------------------------------------------------------------
// P2M at the leaves (SLMKXP, cadap2.f:412-468, with scaled coefficients and psi
// relative to the box centre). One block per leaf (of any level): the leaf's points (32 at a time)
// write their powers w^j to shared memory, then thread j forms the power sums
//   A_j = sum a w^j,  B_j = sum b w^j,  C_j = sum conj(w) a w^j   (a = qa/r, b = qb/r)
// and M_phi[k] = -A_{k-1}, M_psi[k] = -(B_{k-1} + (k-1) C_{k-2}).
// ---------------------------------------------------------------------------------
template <typename T, int E>
__global__ void __launch_bounds__(64) k_p2m(const int* __restrict__ leaves,
                                            const unsigned long long* __restrict__ bkey,
                                            const unsigned char* __restrict__ blev,
                                            const int* __restrict__ pt0, const int* __restrict__ pt1,
                                            const double2* __restrict__ zs,
                                            const c_t<T>* __restrict__ qa,
                                            const c_t<T>* __restrict__ qb, double x0, double y0,
                                            double W, int p, c_t<T>* __restrict__ mpole) {
  extern __shared__ unsigned char smem_raw[];
  const int ps = p + 1;  // odd row stride: conflict-free rows
  c_t<T>* pw = reinterpret_cast<c_t<T>*>(smem_raw);
  c_t<T>* sc = pw + 32 * ps;
  const int b = leaves[blockIdx.x];
  int tid = threadIdx.x;
  const double r = ldexp(W, -(int)blev[b]);
  double2 c = box_center(bkey[b], x0, y0, r);
  const T rinv = (T)(1.0 / r);
  c_t<T> A = cmk<T>(0, 0), B = cmk<T>(0, 0), C = cmk<T>(0, 0);
  int i0 = pt0[b], i1 = pt1[b];
  for (int base = i0; base < i1; base += 32) {
    int cnt = min(32, i1 - base);
    __syncthreads();
    if (tid < cnt) {
      int i = base + tid;
      double2 zi = zs[i];
      c_t<T> w = cmk<T>((T)((zi.x - c.x) / r), (T)((zi.y - c.y) / r));
      c_t<T> ah = cscale<T>(qa[i], rinv);
      sc[tid] = ah;
      if (E == 2) {
        sc[32 + tid] = cscale<T>(qb[i], rinv);
        sc[64 + tid] = cmul<T>(cconj<T>(w), ah);
      }
      c_t<T> pwr = cmk<T>(1, 0);
      c_t<T>* row = pw + tid * ps;
      for (int j = 0; j < p; ++j) {
        row[j] = pwr;
        pwr = cmul<T>(pwr, w);
      }
    }
    __syncthreads();
    if (tid < p) {
      for (int s = 0; s < cnt; ++s) {
        c_t<T> v = pw[s * ps + tid];
        cfma<T>(A, sc[s], v);
        if (E == 2) {
          cfma<T>(B, sc[32 + s], v);
          cfma<T>(C, sc[64 + s], v);
        }
      }
    }
  }
  __syncthreads();
  if (tid < p) pw[tid] = C;
  __syncthreads();
  if (tid < p) {
    c_t<T>* mp = mpole + (size_t)b * E * p;
    mp[tid] = cmk<T>(-A.x, -A.y);
    if (E == 2) {
      c_t<T> v = B;
      if (tid >= 1) crfma<T>(v, (T)tid, pw[tid - 1]);
      mp[p + tid] = cmk<T>(-v.x, -v.y);
    }
  }
}

// ---------------------------------------------------------------------------------
// M2M: one block per parent, one thread per output coefficient (e, n). With e the child
// centre offset in child units and a_k = e^-k M_k:  M'_n = (e/2)^n sum_{k<=n} C(n-1,k-1) a_k.
// psi is first moved to the parent centre: psi_k += conj(e) (k-1) phi_{k-1}.
// ---------------------------------------------------------------------------------
template <typename T, int E>
__global__ void k_m2m(int offp, const unsigned long long* __restrict__ bkey,
                      const int* __restrict__ child0, const int* __restrict__ nchild, int p,
                      const T* __restrict__ binom, int ldb, const c_t<T>* __restrict__ epow2,
                      const c_t<T>* __restrict__ einv, c_t<T>* __restrict__ mpole) {
  extern __shared__ unsigned char smem_raw[];
  c_t<T>* a = reinterpret_cast<c_t<T>*>(smem_raw);
  const int P = offp + blockIdx.x, tid = threadIdx.x, ld = p + 2, nout = E * p;
  const int e = tid / p, nn = tid - e * p;
  const bool active = tid < nout;
  c_t<T> acc = cmk<T>(0, 0);
  int c0 = child0[P], nc = nchild[P];
  if (nc == 0) return;  // a leaf: its multipole comes from its points
  for (int ci = 0; ci < nc; ++ci) {
    int c = c0 + ci;
    int q = quadrant(bkey[c]);
    c_t<T> ec = cscale<T>(epow2[q * ld + 1], (T)2);
    const c_t<T>* mc = mpole + (size_t)c * E * p;
    __syncthreads();
    for (int idx = tid; idx < nout; idx += blockDim.x) {
      int e2 = idx / p, kk = idx - e2 * p, k = kk + 1;
      c_t<T> v = mc[idx];
      if (e2 == 1 && k >= 2) cfma<T>(v, cscale<T>(cconj<T>(ec), (T)(k - 1)), mc[kk - 1]);
      a[idx] = cmul<T>(v, einv[q * ld + k]);
    }
    __syncthreads();
    if (active) {
      int n = nn + 1;
      const T* brow = binom + (size_t)(n - 1) * ldb;
      const c_t<T>* ae = a + e * p;
      c_t<T> s0 = cmk<T>(0, 0), s1 = cmk<T>(0, 0);
      int k = 0;
      for (; k + 1 < n; k += 2) {
        crfma<T>(s0, brow[k], ae[k]);
        crfma<T>(s1, brow[k + 1], ae[k + 1]);
      }
      if (k < n) crfma<T>(s0, brow[k], ae[k]);
      cfma<T>(acc, epow2[q * ld + n], cadd<T>(s0, s1));
    }
  }
  if (active) mpole[(size_t)P * E * p + tid] = acc;
}

// ---------------------------------------------------------------------------------
// L2L: one block per child box, one thread per output (e, j). With e the child offset
// in child units and a_m = (e/2)^m L_m:  L'_j += e^-j sum_{m>=j} C(m, j) a_m.
// psi is first moved to the child centre: psi_m += conj(e/2) (m+1) phi_{m+1}.
// ---------------------------------------------------------------------------------
template <typename T, int E>
__global__ void k_l2l(int offc, const unsigned long long* __restrict__ bkey,
                      const int* __restrict__ parent, int p, const T* __restrict__ binom,
                      int ldb, const c_t<T>* __restrict__ epow2, const c_t<T>* __restrict__ einv,
                      c_t<T>* __restrict__ local) {
  extern __shared__ unsigned char smem_raw[];
  c_t<T>* a = reinterpret_cast<c_t<T>*>(smem_raw);
  const int ldl = p + 1, ld = p + 2, nout = E * ldl, tid = threadIdx.x;
  const int c = offc + blockIdx.x;
  const int P = parent[c];
  const int q = quadrant(bkey[c]);
  c_t<T> eh = epow2[q * ld + 1];
  const c_t<T>* lp = local + (size_t)P * nout;
  for (int idx = tid; idx < nout; idx += blockDim.x) {
    int e2 = idx / ldl, m = idx - e2 * ldl;
    c_t<T> v = lp[idx];
    if (e2 == 1 && m < p) cfma<T>(v, cscale<T>(cconj<T>(eh), (T)(m + 1)), lp[m + 1]);
    a[idx] = cmul<T>(v, epow2[q * ld + m]);
  }
  __syncthreads();
  if (tid < nout) {
    int e = tid / ldl, j = tid - e * ldl;
    const c_t<T>* ae = a + e * ldl;
    c_t<T> s0 = cmk<T>(0, 0), s1 = cmk<T>(0, 0);
    int m = j;
    for (; m + 1 <= p; m += 2) {
      crfma<T>(s0, binom[(size_t)m * ldb + j], ae[m]);
      crfma<T>(s1, binom[(size_t)(m + 1) * ldb + j], ae[m + 1]);
    }
    if (m <= p) crfma<T>(s0, binom[(size_t)m * ldb + j], ae[m]);
    c_t<T>* lc = local + (size_t)c * nout;
    c_t<T> v = lc[tid];
    cfma<T>(v, einv[q * ld + j], cadd<T>(s0, s1));
    lc[tid] = v;
  }
}

// ---------------------------------------------------------------------------------
// M2L over the interaction lists of every box of levels >= 2 (one launch for all
// levels). One block per target box; its 4 warps take every 4th entry of the V list
// and accumulate in shared memory, and the 4 partial expansions are added in a fixed
// order at the end. For offset d = (c_t - c_s)/r and a_k = M_k d^-k,
//   L_m += (-1)^m d^-m sum_{k <= pd} C(m+k-1, m) a_k,   m <= pd(d),
// after moving psi to the target centre: psi_k -= conj(d) (k-1) phi_{k-1}.
// The E (pd+1) outputs of a pair are spread over the lanes, up to 3 per lane.
// ---------------------------------------------------------------------------------
template <typename T, int NS>
__device__ __forceinline__ void m2l_slots(int ob, int lane, int nout, int ldo, int pd, int p,
                                          int ldc, const T* C2, const c_t<T>* a,
                                          const c_t<T>* dv, c_t<T>* acc, int ldl) {
  int o[NS], m[NS], e[NS];
  bool v[NS];
  c_t<T> bsum[NS];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    o[sl] = ob + lane + 32 * sl;
    v[sl] = o[sl] < nout;
    e[sl] = v[sl] ? o[sl] / ldo : 0;
    m[sl] = v[sl] ? o[sl] - e[sl] * ldo : 0;
    bsum[sl] = cmk<T>(0, 0);
  }
  for (int k = 0; k < pd; ++k) {
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) crfma<T>(bsum[sl], C2[k * ldc + m[sl]], a[e[sl] * p + k]);
  }
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    if (v[sl]) {
      c_t<T> post = dv[m[sl]];
      if (m[sl] & 1) post = cmk<T>(-post.x, -post.y);
      c_t<T>* ap = acc + e[sl] * ldl + m[sl];
      c_t<T> t = *ap;
      cfma<T>(t, post, bsum[sl]);
      *ap = t;
    }
  }
}

template <typename T, int E>
__global__ void __launch_bounds__(128) k_m2l(int first, const int* __restrict__ vlist,
                                             const unsigned char* __restrict__ vcode,
                                             const int* __restrict__ vcount, int p,
                                             const T* __restrict__ binom, int ldb,
                                             const c_t<T>* __restrict__ dinv,
                                             const int* __restrict__ pdv,
                                             const c_t<T>* __restrict__ mpole,
                                             c_t<T>* __restrict__ local, int accumulate) {
  extern __shared__ unsigned char smem_raw[];
  const int ldc = p + 1, ldl = p + 1, ldd = p + 2;
  // C2[(k-1)*(p+1) + m] = C(m+k-1, m), k = 1..p, m = 0..p
  T* C2 = reinterpret_cast<T*>(smem_raw);
  c_t<T>* sa = reinterpret_cast<c_t<T>*>(smem_raw + ((sizeof(T) * (size_t)p * ldc + 15) & ~(size_t)15));
  c_t<T>* sacc = sa + 4 * E * p;
  for (int idx = threadIdx.x; idx < p * ldc; idx += blockDim.x) {
    int k = idx / ldc + 1, m = idx % ldc;
    C2[idx] = binom[(size_t)(m + k - 1) * ldb + m];
  }
  for (int idx = threadIdx.x; idx < 4 * E * ldl; idx += blockDim.x) sacc[idx] = cmk<T>(0, 0);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = first + blockIdx.x;
  c_t<T>* a = sa + w * E * p;
  c_t<T>* acc = sacc + w * E * ldl;
  const int nv = vcount[gid];
  for (int j = w; j < nv; j += 4) {
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
        if (k >= 2) cfma<T>(mpsi, cmk<T>(-dxr * (T)(k - 1), dyr * (T)(k - 1)), ms[kk - 1]);
        a[p + kk] = cmul<T>(mpsi, sc);
      }
    }
    __syncwarp();
    const int ldo = pd + 1, nout = E * ldo;
    for (int ob = 0; ob < nout; ob += 96) {
      int rem = nout - ob;
      if (rem > 64) m2l_slots<T, 3>(ob, lane, nout, ldo, pd, p, ldc, C2, a, dv, acc, ldl);
      else if (rem > 32) m2l_slots<T, 2>(ob, lane, nout, ldo, pd, p, ldc, C2, a, dv, acc, ldl);
      else m2l_slots<T, 1>(ob, lane, nout, ldo, pd, p, ldc, C2, a, dv, acc, ldl);
    }
    __syncwarp();
  }
  __syncthreads();
  const int tot = E * ldl;
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    c_t<T> v = cadd<T>(cadd<T>(sacc[idx], sacc[tot + idx]), cadd<T>(sacc[2 * tot + idx], sacc[3 * tot + idx]));
    if (accumulate) v = cadd<T>(local[(size_t)gid * tot + idx], v);
    local[(size_t)gid * tot + idx] = v;
  }
}

// The FP32 M2L for the default order P (20): lane m <= P owns output order m of both
// expansions. Its binomial column C(m+k-1, m) stays in registers, the warp's entries are
// accumulated in registers, the loops over k run to P with a_k = 0 beyond the entry's
// truncation order pd, and outputs m > pd are skipped, so each entry gives exactly the
// sums of k_m2l (same terms, same order).
template <int E, int P>
__global__ void __launch_bounds__(128) k_m2l_f32p(int first, const int* __restrict__ vlist,
                                                  const unsigned char* __restrict__ vcode,
                                                  const int* __restrict__ vcount,
                                                  const float* __restrict__ binom, int ldb,
                                                  const float2* __restrict__ dinv,
                                                  const int* __restrict__ pdv,
                                                  const float2* __restrict__ mpole,
                                                  float2* __restrict__ local, int accumulate) {
  constexpr int ldl = P + 1, ldd = P + 2;
  __shared__ float2 sa[4][E][P];
  __shared__ float2 sred[4][E][ldl];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = first + blockIdx.x;
  const int nv = vcount[gid];
  const int m = lane <= P ? lane : P;
  float c2[P];
#pragma unroll
  for (int k = 1; k <= P; ++k) c2[k - 1] = binom[(size_t)(m + k - 1) * ldb + m];
  float2 acc[E];
#pragma unroll
  for (int e = 0; e < E; ++e) acc[e] = make_float2(0.f, 0.f);
  for (int j = w; j < nv; j += 4) {
    const int src = vlist[(size_t)gid * EB_VMAX + j];
    const int code = vcode[(size_t)gid * EB_VMAX + j];
    const int pd = pdv[code];
    const float2* dv = dinv + (size_t)code * ldd;
    const float2* ms = mpole + (size_t)src * E * P;
    if (lane < P) {
      const int kk = lane, k = kk + 1;
      float2 v0 = make_float2(0.f, 0.f), v1 = v0;
      if (kk < pd) {
        const float2 sc = dv[k];
        v0 = cmul<float>(ms[kk], sc);
        if (E == 2) {
          float2 mpsi = ms[P + kk];
          const float dxr = (float)(code % 7 - 3), dyr = (float)(code / 7 - 3);
          if (k >= 2) cfma<float>(mpsi, make_float2(-dxr * (float)(k - 1), dyr * (float)(k - 1)), ms[kk - 1]);
          v1 = cmul<float>(mpsi, sc);
        }
      }
      sa[w][0][kk] = v0;
      if (E == 2) sa[w][1][kk] = v1;
    }
    __syncwarp();
    if (lane <= pd) {
      float2 post = dv[m];
      if (m & 1) post = make_float2(-post.x, -post.y);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        float2 b = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < P; ++k) crfma<float>(b, c2[k], sa[w][e][k]);
        cfma<float>(acc[e], post, b);
      }
    }
    __syncwarp();
  }
  if (lane <= P) {
#pragma unroll
    for (int e = 0; e < E; ++e) sred[w][e][lane] = acc[e];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < E * ldl; idx += blockDim.x) {
    const int e = idx / ldl, mm = idx - e * ldl;
    float2 v = cadd<float>(cadd<float>(sred[0][e][mm], sred[1][e][mm]), cadd<float>(sred[2][e][mm], sred[3][e][mm]));
    if (accumulate) v = cadd<float>(local[(size_t)gid * E * ldl + idx], v);
    local[(size_t)gid * E * ldl + idx] = v;
  }
}

// ---------------------------------------------------------------------------------
// The same M2L in double-float arithmetic (FP64-class accuracy on the FP32 pipes): the
// multipoles, d^-j and binomial tables are double-float; each output's binomial sum is
// accumulated with compensation; the four warps' partial expansions are added in a
// fixed order and written as FP64.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ cdf cdf_ld(const float4* p) { return cdf_from_float4(*p); }
__device__ __forceinline__ float4 cdf_f4(cdf v) { return make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo); }

template <int NS>
__device__ __forceinline__ void m2l_slots_df(int ob, int lane, int nout, int ldo, int pd, int p, int ldc,
                                             const float2* C2, const float4* a, const float4* dv,
                                             float4* acc, int ldl) {
  int o[NS], m[NS], e[NS];
  bool v[NS];
  dfacc bx[NS], by[NS];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    o[sl] = ob + lane + 32 * sl;
    v[sl] = o[sl] < nout;
    e[sl] = v[sl] ? o[sl] / ldo : 0;
    m[sl] = v[sl] ? o[sl] - e[sl] * ldo : 0;
    bx[sl] = dfacc{0.f, 0.f};
    by[sl] = dfacc{0.f, 0.f};
  }
  for (int k = 0; k < pd; ++k) {
#pragma unroll
    for (int sl = 0; sl < NS; ++sl) {
      const float2 c = C2[k * ldc + m[sl]];
      const float4 av = a[e[sl] * p + k];
      acc_prod(bx[sl], dfl{c.x, c.y}, dfl{av.x, av.y});
      acc_prod(by[sl], dfl{c.x, c.y}, dfl{av.z, av.w});
    }
  }
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    if (v[sl]) {
      cdf post = cdf_ld(dv + m[sl]);
      if (m[sl] & 1) post = cdf{dfl_neg(post.x), dfl_neg(post.y)};
      float4* ap = acc + e[sl] * ldl + m[sl];
      *ap = cdf_f4(cdf_add(cdf_from_float4(*ap), cdf_mul(post, cdf{acc_value(bx[sl]), acc_value(by[sl])})));
    }
  }
}

template <int E>
__global__ void __launch_bounds__(128) k_m2l_df(int first, const int* __restrict__ vlist,
                                                const unsigned char* __restrict__ vcode,
                                                const int* __restrict__ vcount, int p,
                                                const float2* __restrict__ binom, int ldb,
                                                const float4* __restrict__ dinv,
                                                const int* __restrict__ pdv,
                                                const float4* __restrict__ mpole,
                                                float4* __restrict__ local, int accumulate) {
  extern __shared__ float4 smem_f4[];
  const int ldc = p + 1, ldl = p + 1, ldd = p + 2;
  float2* C2 = reinterpret_cast<float2*>(smem_f4);
  float4* sa = smem_f4 + (p * ldc + 1) / 2;
  float4* sacc = sa + 4 * E * p;
  for (int idx = threadIdx.x; idx < p * ldc; idx += blockDim.x) {
    int k = idx / ldc + 1, m = idx % ldc;
    C2[idx] = binom[(size_t)(m + k - 1) * ldb + m];
  }
  for (int idx = threadIdx.x; idx < 4 * E * ldl; idx += blockDim.x) sacc[idx] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = first + blockIdx.x;
  float4* a = sa + w * E * p;
  float4* acc = sacc + w * E * ldl;
  const int nv = vcount[gid];
  for (int j = w; j < nv; j += 4) {
    const int s = vlist[(size_t)gid * EB_VMAX + j];
    const int code = vcode[(size_t)gid * EB_VMAX + j];
    const int pd = pdv[code];
    const float4* dv = dinv + (size_t)code * ldd;
    const float4* ms = mpole + (size_t)s * E * p;
    const float dxr = (float)(code % 7 - 3), dyr = (float)(code / 7 - 3);
    for (int kk = lane; kk < pd; kk += 32) {
      const int k = kk + 1;
      const cdf sc = cdf_ld(dv + k);
      a[kk] = cdf_f4(cdf_mul(cdf_ld(ms + kk), sc));
      if (E == 2) {
        cdf mpsi = cdf_ld(ms + p + kk);
        if (k >= 2) {
          const cdf f = cdf{{-dxr * (float)(k - 1), 0.f}, {dyr * (float)(k - 1), 0.f}};
          mpsi = cdf_add(mpsi, cdf_mul(f, cdf_ld(ms + kk - 1)));
        }
        a[p + kk] = cdf_f4(cdf_mul(mpsi, sc));
      }
    }
    __syncwarp();
    const int ldo = pd + 1, nout = E * ldo;
    for (int ob = 0; ob < nout; ob += 96) {
      int rem = nout - ob;
      if (rem > 64) m2l_slots_df<3>(ob, lane, nout, ldo, pd, p, ldc, C2, a, dv, acc, ldl);
      else if (rem > 32) m2l_slots_df<2>(ob, lane, nout, ldo, pd, p, ldc, C2, a, dv, acc, ldl);
      else m2l_slots_df<1>(ob, lane, nout, ldo, pd, p, ldc, C2, a, dv, acc, ldl);
    }
    __syncwarp();
  }
  __syncthreads();
  const int tot = E * ldl;
  for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
    cdf v01 = cdf_add(cdf_from_float4(sacc[idx]), cdf_from_float4(sacc[tot + idx]));
    cdf v23 = cdf_add(cdf_from_float4(sacc[2 * tot + idx]), cdf_from_float4(sacc[3 * tot + idx]));
    cdf v = cdf_add(v01, v23);
    if (accumulate) v = cdf_add(cdf_from_float4(local[(size_t)gid * tot + idx]), v);
    local[(size_t)gid * tot + idx] = cdf_f4(v);
  }
}

// ---------------------------------------------------------------------------------
// Upward and downward passes of the double-float pipeline: the P2M, M2M and L2L of the
// FP64 kernels above with double-float operands and compensated sums.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ cdf cdf_conj(cdf a) { return cdf{a.x, dfl_neg(a.y)}; }
__device__ __forceinline__ cdf cdf_scale(cdf a, float f) { return cdf{dfl_mul_f(a.x, f), dfl_mul_f(a.y, f)}; }

// acc += a * b (complex) with compensated real and imaginary sums
__device__ __forceinline__ void cacc_mul(dfacc& rx, dfacc& ry, cdf a, cdf b) {
  acc_prod(rx, a.x, b.x);
  acc_prod(rx, dfl_neg(a.y), b.y);
  acc_prod(ry, a.x, b.y);
  acc_prod(ry, a.y, b.x);
}

// acc += c * a (c real)
__device__ __forceinline__ void cacc_rmul(dfacc& rx, dfacc& ry, dfl c, cdf a) {
  acc_prod(rx, c, a.x);
  acc_prod(ry, c, a.y);
}

__device__ __forceinline__ cdf cacc_value(const dfacc& rx, const dfacc& ry) {
  return cdf{acc_value(rx), acc_value(ry)};
}

// P2M at the leaves from the leaf-relative offsets w (units of the leaf side) and the
// charges qa/r, qb/r: M_phi[k] = -A_{k-1}, M_psi[k] = -(B_{k-1} + (k-1) C_{k-2}).
template <int E>
__global__ void k_p2m_df(const int* __restrict__ leaves, const int* __restrict__ pt0, const int* __restrict__ pt1,
                         const float4* __restrict__ wa, const float4* __restrict__ q, int p,
                         float4* __restrict__ mpole) {
  // thread (which, k) < NA p sums one of A_k, B_k, C_k over the leaf's points
  constexpr int NA = E == 2 ? 3 : 1;
  extern __shared__ float4 sm4[];
  const int ps = p + 1;
  float4* pw = sm4;
  float4* sc = pw + 32 * ps;
  const int b = leaves[blockIdx.x], tid = threadIdx.x;
  const int which = tid / p, kq = tid - which * p;
  const bool acc_thread = which < NA;
  dfacc Rx{0.f, 0.f}, Ry{0.f, 0.f};
  const int i0 = pt0[b], i1 = pt1[b];
  for (int base = i0; base < i1; base += 32) {
    const int cnt = min(32, i1 - base);
    __syncthreads();
    if (tid < cnt) {
      const int i = base + tid;
      const float4 wv = wa[i];
      const cdf w = cdf{{wv.x, wv.z}, {wv.y, wv.w}};
      const cdf ah = cdf_from_float4(q[(size_t)E * i]);
      sc[tid] = cdf_f4(ah);
      if (E == 2) {
        sc[32 + tid] = q[2 * (size_t)i + 1];
        sc[64 + tid] = cdf_f4(cdf_mul(cdf_conj(w), ah));
      }
      float4* row = pw + tid * ps;
      row[0] = make_float4(1.f, 0.f, 0.f, 0.f);
      row[1] = cdf_f4(w);
    }
    __syncthreads();
    // powers w^j, j < p, by doubling: w^j = w^(j-len) w^len for len < j <= 2 len, all
    // (point, j) pairs of a step in parallel
    for (int len = 1; len + 1 < p; len <<= 1) {
      const int span = min(len, p - 1 - len);
      for (int pr = tid; pr < cnt * span; pr += blockDim.x) {
        const int sp = pr / span, jj = len + 1 + (pr - sp * span);
        float4* row = pw + sp * ps;
        row[jj] = cdf_f4(cdf_mul(cdf_from_float4(row[jj - len]), cdf_from_float4(row[len])));
      }
      __syncthreads();
    }
    if (acc_thread) {
      const float4* scw = sc + 32 * which;
      for (int s2 = 0; s2 < cnt; ++s2) cacc_mul(Rx, Ry, cdf_from_float4(scw[s2]), cdf_from_float4(pw[s2 * ps + kq]));
    }
  }
  __syncthreads();
  float4* red = pw;  // [NA][p]
  if (acc_thread) red[which * p + kq] = cdf_f4(cacc_value(Rx, Ry));
  __syncthreads();
  if (tid < p) {
    float4* mp = mpole + (size_t)b * E * p;
    const cdf A = cdf_from_float4(red[tid]);
    mp[tid] = cdf_f4(cdf{dfl_neg(A.x), dfl_neg(A.y)});
    if (E == 2) {
      cdf v = cdf_from_float4(red[p + tid]);
      if (tid >= 1) v = cdf_add(v, cdf_scale(cdf_from_float4(red[2 * p + tid - 1]), (float)tid));
      mp[p + tid] = cdf_f4(cdf{dfl_neg(v.x), dfl_neg(v.y)});
    }
  }
}

// merge the compensated complex sums of the 4 lanes of an output (lanes 4o .. 4o+3),
// in a fixed order; every lane ends with the total
__device__ __forceinline__ cdf quad_merge(dfacc rx, dfacc ry) {
  cdf v = cacc_value(rx, ry);
#pragma unroll
  for (int o = 1; o <= 2; o <<= 1) {
    cdf u{{__shfl_xor_sync(0xffffffffu, v.x.hi, o), __shfl_xor_sync(0xffffffffu, v.x.lo, o)},
          {__shfl_xor_sync(0xffffffffu, v.y.hi, o), __shfl_xor_sync(0xffffffffu, v.y.lo, o)}};
    v = (threadIdx.x & o) ? cdf_add(u, v) : cdf_add(v, u);
  }
  return v;
}

// M2M: 4 lanes per output coefficient, each summing every 4th term, so the dependent
// chain of compensated products is a quarter as long.
template <int E>
__global__ void k_m2m_df(int offp, const unsigned long long* __restrict__ bkey,
                         const int* __restrict__ child0, const int* __restrict__ nchild, int p,
                         const float2* __restrict__ binom, int ldb, const float4* __restrict__ epow2,
                         const float4* __restrict__ einv, float4* __restrict__ mpole) {
  extern __shared__ float4 sm4[];
  float4* a = sm4;  // [child][E*p]
  const int P = offp + blockIdx.x, tid = threadIdx.x, ld = p + 2, nout = E * p;
  const int c0 = child0[P], nc = nchild[P];
  if (nc == 0) return;  // a leaf: its multipole comes from its points
  for (int idx = tid; idx < nc * nout; idx += blockDim.x) {
    const int ci = idx / nout, o = idx - ci * nout;
    const int c = c0 + ci, q = quadrant(bkey[c]);
    const int e2 = o / p, kk = o - e2 * p, k = kk + 1;
    const float4* mc = mpole + (size_t)c * nout;
    cdf v = cdf_from_float4(mc[o]);
    if (e2 == 1 && k >= 2) {
      const cdf ec = cdf_scale(cdf_from_float4(epow2[q * ld + 1]), 2.f);
      v = cdf_add(v, cdf_mul(cdf_scale(cdf_conj(ec), (float)(k - 1)), cdf_from_float4(mc[kk - 1])));
    }
    a[idx] = cdf_f4(cdf_mul(v, cdf_from_float4(einv[q * ld + k])));
  }
  __syncthreads();
  const int o = tid >> 2, part = tid & 3;
  const bool act = o < nout;
  const int oo = act ? o : 0;
  const int e = oo / p, n = oo - e * p + 1;
  const float2* brow = binom + (size_t)(n - 1) * ldb;
  dfacc rx{0.f, 0.f}, ry{0.f, 0.f};
  if (act) {
    for (int ci = 0; ci < nc; ++ci) {
      const int q = quadrant(bkey[c0 + ci]);
      const float4* ae = a + ci * nout + e * p;
      dfacc sx{0.f, 0.f}, sy{0.f, 0.f};
      for (int k = part; k < n; k += 4) cacc_rmul(sx, sy, dfl{brow[k].x, brow[k].y}, cdf_from_float4(ae[k]));
      cacc_mul(rx, ry, cdf_from_float4(epow2[q * ld + n]), cacc_value(sx, sy));
    }
  }
  const cdf v = quad_merge(rx, ry);
  if (act && part == 0) mpole[(size_t)P * nout + o] = cdf_f4(v);
}

template <int E>
__global__ void k_l2l_df(int offc, const unsigned long long* __restrict__ bkey,
                         const int* __restrict__ parent, int p, const float2* __restrict__ binom,
                         int ldb, const float4* __restrict__ epow2, const float4* __restrict__ einv,
                         float4* __restrict__ local) {
  extern __shared__ float4 sm4[];
  float4* a = sm4;
  const int ldl = p + 1, ld = p + 2, nout = E * ldl, tid = threadIdx.x;
  const int c = offc + blockIdx.x;
  const int P = parent[c];
  const int q = quadrant(bkey[c]);
  const cdf eh = cdf_from_float4(epow2[q * ld + 1]);
  const float4* lp = local + (size_t)P * nout;
  for (int idx = tid; idx < nout; idx += blockDim.x) {
    const int e2 = idx / ldl, m = idx - e2 * ldl;
    cdf v = cdf_from_float4(lp[idx]);
    if (e2 == 1 && m < p)
      v = cdf_add(v, cdf_mul(cdf_scale(cdf_conj(eh), (float)(m + 1)), cdf_from_float4(lp[m + 1])));
    a[idx] = cdf_f4(cdf_mul(v, cdf_from_float4(epow2[q * ld + m])));
  }
  __syncthreads();
  // 4 lanes per output, each summing every 4th term
  const int o = tid >> 2, part = tid & 3;
  const bool act = o < nout;
  const int oo = act ? o : 0;
  const int e = oo / ldl, j = oo - e * ldl;
  const float4* ae = a + e * ldl;
  dfacc sx{0.f, 0.f}, sy{0.f, 0.f};
  if (act) {
    for (int m = j + part; m <= p; m += 4) {
      const float2 bm = binom[(size_t)m * ldb + j];
      cacc_rmul(sx, sy, dfl{bm.x, bm.y}, cdf_from_float4(ae[m]));
    }
  }
  const cdf ssum = quad_merge(sx, sy);
  if (act && part == 0) {
    float4* lc = local + (size_t)c * nout;
    dfacc rx{0.f, 0.f}, ry{0.f, 0.f};
    const cdf old = cdf_from_float4(lc[o]);
    acc_dfl(rx, old.x);
    acc_dfl(ry, old.y);
    cacc_mul(rx, ry, cdf_from_float4(einv[q * ld + j]), ssum);
    lc[o] = cdf_f4(cacc_value(rx, ry));
  }
}

// ---------------------------------------------------------------------------------
// FP32 multipoles of every box of the finest levels directly from its points, in
// parallel over those levels (no dependent M2M chain): one block per chunk of at most
// EB_CHUNK points forms that chunk's contribution (the P2M sums of SLMKXP,
// cadap2.f:412-468, scaled by the box side and relative to the box centre), and the
// last chunk of a box to finish adds the chunks of the box in order. The offset of a point from an ancestor's centre in the
// ancestor's units is u 2^-sh + (i + 1/2) 2^-sh - (i >> sh) - 1/2 from its leaf offset
// u and leaf grid index i (sh levels between the point's leaf and the box), exact apart
// from the rounding of u.
// ---------------------------------------------------------------------------------
struct LevOff {
  int v[EB_KEY_LEVELS + 2];
  float rinv[EB_KEY_LEVELS + 2];  // 1 / (box side) per level, rounded to float on the host
};

template <int E>
__global__ void __launch_bounds__(128) k_p2m_chunks(LevOff lo, int first2, const unsigned char* __restrict__ blev,
                                                    const unsigned char* __restrict__ plev,
                                                    const int* __restrict__ chunk_box,
                                                    const int* __restrict__ cstart,
                                                    const unsigned long long* __restrict__ keys,
                                                    const int* __restrict__ pt0, const int* __restrict__ pt1,
                                                    const float4* __restrict__ wa, const float2* __restrict__ qa,
                                                    const float2* __restrict__ qb, double W, int p,
                                                    float2* __restrict__ mpart, int* __restrict__ cdone,
                                                    float2* __restrict__ mpole) {
  // Sums per chunk: A_k = sum a w^k, B_k = sum b w^k, C_k = sum conj(w) a w^k (a, b the
  // scaled charges), multipole -A_k and -(B_k + k C_(k-1)).
  constexpr int NA = E == 2 ? 3 : 1;
  extern __shared__ float2 sm2[];
  const int ps = p + 1, nacc = NA * p, nout = E * p;
  float2* pw = sm2;                  // [EB_CHUNK][p + 1]: w^k per point
  float2* sc = pw + EB_CHUNK * ps;   // [NA][EB_CHUNK]: a, b, conj(w) a per point
  float2* red = sc + NA * EB_CHUNK;  // [2][nacc]: the sums over each half of the points
  __shared__ int s_last;
  const int c = blockIdx.x, tid = threadIdx.x;
  const int b = chunk_box[c];
  const int l = blev[b];
  const float rinv = lo.rinv[l];
  const int bb = b - first2, c0 = cstart[bb], nc = cstart[bb + 1] - c0;
  const int i0 = pt0[b] + (c - c0) * EB_CHUNK;
  const int cnt = min(pt1[b], i0 + EB_CHUNK) - i0;
  {
    // two threads per point: even and odd powers
    const int sp = tid >> 1, h = tid & 1;
    if (sp < cnt) {
      const int i = i0 + sp;
      const int lam = plev[i], sh = lam - l;
      const float f = __int_as_float((127 - sh) << 23);  // 2^-sh
      const unsigned long long kl = keys[i] >> (2 * (EB_KEY_LEVELS - lam));
      const unsigned int ix = compact2d(kl), iy = compact2d(kl >> 1);
      const float4 wv = wa[i];
      const float gx = fmaf((float)ix + 0.5f, f, -((float)(ix >> sh) + 0.5f));
      const float gy = fmaf((float)iy + 0.5f, f, -((float)(iy >> sh) + 0.5f));
      const float2 w = make_float2(fmaf(wv.x, f, gx), fmaf(wv.y, f, gy));
      if (h == 0) {
        const float2 ah = cscale<float>(qa[i], rinv);
        sc[sp] = ah;
        if (E == 2) {
          sc[EB_CHUNK + sp] = cscale<float>(qb[i], rinv);
          sc[2 * EB_CHUNK + sp] = cmul<float>(cconj<float>(w), ah);
        }
      }
      const float2 w2 = cmul<float>(w, w);
      float2 cur = h ? w : make_float2(1.f, 0.f);
      float2* row = pw + sp * ps;
      for (int j = h; j < p; j += 2) {
        row[j] = cur;
        cur = cmul<float>(cur, w2);
      }
    }
  }
  __syncthreads();
  {
    const int half = tid >> 6, s0 = half * 32, s1 = min(cnt, s0 + 32);
    for (int o = tid & 63; o < nacc; o += 64) {
      const int which = o / p, k = o - which * p;
      const float2* scw = sc + which * EB_CHUNK;
      float2 acc = make_float2(0.f, 0.f);
      for (int s2 = s0; s2 < s1; ++s2) cfma<float>(acc, scw[s2], pw[s2 * ps + k]);
      red[half * nacc + o] = acc;
    }
  }
  __syncthreads();
  // a box of one chunk gets its multipole directly; otherwise the chunk's part goes to
  // mpart and the box's last chunk to finish adds the parts in chunk order
  float2* dst = nc == 1 ? mpole + (size_t)b * nout : mpart + (size_t)c * nout;
  for (int o = tid; o < nout; o += 128) {
    const int e = o / p, k = o - e * p;
    float2 v = cadd<float>(red[o], red[nacc + o]);
    if (E == 2 && e == 1 && k >= 1) {
      const float2 cm = cadd<float>(red[2 * p + k - 1], red[nacc + 2 * p + k - 1]);
      crfma<float>(v, (float)k, cm);
    }
    dst[o] = make_float2(-v.x, -v.y);
  }
  if (nc == 1) return;
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(&cdone[bb], 1) == nc - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int o = tid; o < nout; o += 128) {
    float2 acc = __ldcg(&mpart[(size_t)c0 * nout + o]);
    for (int cc = c0 + 1; cc < c0 + nc; ++cc) acc = cadd<float>(acc, __ldcg(&mpart[(size_t)cc * nout + o]));
    mpole[(size_t)b * nout + o] = acc;
  }
  if (tid == 0) cdone[bb] = 0;
}

// M2M into the boxes of one level from their children (FP32 coarse levels): all
// children's shifted coefficients are staged in one round of loads, then each output
// sums over the children in their fixed order.
template <int E>
__global__ void k_m2m_f32(int offp, const unsigned long long* __restrict__ bkey,
                          const int* __restrict__ child0, const int* __restrict__ nchild, int p,
                          const float* __restrict__ binom, int ldb, const float2* __restrict__ epow2,
                          const float2* __restrict__ einv, float2* __restrict__ mpole) {
  extern __shared__ float2 sm2[];
  float2* a = sm2;
  const int P = offp + blockIdx.x, tid = threadIdx.x, ld = p + 2, nout = E * p;
  const int c0 = child0[P], nc = nchild[P];
  if (nc == 0) return;  // a leaf: its multipole comes from its points
  for (int idx = tid; idx < nc * nout; idx += blockDim.x) {
    const int ci = idx / nout, o = idx - ci * nout;
    const int c = c0 + ci, q = quadrant(bkey[c]);
    const int e2 = o / p, kk = o - e2 * p, k = kk + 1;
    const float2* mc = mpole + (size_t)c * nout;
    float2 v = mc[o];
    if (e2 == 1 && k >= 2) {
      const float2 ec = cscale<float>(epow2[q * ld + 1], 2.f);
      cfma<float>(v, cscale<float>(cconj<float>(ec), (float)(k - 1)), mc[kk - 1]);
    }
    a[idx] = cmul<float>(v, einv[q * ld + k]);
  }
  __syncthreads();
  if (tid < nout) {
    const int e = tid / p, n = tid - e * p + 1;
    const float* brow = binom + (size_t)(n - 1) * ldb;
    float2 acc = make_float2(0.f, 0.f);
    for (int ci = 0; ci < nc; ++ci) {
      const int q = quadrant(bkey[c0 + ci]);
      const float2* ae = a + ci * nout + e * p;
      float2 s0 = make_float2(0.f, 0.f), s1 = s0;
      int k = 0;
      for (; k + 1 < n; k += 2) {
        crfma<float>(s0, brow[k], ae[k]);
        crfma<float>(s1, brow[k + 1], ae[k + 1]);
      }
      if (k < n) crfma<float>(s0, brow[k], ae[k]);
      cfma<float>(acc, epow2[q * ld + n], cadd<float>(s0, s1));
    }
    mpole[(size_t)P * nout + tid] = acc;
  }
}

// ---------------------------------------------------------------------------------
// Leaf evaluation: L2P plus the near field over the U list (SLSELFDR/SLDIRDR,
// cadapdrop2.f:564-620, 724-769; DABARR's pair loop, dapif3.f:460-545), self excluded.
// One warp per group of up to 8 targets of a leaf; 4 lanes per target split the
// sources (and the terms of the local expansion), and their partial sums are added
// with two shuffles in a fixed order.
// ---------------------------------------------------------------------------------
// Terms m0 <= m < m1 of the local expansions at u.
template <typename T, int E>
__device__ __forceinline__ void l2p_range(const c_t<T>* lb, int p, int m0, int m1, c_t<T> u, T s, T& gx,
                                          T& gy) {
  const int ldl = p + 1;
  if (m0 >= m1) return;
  c_t<T> ph = lb[m1 - 1], dph = cmk<T>(0, 0);
  for (int m = m1 - 2; m >= m0; --m) {
    dph = cadd<T>(cmul<T>(dph, u), ph);
    ph = cadd<T>(cmul<T>(ph, u), lb[m]);
  }
  c_t<T> ps = cmk<T>(0, 0);
  if (E == 2) {
    ps = lb[ldl + m1 - 1];
    for (int m = m1 - 2; m >= m0; --m) ps = cadd<T>(cmul<T>(ps, u), lb[ldl + m]);
  }
  if (m0 > 0) {
    c_t<T> um1 = cpow_int<T>(u, m0 - 1);  // u^(m0-1)
    // d/du (u^m0 H) = u^(m0-1) (u H' + m0 H)
    dph = cmul<T>(um1, cadd<T>(cmul<T>(u, dph), cscale<T>(ph, (T)m0)));
    c_t<T> um = cmul<T>(um1, u);
    ph = cmul<T>(um, ph);
    if (E == 2) ps = cmul<T>(um, ps);
  }
  if (E == 2) {
    c_t<T> t = cmulc<T>(u, dph);
    gx += ph.x + s * (t.x + ps.x);
    gy += ph.y + s * (t.y - ps.y);
  } else {
    gx -= ph.x;
    gy -= ph.y;
  }
}

// Partial far field of lane sl of 4: a quarter of the terms.
template <typename T, int E>
__device__ __forceinline__ void l2p_part(const c_t<T>* lb, int p, int sl, c_t<T> u, T s, T& gx,
                                         T& gy) {
  const int ldl = p + 1, q = (ldl + 3) / 4;
  const int m0 = sl * q, m1 = min(ldl, m0 + q);
  l2p_range<T, E>(lb, p, m0, m1, u, s, gx, gy);
}

// M2P: the far field at u (the target's offset from the box centre in box units) of a
// box's multipole expansions M (phi at M[0, p), psi relative to the centre at M[p, 2p),
// coefficient k at index k - 1): phi = sum_k M_k u^-k, and GW += phi + s (u conj(phi_u) +
// conj(psi)) for Stokes, F -= phi for Cauchy. The evaluation of SLMVALDR
// (cadapdrop2.f:251-301) and DSLOR1 (dapif3.f:1724-1749), used for the W lists.
template <typename T, int E>
__device__ __forceinline__ void m2p_eval(const c_t<T>* M, int p, c_t<T> u, T s, T& gx, T& gy) {
  const c_t<T> v = cinv<T>(u);
  c_t<T> a = M[p - 1];
  c_t<T> da = cscale<T>(M[p - 1], (T)p);
  for (int k = p - 1; k >= 1; --k) {
    a = cadd<T>(cmul<T>(a, v), M[k - 1]);
    if (E == 2) da = cadd<T>(cmul<T>(da, v), cscale<T>(M[k - 1], (T)k));
  }
  const c_t<T> ph = cmul<T>(a, v);  // sum M_k v^k
  if (E == 2) {
    const c_t<T> dph = cmul<T>(da, cmul<T>(v, v));  // sum k M_k v^(k+1) = -phi_u
    c_t<T> b = M[2 * p - 1];
    for (int k = p - 1; k >= 1; --k) b = cadd<T>(cmul<T>(b, v), M[p + k - 1]);
    const c_t<T> ps = cmul<T>(b, v);
    const c_t<T> t = cmulc<T>(u, dph);  // -u conj(phi_u)
    gx += ph.x + s * (ps.x - t.x);
    gy += ph.y - s * (ps.y + t.y);
  } else {
    gx -= ph.x;
    gy -= ph.y;
  }
}

template <int E>
__global__ void __launch_bounds__(128) k_leaf64(int ngroup, const int* __restrict__ gleaf,
                                                const int* __restrict__ gfirst, const int* __restrict__ leaves,
                                                int has_far, const unsigned long long* __restrict__ bkey,
                                                const unsigned char* __restrict__ blev,
                                                const int* __restrict__ pt0, const int* __restrict__ pt1,
                                                const int* __restrict__ ustart, const int* __restrict__ ulist,
                                                const int* __restrict__ wstart, const int* __restrict__ wlist,
                                                const int* __restrict__ perm,
                                                const double2* __restrict__ zs,
                                                const double2* __restrict__ pq,
                                                const double2* __restrict__ aa,
                                                const double2* __restrict__ qa, double x0, double y0,
                                                double W, int p, double s,
                                                const double2* __restrict__ local,
                                                const double2* __restrict__ mpole,
                                                double2* __restrict__ out, EbPost post) {
  int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g >= ngroup) return;
  const int lane = threadIdx.x & 31, tg = lane >> 2, sl = lane & 3;
  const int leaf = gleaf[g], b = leaves[leaf];
  const int i = gfirst[g] + tg;
  const bool act = i < pt1[b];
  const int ii = act ? i : gfirst[g];
  const double2 zi = zs[ii];
  double gx = 0.0, gy = 0.0;
  if (has_far && blev[b] >= 2) {
    const double r = ldexp(W, -(int)blev[b]);
    double2 c = box_center(bkey[b], x0, y0, r);
    double2 u = make_double2((zi.x - c.x) / r, (zi.y - c.y) / r);
    l2p_part<double, E>(local + (size_t)b * E * (p + 1), p, sl, u, s, gx, gy);
  }
  if (has_far) {
    // W list: the lanes of a target take every 4th box
    for (int jw = wstart[leaf] + sl; jw < wstart[leaf + 1]; jw += 4) {
      const int w = wlist[jw];
      const double rw = ldexp(W, -(int)blev[w]);
      const double2 cw = box_center(bkey[w], x0, y0, rw);
      m2p_eval<double, E>(mpole + (size_t)w * E * p, p, make_double2((zi.x - cw.x) / rw, (zi.y - cw.y) / rw),
                          s, gx, gy);
    }
  }
  for (int jl = ustart[leaf]; jl < ustart[leaf + 1]; ++jl) {
    const int sb = ulist[jl];
    const int j1 = pt1[sb];
    for (int j = pt0[sb] + sl; j < j1; j += 4) {
      if (j == ii) continue;
      double2 zj = zs[j];
      double dx = zj.x - zi.x, dy = zj.y - zi.y;
      double rr = rcp_nr(fma(dx, dx, dy * dy));
      double ix = dx * rr, iy = -dy * rr;  // 1/D
      if (E == 2) {
        double2 P = pq[2 * j], Q = pq[2 * j + 1], A = aa[j];
        gx = fma(P.x, ix, fma(-P.y, iy, gx));  // qa/D + s conj(qb/D)
        gy = fma(Q.x, iy, fma(Q.y, ix, gy));
        double w2x = fma(ix, ix, -iy * iy), w2y = -2.0 * ix * iy;  // conj(1/D)^2
        double tx = fma(dx, w2x, -dy * w2y), ty = fma(dx, w2y, dy * w2x);
        gx = fma(A.x, tx, fma(-A.y, ty, gx));  // - s D conj(qa) conj(1/D)^2
        gy = fma(A.x, ty, fma(A.y, tx, gy));
      } else {
        double2 q = qa[j];
        gx = fma(-q.x, ix, fma(q.y, iy, gx));  // q/(z_i - z_j) = -q/D
        gy = fma(-q.x, iy, fma(-q.y, ix, gy));
      }
    }
  }
  gx += __shfl_xor_sync(0xffffffffu, gx, 1);
  gy += __shfl_xor_sync(0xffffffffu, gy, 1);
  gx += __shfl_xor_sync(0xffffffffu, gx, 2);
  gy += __shfl_xor_sync(0xffffffffu, gy, 2);
  if (sl == 0 && act) eb_post_store(post, perm[i], make_double2(gx, gy), out);
}

// ---------------------------------------------------------------------------------
// FP64-accurate leaf evaluation in double-float arithmetic (the same sums as k_leaf64,
// about 2^-47 relative per operation, several times faster on GB300's FP32 pipes).
// Offsets are leaf-relative: for target i in leaf b and source j in neighbour b',
// (z_j - z_i)/r = w_j - (w_i - (b' - b)), exact up to the double-float rounding of w;
// the charges carry the factor 1/r. The local expansions are double-float already.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ cdf cdf_pow(cdf u, int n) {
  cdf r = cdf{{1.f, 0.f}, {0.f, 0.f}}, b = u;
  while (n > 0) {
    if (n & 1) r = cdf_mul(r, b);
    b = cdf_mul(b, b);
    n >>= 1;
  }
  return r;
}

// (hi, mid, lo) - d for a small integer d, renormalised into three floats
__device__ __forceinline__ float3 tf_shift(float hi, float mid, float lo, float d) {
  dfl a = two_sum(hi, -d);
  dfl b = two_sum(mid, a.lo);
  return make_float3(a.hi, b.hi, __fadd_rn(lo, b.lo));
}

// (ah + am + al) - (b.x + b.y + b.z) as a double-float; the hi and mid differences are
// formed exactly, so the result carries the full precision of the three-float inputs.
__device__ __forceinline__ dfl tf_diff(float ah, float am, float al, float3 b) {
  dfl s = two_sum(ah, -b.x);
  dfl t = two_sum(am, -b.y);
  float u = __fadd_rn(__fadd_rn(__fsub_rn(al, b.z), s.lo), t.lo);
  dfl h = two_sum(s.hi, t.hi);
  return fast_two_sum(h.hi, __fadd_rn(h.lo, u));
}

template <int E>
__device__ __forceinline__ void l2p_part_df(const float4* L, int p, int sl, cdf u, bool neg, dfacc& gx,
                                            dfacc& gy) {
  const int ldl = p + 1, q = (ldl + 3) / 4;
  int m0 = sl * q, m1 = min(ldl, m0 + q);
  if (m0 >= m1) return;
  cdf ph = cdf_from_float4(L[m1 - 1]), dph = cdf{{0.f, 0.f}, {0.f, 0.f}};
  for (int m = m1 - 2; m >= m0; --m) {
    dph = cdf_add(cdf_mul(dph, u), ph);
    ph = cdf_add(cdf_mul(ph, u), cdf_from_float4(L[m]));
  }
  cdf ps = cdf{{0.f, 0.f}, {0.f, 0.f}};
  if (E == 2) {
    ps = cdf_from_float4(L[ldl + m1 - 1]);
    for (int m = m1 - 2; m >= m0; --m) ps = cdf_add(cdf_mul(ps, u), cdf_from_float4(L[ldl + m]));
  }
  if (m0 > 0) {
    cdf um1 = cdf_pow(u, m0 - 1);
    cdf t = cdf_add(cdf_mul(u, dph), cdf{dfl_mul_f(ph.x, (float)m0), dfl_mul_f(ph.y, (float)m0)});
    dph = cdf_mul(um1, t);
    cdf um = cdf_mul(um1, u);
    ph = cdf_mul(um, ph);
    if (E == 2) ps = cdf_mul(um, ps);
  }
  if (E == 2) {
    // phi + s (u conj(phi') + conj(psi))
    dfl tx = dfl_add(dfl_mul(u.x, dph.x), dfl_mul(u.y, dph.y));
    dfl ty = dfl_sub(dfl_mul(u.y, dph.x), dfl_mul(u.x, dph.y));
    dfl sx = dfl_add(tx, ps.x), sy = dfl_sub(ty, ps.y);
    if (neg) {
      sx = dfl_neg(sx);
      sy = dfl_neg(sy);
    }
    acc_dfl(gx, ph.x);
    acc_dfl(gx, sx);
    acc_dfl(gy, ph.y);
    acc_dfl(gy, sy);
  } else {
    acc_dfl(gx, dfl_neg(ph.x));
    acc_dfl(gy, dfl_neg(ph.y));
  }
}

// Offset between the centres of a box of level lt (grid index it) and a box of level
// ls = lt + ds (index is), in units of the second box's side: (c_t - c_s) / r_s =
// ((2 it + 1) 2^ds - (2 is + 1)) / 2, formed in integers and exact in float for boxes
// that touch or nearly touch.
__device__ __forceinline__ float box_delta(int it, int is, int ds) {
  long long num;
  int e;
  if (ds >= 0) {
    num = ((2LL * it + 1) << ds) - (2LL * is + 1);
    e = -1;
  } else {
    num = (2LL * it + 1) - ((2LL * is + 1) << (-ds));
    e = ds - 1;
  }
  return ldexpf((float)num, e);
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }

// A target's position relative to the centre of a box ds levels below (ds < 0: above)
// its leaf, in that box's units, as three floats: w 2^ds + (c_leaf - c_box) / r_box.
__device__ __forceinline__ void frame_shift(float4 wa, float2 wb, int ds, int bx, int by, int sx, int sy,
                                            float3& tx, float3& ty) {
  const float f = pow2f(ds);
  tx = tf_shift(wa.x * f, wa.z * f, wb.x * f, -box_delta(bx, sx, ds));
  ty = tf_shift(wa.y * f, wa.w * f, wb.y * f, -box_delta(by, sy, ds));
}

__device__ __forceinline__ dfl tf_to_dfl(float3 t) {
  return dfl_add(two_sum(t.x, t.y), dfl{t.z, 0.f});
}

// M2P in double-float (m2p_eval's sums): M the box's double-float multipoles, u the
// target's offset in box units.
template <int E>
__device__ __forceinline__ void m2p_df(const float4* M, int p, cdf u, bool neg, dfacc& gx, dfacc& gy) {
  const dfl rr = dfl_rcp(dfl_add(dfl_sqr(u.x), dfl_sqr(u.y)));
  const cdf v = cdf{dfl_mul(u.x, rr), dfl_neg(dfl_mul(u.y, rr))};
  cdf a = cdf_from_float4(M[p - 1]);
  cdf da = cdf_scale(a, (float)p);
  for (int k = p - 1; k >= 1; --k) {
    const cdf mk = cdf_from_float4(M[k - 1]);
    a = cdf_add(cdf_mul(a, v), mk);
    if (E == 2) da = cdf_add(cdf_mul(da, v), cdf_scale(mk, (float)k));
  }
  const cdf ph = cdf_mul(a, v);
  if (E == 2) {
    const cdf dph = cdf_mul(da, cdf_mul(v, v));  // -phi_u
    cdf b = cdf_from_float4(M[2 * p - 1]);
    for (int k = p - 1; k >= 1; --k) b = cdf_add(cdf_mul(b, v), cdf_from_float4(M[p + k - 1]));
    const cdf ps = cdf_mul(b, v);
    const dfl tx = dfl_add(dfl_mul(u.x, dph.x), dfl_mul(u.y, dph.y));  // -u conj(phi_u)
    const dfl ty = dfl_sub(dfl_mul(u.y, dph.x), dfl_mul(u.x, dph.y));
    dfl sx = dfl_sub(ps.x, tx), sy = dfl_neg(dfl_add(ps.y, ty));
    if (neg) {
      sx = dfl_neg(sx);
      sy = dfl_neg(sy);
    }
    acc_dfl(gx, ph.x);
    acc_dfl(gx, sx);
    acc_dfl(gy, ph.y);
    acc_dfl(gy, sy);
  } else {
    acc_dfl(gx, dfl_neg(ph.x));
    acc_dfl(gy, dfl_neg(ph.y));
  }
}

// MODE 0: far and near field; 1: near field only, into nearbuf (sorted order);
// 2: far field only, plus nearbuf, then the post-processing. Modes 1 and 2 let the near
// field run concurrently with the expansion passes.
template <int E, int MODE>
__global__ void __launch_bounds__(128) k_leaf_df(int ngroup, const int* __restrict__ gleaf,
                                                 const int* __restrict__ gfirst, const int* __restrict__ leaves,
                                                 int has_far, const unsigned long long* __restrict__ bkey,
                                                 const unsigned char* __restrict__ blev,
                                                 const int* __restrict__ pt0, const int* __restrict__ pt1,
                                                 const int* __restrict__ ustart, const int* __restrict__ ulist,
                                                 const int* __restrict__ wstart, const int* __restrict__ wlist,
                                                 const float4* __restrict__ mpole,
                                                 const int* __restrict__ perm,
                                                 const float4* __restrict__ wa,
                                                 const float2* __restrict__ wb,
                                                 const float4* __restrict__ pq,
                                                 const float4* __restrict__ aa, int p, double s,
                                                 const float4* __restrict__ local,
                                                 double2* __restrict__ out, EbPost post,
                                                 double2* __restrict__ nearbuf) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (g >= ngroup) return;
  const int lane = threadIdx.x & 31, tg = lane >> 2, sl = lane & 3;
  const int leaf = gleaf[g], b = leaves[leaf];
  const int i = gfirst[g] + tg;
  const bool act = i < pt1[b];
  const int ii = act ? i : gfirst[g];
  const float4 wia = wa[ii];
  const float2 wib = wb[ii];
  const cdf wi = cdf{{wia.x, wia.z}, {wia.y, wia.w}};
  const bool neg = s < 0.0;
  const int lt = blev[b];
  dfacc gx{0.f, 0.f}, gy{0.f, 0.f};
  if (MODE != 1 && has_far && lt >= 2) l2p_part_df<E>(local + (size_t)b * E * (p + 1), p, sl, wi, neg, gx, gy);
  const unsigned long long kb = bkey[b];
  const int bx = (int)compact2d(kb), by = (int)compact2d(kb >> 1);
  if (MODE != 1 && has_far) {
    // W list: the lanes of a target take every 4th box
    for (int jw = wstart[leaf] + sl; jw < wstart[leaf + 1]; jw += 4) {
      const int w = wlist[jw];
      const unsigned long long kw = bkey[w];
      float3 tx, ty;
      frame_shift(wia, wib, blev[w] - lt, bx, by, (int)compact2d(kw), (int)compact2d(kw >> 1), tx, ty);
      m2p_df<E>(mpole + (size_t)w * E * p, p, cdf{tf_to_dfl(tx), tf_to_dfl(ty)}, neg, gx, gy);
    }
  }
  const int u0 = ustart[leaf], u1 = MODE == 2 ? u0 : ustart[leaf + 1];
  for (int jl = u0; jl < u1; ++jl) {
    const int sb = ulist[jl];
    const unsigned long long ks = bkey[sb];
    // the target relative to the source leaf's centre, in that leaf's units (three
    // floats); the source charges carry the factor 1 / r of their own leaf
    float3 tx, ty;
    frame_shift(wia, wib, blev[sb] - lt, bx, by, (int)compact2d(ks), (int)compact2d(ks >> 1), tx, ty);
    const int j1 = pt1[sb];
    for (int j = pt0[sb] + sl; j < j1; j += 4) {
      if (j == ii) continue;
      const float4 ja = wa[j];
      const float2 jb = wb[j];
      // D / r = w_j - (w_i - offset): hi and mid parts subtracted exactly
      const dfl dx = tf_diff(ja.x, ja.z, jb.x, tx), dy = tf_diff(ja.y, ja.w, jb.y, ty);
      const dfl rr = dfl_rcp(dfl_add(dfl_sqr(dx), dfl_sqr(dy)));
      const dfl ix = dfl_mul(dx, rr), iy = dfl_neg(dfl_mul(dy, rr));  // 1/D
      if (E == 2) {
        const cdf P = cdf_from_float4(pq[2 * j]), Q = cdf_from_float4(pq[2 * j + 1]);
        const cdf A = cdf_from_float4(aa[j]);
        acc_prod(gx, P.x, ix);  // qa/D + s conj(qb/D)
        acc_prod(gx, dfl_neg(P.y), iy);
        acc_prod(gy, Q.x, iy);
        acc_prod(gy, Q.y, ix);
        const dfl w2x = dfl_mul(dfl_add(ix, iy), dfl_sub(ix, iy));  // conj(1/D)^2
        const dfl ixy = dfl_mul(ix, iy);
        const dfl w2y = dfl{-2.f * ixy.hi, -2.f * ixy.lo};
        const dfl t2x = dfl_sub(dfl_mul(dx, w2x), dfl_mul(dy, w2y));
        const dfl t2y = dfl_add(dfl_mul(dx, w2y), dfl_mul(dy, w2x));
        acc_prod(gx, A.x, t2x);  // - s D conj(qa) conj(1/D)^2
        acc_prod(gx, dfl_neg(A.y), t2y);
        acc_prod(gy, A.x, t2y);
        acc_prod(gy, A.y, t2x);
      } else {
        const cdf q = cdf_from_float4(pq[j]);  // q/(z_i - z_j) = -q/D
        acc_prod(gx, dfl_neg(q.x), ix);
        acc_prod(gx, q.y, iy);
        acc_prod(gy, dfl_neg(q.x), iy);
        acc_prod(gy, dfl_neg(q.y), ix);
      }
    }
  }
  dfl vx = acc_value(gx), vy = acc_value(gy);
#pragma unroll
  for (int o = 1; o <= 2; o <<= 1) {
    dfl ox{__shfl_xor_sync(0xffffffffu, vx.hi, o), __shfl_xor_sync(0xffffffffu, vx.lo, o)};
    dfl oy{__shfl_xor_sync(0xffffffffu, vy.hi, o), __shfl_xor_sync(0xffffffffu, vy.lo, o)};
    vx = (sl & o) ? dfl_add(ox, vx) : dfl_add(vx, ox);
    vy = (sl & o) ? dfl_add(oy, vy) : dfl_add(vy, oy);
  }
  if (sl == 0 && act) {
    double2 v = make_double2(dfl_to_double(vx), dfl_to_double(vy));
    if (MODE == 1) {
      nearbuf[i] = v;
    } else {
      if (MODE == 2) {
        const double2 nv = nearbuf[i];
        v = make_double2(v.x + nv.x, v.y + nv.y);
      }
      eb_post_store(post, perm[i], v, out);
    }
  }
}

// FP32 far field, one block per tile of the near field: the local expansions of the
// leaf and of its nearest ancestors (at most EB_FAR_LEVELS boxes, the coarsest holding
// the L2L-accumulated expansion of the levels above) are staged in shared memory, and
// each expansion is evaluated directly about its own centre at every target (the sum
// equals L2P of the L2L-accumulated leaf expansion). Thread slice sl of 128 / EB_NTILE
// takes every slice-th level, and every slice-th box of the leaf's W list, whose
// multipoles are evaluated at the targets (M2P). Adds the near-field sums of k_near32
// and applies the post-processing.
template <int E>
__global__ void __launch_bounds__(128) k_far32(const int4* __restrict__ tiles, const int* __restrict__ leaves,
                                               const unsigned long long* __restrict__ bkey,
                                               const unsigned char* __restrict__ blev,
                                               const int* __restrict__ anc, const int* __restrict__ wstart,
                                               const int* __restrict__ wlist,
                                               const int* __restrict__ perm,
                                               const float4* __restrict__ wa, int p, float s,
                                               const float2* __restrict__ local,
                                               const float2* __restrict__ mpole,
                                               double2* __restrict__ out, EbPost post,
                                               const double2* __restrict__ nearbuf) {
  constexpr int T = EB_NTILE, NS = 128 / T;
  extern __shared__ float2 sloc[];  // [nf][E][p + 1]
  __shared__ float2 sred[NS][T];
  const int4 tl = tiles[blockIdx.x];
  const int leaf = tl.x, b = leaves[leaf];
  const int tid = threadIdx.x, tt = tid % T, sl = tid / T;
  const int i = tl.y + tt;
  const bool act = i < tl.z;
  const int ii = act ? i : tl.y;
  const int ldl = p + 1, nco = E * ldl;
  const int* fb = anc + (size_t)leaf * EB_FAR_LEVELS;
  int nf = 0;
  while (nf < EB_FAR_LEVELS && fb[nf] >= 0) ++nf;
  for (int idx = tid; idx < nf * nco; idx += 128) {
    const int q = idx / nco, o = idx - q * nco;
    sloc[idx] = local[(size_t)fb[q] * nco + o];
  }
  __syncthreads();
  float fx = 0.f, fy = 0.f;
  const unsigned long long kb = bkey[b];
  const unsigned int ix = compact2d(kb), iy = compact2d(kb >> 1);
  const float4 wv = wa[ii];
  // With u the leaf-scaled offset, the offset scaled to the ancestor sh levels up is
  //   u 2^-sh + (i + 1/2) 2^-sh - (i >> sh) - 1/2   (i the leaf's grid index),
  // whose constant part is exact in FP32 (i < 2^20).
  for (int sh = sl; sh < nf; sh += NS) {
    const float f = __int_as_float((127 - sh) << 23);  // 2^-sh
    const float gx = fmaf((float)ix + 0.5f, f, -((float)(ix >> sh) + 0.5f));
    const float gy = fmaf((float)iy + 0.5f, f, -((float)(iy >> sh) + 0.5f));
    const float2 u = make_float2(fmaf(wv.x, f, gx), fmaf(wv.y, f, gy));
    l2p_range<float, E>(sloc + sh * nco, p, 0, ldl, u, s, fx, fy);
  }
  // W list (boxes below the leaf's level): the target's offset in the box's units is
  // u 2^ds + (c_leaf - c_box) / r_box, the high part of u first, so that the cancelling
  // terms meet exactly, then the middle part
  const int lt = blev[b];
  for (int jw = wstart[leaf] + sl; jw < wstart[leaf + 1]; jw += NS) {
    const int w = wlist[jw];
    const unsigned long long kw = bkey[w];
    const int ds = blev[w] - lt;
    const float f = pow2f(ds);
    const float dx = box_delta((int)ix, (int)compact2d(kw), ds), dy = box_delta((int)iy, (int)compact2d(kw >> 1), ds);
    const float2 u = make_float2(fmaf(wv.z, f, fmaf(wv.x, f, dx)), fmaf(wv.w, f, fmaf(wv.y, f, dy)));
    m2p_eval<float, E>(mpole + (size_t)w * E * p, p, u, s, fx, fy);
  }
  sred[sl][tt] = make_float2(fx, fy);
  __syncthreads();
  if (sl == 0 && act) {
    float2 v = sred[0][tt];
#pragma unroll
    for (int q = 1; q < NS; ++q) {
      v.x += sred[q][tt].x;
      v.y += sred[q][tt].y;
    }
    const double2 nv = nearbuf[i];
    eb_post_store_f32(post, perm[i], make_float2(v.x + (float)nv.x, v.y + (float)nv.y), out);
  }
}

// FP32 near field, one block per tile of up to EB_NTILE (32) targets of one leaf: the
// sources of the leaf's U list (32 boxes at a time) are staged through shared memory in
// slabs of NEAR_SLAB. Each thread holds two targets of the tile (lanes l and l + 16 of
// the tile) and each half-warp takes one of 8 source slices, so every staged source is
// read once per two targets (a broadcast within the half-warp). The slices are added in
// a fixed order. The self pair needs no test: its offset is exactly zero, and with the
// squared distance offset by 1e-36 its terms are exact zeros. Plain FP32 sums: the error
// of the FP32 terms themselves (~1e-6 of the largest) dominates the summation error, so
// compensated sums buy nothing. Writes the near-field sums in sorted order. Positions are
// absolute (float hi + lo), so sources of any level are alike.
#define NEAR_SLAB 256
template <int E>
__device__ __forceinline__ void near_pair(const float4 hlj, const float4 PQ, const float2 A, const float4 hl,
                                          float& gx, float& gy) {
  const float dx = (hlj.x - hl.x) + (hlj.z - hl.z);
  const float dy = (hlj.y - hl.y) + (hlj.w - hl.w);
  const float rr = __fdividef(1.0f, fmaf(dx, dx, fmaf(dy, dy, 1e-36f)));
  const float ix = dx * rr, iy = -dy * rr;  // 1 / (z_s - z_t)
  if (E == 2) {
    const float w2x = fmaf(ix, ix, -iy * iy), w2y = -2.0f * ix * iy;
    const float tx = fmaf(dx, w2x, -dy * w2y), ty = fmaf(dx, w2y, dy * w2x);
    gx = fmaf(PQ.x, ix, fmaf(-PQ.y, iy, fmaf(A.x, tx, fmaf(-A.y, ty, gx))));
    gy = fmaf(PQ.z, iy, fmaf(PQ.w, ix, fmaf(A.x, ty, fmaf(A.y, tx, gy))));
  } else {
    gx = fmaf(-A.x, ix, fmaf(A.y, iy, gx));
    gy = fmaf(-A.x, iy, fmaf(-A.y, ix, gy));
  }
}

template <int E>
__global__ void __launch_bounds__(128, 8) k_near32(const int4* __restrict__ tiles, const int* __restrict__ leaves,
                                                   const int* __restrict__ pt0, const int* __restrict__ pt1,
                                                   const int* __restrict__ ustart, const int* __restrict__ ulist,
                                                   const float4* __restrict__ zhl,
                                                   const float2* __restrict__ pq,
                                                   const float2* __restrict__ aa,
                                                   const float2* __restrict__ qa,
                                                   double2* __restrict__ nearbuf) {
  static_assert(EB_NTILE == 32, "two targets per thread over 16 lanes");
  constexpr int NS = 8;
  __shared__ float4 sz[NEAR_SLAB];
  __shared__ float4 sp[E == 2 ? NEAR_SLAB : 1];
  __shared__ float2 sa[NEAR_SLAB];
  __shared__ int spre[33], sj0[32];
  __shared__ float2 sred[NS][EB_NTILE];
  const int4 tl = tiles[blockIdx.x];
  const int leaf = tl.x;
  const int tid = threadIdx.x, lane = tid & 31;
  const int sl = 2 * (tid >> 5) + (lane >> 4);  // source slice 0..7
  const int t0 = lane & 15;                       // targets t0 and t0 + 16 of the tile
  const int i0 = tl.y + t0, i1 = i0 + 16;
  const float4 h0 = zhl[i0 < tl.z ? i0 : tl.y], h1 = zhl[i1 < tl.z ? i1 : tl.y];
  float gx0 = 0.f, gy0 = 0.f, gx1 = 0.f, gy1 = 0.f;
  const int ub = ustart[leaf], ue = ustart[leaf + 1];
  for (int cb = ub; cb < ue; cb += 32) {
    const int nc = min(32, ue - cb);
    if (cb > ub) __syncthreads();  // the previous boxes' slabs are consumed
    if (tid < 32) {
      int c = 0, j0 = 0;
      if (tid < nc) {
        const int sbx = ulist[cb + tid];
        j0 = pt0[sbx];
        c = pt1[sbx] - j0;
      }
      int x = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (tid >= o) x += y;
      }
      sj0[tid] = j0;
      spre[tid + 1] = x;
      if (tid == 0) spre[0] = 0;
    }
    __syncthreads();
    const int total = spre[nc];
    for (int base = 0; base < total; base += NEAR_SLAB) {
      const int ns = min(NEAR_SLAB, total - base);
      if (base > 0) __syncthreads();
      for (int s2 = tid; s2 < ns; s2 += 128) {
        const int gs = base + s2;
        int lo = 0, hi = nc;  // the box k with spre[k] <= gs < spre[k + 1]
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (spre[mid] <= gs) lo = mid;
          else hi = mid;
        }
        const int j = sj0[lo] + gs - spre[lo];
        sz[s2] = zhl[j];
        if (E == 2) {
          sp[s2] = reinterpret_cast<const float4*>(pq)[j];
          sa[s2] = aa[j];
        } else {
          sa[s2] = qa[j];
        }
      }
      __syncthreads();
#pragma unroll 2
      for (int jj = sl; jj < ns; jj += NS) {
        const float4 hlj = sz[jj];
        const float4 PQ = E == 2 ? sp[jj] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float2 A = sa[jj];
        near_pair<E>(hlj, PQ, A, h0, gx0, gy0);
        near_pair<E>(hlj, PQ, A, h1, gx1, gy1);
      }
    }
  }
  sred[sl][t0] = make_float2(gx0, gy0);
  sred[sl][t0 + 16] = make_float2(gx1, gy1);
  __syncthreads();
  if (tid < EB_NTILE && tl.y + tid < tl.z) {
    float2 v = sred[0][tid];
#pragma unroll
    for (int q = 1; q < NS; ++q) {
      v.x += sred[q][tid].x;
      v.y += sred[q][tid].y;
    }
    nearbuf[tl.y + tid] = make_double2((double)v.x, (double)v.y);
  }
}

// ---------------------------------------------------------------------------------
// Direct sums for small point sets (at most eb_opts.direct_max points, one problem, free
// space). Every pair by the near-field formula of the leaf kernels, with the FMM's charges
// (sorted order) and its fused post-processing; one block of 128 threads per target, the
// threads over the sources, their partial sums added in a fixed order (direct_block_sum). On a few hundred points the
// FMM's chain of about a dozen dependent launches, each on a handful of SMs, costs far
// more than all N^2 pairs: an FP64 pair is ~35 FP64 instructions, so 1,024 points take
// ~60 us of the GPU's FP64 rate. The sums are exact up to rounding (no truncation).
// ---------------------------------------------------------------------------------
// The sum of a block's partial sums, in thread 0 (warp butterflies, then the warps in
// order through shared memory).
template <typename T>
__device__ __forceinline__ void direct_block_sum(T& gx, T& gy) {
  __shared__ T sx[4], sy[4];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gx += __shfl_xor_sync(0xffffffffu, gx, o);
    gy += __shfl_xor_sync(0xffffffffu, gy, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sx[w] = gx;
    sy[w] = gy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    gx = sx[0] + sx[1] + sx[2] + sx[3];
    gy = sy[0] + sy[1] + sy[2] + sy[3];
  }
}

template <int E>
__global__ void __launch_bounds__(128) k_direct64(int n, const double2* __restrict__ zs,
                                                  const double2* __restrict__ pq,
                                                  const double2* __restrict__ aa,
                                                  const double2* __restrict__ qa, const int* __restrict__ perm,
                                                  double2* __restrict__ out, EbPost post) {
  const int i = blockIdx.x;  // one block of 128 threads per target, the threads over the sources
  const double2 zi = zs[i];
  double gx = 0.0, gy = 0.0;
  for (int j = threadIdx.x; j < n; j += 128) {
    if (j == i) continue;
    const double2 zj = zs[j];
    const double dx = zj.x - zi.x, dy = zj.y - zi.y;
    const double rr = rcp_nr(fma(dx, dx, dy * dy));
    const double ix = dx * rr, iy = -dy * rr;  // 1/D
    if (E == 2) {
      const double2 P = pq[2 * j], Q = pq[2 * j + 1], A = aa[j];
      gx = fma(P.x, ix, fma(-P.y, iy, gx));  // qa/D + s conj(qb/D)
      gy = fma(Q.x, iy, fma(Q.y, ix, gy));
      const double w2x = fma(ix, ix, -iy * iy), w2y = -2.0 * ix * iy;  // conj(1/D)^2
      const double tx = fma(dx, w2x, -dy * w2y), ty = fma(dx, w2y, dy * w2x);
      gx = fma(A.x, tx, fma(-A.y, ty, gx));  // - s D conj(qa) conj(1/D)^2
      gy = fma(A.x, ty, fma(A.y, tx, gy));
    } else {
      const double2 q = qa[j];
      gx = fma(-q.x, ix, fma(q.y, iy, gx));  // q/(z_i - z_j) = -q/D
      gy = fma(-q.x, iy, fma(-q.y, ix, gy));
    }
  }
  direct_block_sum<double>(gx, gy);
  if (threadIdx.x == 0) eb_post_store(post, perm[i], make_double2(gx, gy), out);
}

// The FP32 operator's direct sums: positions as float hi + lo, the pair of k_near32.
template <int E>
__global__ void __launch_bounds__(128) k_direct32(int n, const float4* __restrict__ zhl,
                                                  const float4* __restrict__ pq, const float2* __restrict__ aa,
                                                  const float2* __restrict__ qa, const int* __restrict__ perm,
                                                  double2* __restrict__ out, EbPost post) {
  const int i = blockIdx.x;
  const float4 hi = zhl[i];
  float gx = 0.f, gy = 0.f;
  for (int j = threadIdx.x; j < n; j += 128) {
    if (j == i) continue;
    const float4 PQ = E == 2 ? pq[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 A = E == 2 ? aa[j] : qa[j];
    near_pair<E>(zhl[j], PQ, A, hi, gx, gy);
  }
  direct_block_sum<float>(gx, gy);
  if (threadIdx.x == 0) eb_post_store_f32(post, perm[i], make_float2(gx, gy), out);
}

// ---------------------------------------------------------------------------------
// Wall-bounded flow (IFLAG2 = 1 of CADAPDR / CADAPMOD): the images of the sources across
// the wall y = 0, the bottom edge of the root square.
// ---------------------------------------------------------------------------------
// MPREFLECT (cadap2.f:1468-1507) for scaled coefficients with psi relative to the
// centre: a box of centre c, side r and height yh = Im(c) / r = iy + 1/2 has the
// mirrored expansions about conj(c)
//   Mphi'[k] = conj(-Mpsi[k] + (k+1) Mphi[k] + 2 i yh k Mphi[k-1]),
//   Mpsi'[k] = -conj(Mphi[k]) + (k+1) Mphi'[k] - 2 i yh k Mphi'[k-1]
// (the reference's formulas with its absolute psi, psi = psi_c - conj(c) phi', and the
// factor r^(k+1) of each coefficient taken out). One thread per (box, k).
// Mphi'[k] from Mphi[k], Mpsi[k] and Mphi[k-1]:
template <typename T>
__device__ __forceinline__ c_t<T> reflect_phi(c_t<T> phk, c_t<T> psk, c_t<T> phk1, int k, T yh) {
  c_t<T> v = csub<T>(cscale<T>(phk, (T)(k + 1)), psk);
  const T f = (T)2 * yh * (T)k;  // + 2 i yh k Mphi[k-1]
  v.x -= f * phk1.y;
  v.y += f * phk1.x;
  return cconj<T>(v);
}

// Mphi'[k] and Mpsi'[k] from the orders k, k-1 and k-2 (zeros below order 0)
template <typename T>
__device__ __forceinline__ void reflect_pair(c_t<T> phk, c_t<T> psk, c_t<T> phk1, c_t<T> psk1, c_t<T> phk2,
                                             int k, T yh, c_t<T>& a, c_t<T>& b) {
  a = reflect_phi<T>(phk, psk, phk1, k, yh);
  b = csub<T>(cscale<T>(a, (T)(k + 1)), cconj<T>(phk));
  if (k >= 1) {
    const c_t<T> a1 = reflect_phi<T>(phk1, psk1, phk2, k - 1, yh);
    const T f = (T)2 * yh * (T)k;  // - 2 i yh k Mphi'[k-1]
    b.x += f * a1.y;
    b.y -= f * a1.x;
  }
}

template <typename T>
__global__ void k_reflect(int first, int nb, const unsigned long long* __restrict__ bkey, int p,
                          const c_t<T>* __restrict__ mpole, c_t<T>* __restrict__ mimg) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)nb * p) return;
  const int b = first + (int)(idx / p), k = (int)(idx % p);
  const T yh = (T)compact2d(bkey[b] >> 1) + (T)0.5;
  const c_t<T>* m = mpole + (size_t)b * 2 * p;
  const c_t<T> z = cmk<T>(0, 0);
  c_t<T> a, c;
  reflect_pair<T>(m[k], m[p + k], k >= 1 ? m[k - 1] : z, k >= 1 ? m[p + k - 1] : z, k >= 2 ? m[k - 2] : z, k, yh,
                  a, c);
  mimg[(size_t)b * 2 * p + k] = a;
  mimg[(size_t)b * 2 * p + p + k] = c;
}

// The same for double-float multipoles, the mirror formed in FP64
__global__ void k_reflect_df(int first, int nb, const unsigned long long* __restrict__ bkey, int p,
                             const float4* __restrict__ mpole, float4* __restrict__ mimg) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)nb * p) return;
  const int b = first + (int)(idx / p), k = (int)(idx % p);
  const double yh = (double)compact2d(bkey[b] >> 1) + 0.5;
  const float4* m = mpole + (size_t)b * 2 * p;
  auto ld = [&](int i, int lo) {
    if (i < lo) return make_double2(0.0, 0.0);
    const float4 v = m[i];
    return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
  };
  double2 a, c;
  reflect_pair<double>(ld(k, 0), ld(p + k, 0), ld(k - 1, 0), ld(p + k - 1, p), ld(k - 2, 0), k, yh, a, c);
  mimg[(size_t)b * 2 * p + k] = df4(a);
  mimg[(size_t)b * 2 * p + p + k] = df4(c);
}

// The reflected near field: for every box T of level ld in the first row (on the wall),
// the images of the points of the first-row boxes next to T and of T's own at T's points
// (DONN0DR's IFLAG2 loop with MKNBRRFL, cadapdrop2.f:690-721, and the pair terms of
// SLDREFDR / SLDREF, cadapdrop2.f:857-934 and cadap2.f:1509-1586), in FP64 whatever the
// operator's arithmetic, added to the operator's output. With qc = -conj(z) qa,
//   gamma1 = conj(qa) - conj(qb), gamma2 = 2 i y_j conj(qa), delta1 = -conj(qb),
//   t = 1 / (conj(z_j) - z):  Phi = gamma1 t + gamma2 t^2, and
//   z conj(Phi') + conj(Psi) = (z - z_j) conj(gamma1 t^2 + 2 gamma2 t^3)
//                              + 2 conj(gamma2 t^2) + conj(delta1 t),
// which has no terms of size |z|. One block per box of level ld (blocks off the wall
// return at once); sources staged through shared memory. sorted: add into dst in the
// sorted order (the near-field buffer of the split passes), else in node order.
#define IMG_TILE 128
__global__ void __launch_bounds__(IMG_TILE) k_img_near(int off, int nb, int lev,
                                                       const unsigned long long* __restrict__ bkey,
                                                       const int* __restrict__ pt0, const int* __restrict__ pt1,
                                                       const double2* __restrict__ zs, const int* __restrict__ perm,
                                                       const double2* __restrict__ dens,
                                                       const double2* __restrict__ dz,
                                                       const double* __restrict__ hpt, double s,
                                                       double2* __restrict__ dst, int sorted) {
  __shared__ double2 sz[IMG_TILE], sg1[IMG_TILE], sg2[IMG_TILE], sd1[IMG_TILE];
  const int b = off + blockIdx.x;
  const unsigned long long key = bkey[b];
  if (compact2d(key >> 1) != 0) return;
  const int ix = (int)compact2d(key), side = 1 << lev;
  int src[3], nsrc = 0;
  for (int dx = -1; dx <= 1; ++dx) {
    const int sx = ix + dx;
    if (sx < 0 || sx >= side) continue;
    const unsigned long long kk = morton_key((unsigned)sx, 0u);
    int lo = 0, hi = nb - 1, f = -1;
    while (lo <= hi) {
      const int mid = (lo + hi) >> 1;
      const unsigned long long v = bkey[off + mid];
      if (v == kk) {
        f = off + mid;
        break;
      }
      if (v < kk) lo = mid + 1;
      else hi = mid - 1;
    }
    if (f >= 0) src[nsrc++] = f;
  }
  const double c2pi = 1.0 / (2.0 * EB_PI);
  for (int tb = pt0[b]; tb < pt1[b]; tb += IMG_TILE) {
    const int i = tb + threadIdx.x;
    const bool act = i < pt1[b];
    const double2 zt = zs[act ? i : pt0[b]];
    double2 acc = make_double2(0.0, 0.0);
    for (int q = 0; q < nsrc; ++q) {
      for (int jb = pt0[src[q]]; jb < pt1[src[q]]; jb += IMG_TILE) {
        const int cnt = min(IMG_TILE, pt1[src[q]] - jb);
        __syncthreads();
        if (threadIdx.x < cnt) {
          const int j = jb + threadIdx.x, o = perm[j];
          const double2 u = dens[o], d = dz[o];
          const double h = hpt[o] * c2pi;
          const double2 w = cmul<double>(u, d);
          const double2 qa = make_double2(w.y * h, -w.x * h);  // u dz h / (2 pi i)
          const double2 v = csub<double>(cmul<double>(u, cconj<double>(d)), cmul<double>(cconj<double>(u), d));
          const double2 qb = make_double2(v.y * h, -v.x * h);
          const double2 zj = zs[j];
          sz[threadIdx.x] = zj;
          sg1[threadIdx.x] = make_double2(qa.x - qb.x, qb.y - qa.y);            // conj(qa) - conj(qb)
          sg2[threadIdx.x] = make_double2(2.0 * zj.y * qa.y, 2.0 * zj.y * qa.x);  // 2 i y conj(qa)
          sd1[threadIdx.x] = make_double2(-qb.x, qb.y);                         // -conj(qb)
        }
        __syncthreads();
        if (act) {
          for (int jj = 0; jj < cnt; ++jj) {
            const double2 zj = sz[jj], g1 = sg1[jj], g2 = sg2[jj], d1 = sd1[jj];
            const double2 ze = make_double2(zj.x - zt.x, -zj.y - zt.y);  // conj(z_j) - z
            const double rd = 1.0 / (ze.x * ze.x + ze.y * ze.y);
            const double2 t1 = make_double2(ze.x * rd, -ze.y * rd);
            const double2 t2 = cmul<double>(t1, t1);
            const double2 dd = make_double2(zt.x - zj.x, zt.y - zj.y);
            const double2 g2t2 = cmul<double>(g2, t2);
            const double2 phi = cadd<double>(cmul<double>(g1, t1), g2t2);
            const double2 dphi = cadd<double>(cmul<double>(g1, t2), cscale<double>(cmul<double>(g2t2, t1), 2.0));
            const double2 r = cadd<double>(cmul<double>(dd, cconj<double>(dphi)),
                                           cadd<double>(cscale<double>(cconj<double>(g2t2), 2.0),
                                                        cconj<double>(cmul<double>(d1, t1))));
            acc.x += phi.x + s * r.x;
            acc.y += phi.y + s * r.y;
          }
        }
      }
    }
    if (act) {
      const int o = sorted ? i : perm[i];
      dst[o] = make_double2(dst[o].x + acc.x, dst[o].y + acc.y);
    }
  }
}

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }
inline int round32(int n) { return (n + 31) & ~31; }
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
  if (sizeof(T) == 8) {
    auto split = [](double v, float& h, float& l) {
      h = (float)v;
      l = (float)(v - (double)h);
    };
    std::vector<float2> bdf(bd.size());
    for (size_t i = 0; i < bd.size(); ++i) split(bd[i], bdf[i].x, bdf[i].y);
    auto to_df = [&](const std::vector<c_t<T>>& v) {
      std::vector<float4> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        split((double)v[i].x, o[i].x, o[i].y);
        split((double)v[i].y, o[i].z, o[i].w);
      }
      return o;
    };
    std::vector<float4> ddf = to_df(dinv), edf = to_df(epow2), idf = to_df(einv);
    EB_TRY(tb.binom_df.ensure(sizeof(float2) * bdf.size()));
    EB_TRY(tb.dinv_df.ensure(sizeof(float4) * ddf.size()));
    EB_TRY(tb.epow_df.ensure(sizeof(float4) * edf.size()));
    EB_TRY(tb.einv_df.ensure(sizeof(float4) * idf.size()));
    EB_CUDA_TRY(cudaMemcpy(tb.binom_df.p, bdf.data(), sizeof(float2) * bdf.size(), cudaMemcpyHostToDevice));
    EB_CUDA_TRY(cudaMemcpy(tb.dinv_df.p, ddf.data(), sizeof(float4) * ddf.size(), cudaMemcpyHostToDevice));
    EB_CUDA_TRY(cudaMemcpy(tb.epow_df.p, edf.data(), sizeof(float4) * edf.size(), cudaMemcpyHostToDevice));
    EB_CUDA_TRY(cudaMemcpy(tb.einv_df.p, idf.data(), sizeof(float4) * idf.size(), cudaMemcpyHostToDevice));
  }
  return EB_OK;
}

struct ProfScope {
  eb_ctx* ctx;
  int cls;
  cudaStream_t st;
  cudaEvent_t e0, e1;
  ProfScope(eb_ctx* c, int k, cudaStream_t s) : ctx(c), cls(k), st(s) {
    e0 = k == 2 ? ctx->ev_near0 : ctx->ev0;
    e1 = k == 2 ? ctx->ev_near1 : ctx->ev1;
    if (ctx->profiling) cudaEventRecord(e0, st);
  }
  void done() {
    if (!ctx->profiling) return;
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ctx->prof_launch[cls]++;
    ctx->prof_ms[cls] += ms;
  }
};

// Upward pass, M2L and downward pass, shared by both kernels. Leaves the local
// expansions of every box in w.local.
// Expansions of the double-float pipeline (FP64-class accuracy on the FP32 pipes):
// P2M, M2M per level, M2L, L2L per level; multipoles and locals stay double-float.
template <int E>
int fmm_expansions_df(eb_ctx* ctx, EbTree& t, EbTables& tb, EbFmmWork& w) {
  cudaStream_t st = eb_stream(ctx);
  const int p = tb.p, L = t.L;
  const int ldb = 2 * p + 2;
  EB_TRY(w.mpole_df.ensure(sizeof(float4) * (size_t)t.nbox * E * p));
  EB_TRY(w.local_df.ensure(sizeof(float4) * (size_t)t.nbox * E * (p + 1)));
  float4* mp = w.mpole_df.as<float4>();
  float4* lo = w.local_df.as<float4>();
  {
    size_t sm = sizeof(float4) * (32 * (size_t)(p + 1) + 96);
    if (sm > 48 * 1024) EB_CUDA_TRY(cudaFuncSetAttribute(k_p2m_df<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_p2m_df<E><<<t.nleaf, std::max(128, round32((E == 2 ? 3 : 1) * p)), sm, st>>>(t.leaves.as<int>(), t.pt0.as<int>(), t.pt1.as<int>(), t.wdf.as<float4>(),
                                          E == 2 ? w.qdf.as<float4>() : w.pqdf.as<float4>(), p, mp);
    eb_count_launch(ctx);
  }
  for (int l = L - 1; l >= 2; --l) {
    int nb = t.lev_off[l + 1] - t.lev_off[l];
    size_t sm = sizeof(float4) * 4 * E * p;
    k_m2m_df<E><<<nb, round32(4 * E * p), sm, st>>>(t.lev_off[l], t.bkey.as<unsigned long long>(), t.child0.as<int>(),
                                                t.nchild.as<int>(), p, tb.binom_df.as<float2>(), ldb,
                                                tb.epow_df.as<float4>(), tb.einv_df.as<float4>(), mp);
    eb_count_launch(ctx);
  }
  {
    int first = t.lev_off[2], nt = t.nbox - first;
    size_t sm = sizeof(float4) * ((size_t)(p * (p + 1) + 1) / 2 + 4 * E * (size_t)(2 * p + 1));
    if (sm > 48 * 1024)
      EB_CUDA_TRY(cudaFuncSetAttribute(k_m2l_df<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    ProfScope ps(ctx, 1, st);
    if (nt > 0) {
      k_m2l_df<E><<<nt, 128, sm, st>>>(first, t.vlist.as<int>(), t.vcode.as<unsigned char>(), t.vcount.as<int>(),
                                       p, tb.binom_df.as<float2>(), ldb, tb.dinv_df.as<float4>(), tb.pd.as<int>(),
                                       mp, lo, 0);
      eb_count_launch(ctx);
    }
    if (E == 2 && t.wall && t.ld >= 2) {  // the wall's reflected boxes
      const int nimg = t.lev_off[t.ld + 1], nbi = nimg - first;
      EB_TRY(w.mimg.ensure(sizeof(float4) * (size_t)nimg * E * p));
      k_reflect_df<<<nblk((long long)nbi * p, 128), 128, 0, st>>>(first, nbi, t.bkey.as<unsigned long long>(), p,
                                                                 mp, w.mimg.as<float4>());
      k_m2l_df<E><<<nbi, 128, sm, st>>>(first, t.ilist.as<int>(), t.icode.as<unsigned char>(), t.icount.as<int>(),
                                        p, tb.binom_df.as<float2>(), ldb, tb.dinv_df.as<float4>(), tb.pd.as<int>(),
                                        w.mimg.as<float4>(), lo, 1);
      ctx->launches += 2;
    }
    ps.done();
  }
  for (int l = 3; l <= L; ++l) {
    int nb = t.lev_off[l + 1] - t.lev_off[l];
    size_t sm = sizeof(float4) * E * (p + 1);
    k_l2l_df<E><<<nb, round32(4 * E * (p + 1)), sm, st>>>(t.lev_off[l], t.bkey.as<unsigned long long>(),
                                                     t.parent.as<int>(), p, tb.binom_df.as<float2>(), ldb,
                                                     tb.epow_df.as<float4>(), tb.einv_df.as<float4>(), lo);
    eb_count_launch(ctx);
  }
  return EB_OK;
}

template <typename T, int E>
int fmm_expansions(eb_ctx* ctx, EbTree& t, EbTables& tb, EbFmmWork& w) {
  cudaStream_t st = eb_stream(ctx);
  const int p = tb.p, L = t.L;
  const int ldb = 2 * p + 2;
  EB_TRY(w.mpole.ensure(sizeof(c_t<T>) * (size_t)t.nbox * E * p));
  EB_TRY(w.local.ensure(sizeof(c_t<T>) * (size_t)t.nbox * E * (p + 1)));
  // Upward pass. FP32: direct P2M (in chunks) for every box of the EB_DIRECT_LEVELS
  // finest levels in one launch, then M2M per coarser level. FP64: P2M and one M2M
  // launch per level.
  if (sizeof(T) == 4) {
    const int lmin = t.chunk_lmin;
    const int first2 = t.lev_off[2], nout = E * p;
    EB_TRY(w.mpart.ensure(sizeof(float2) * (size_t)t.nchunk * nout));
    LevOff lo;
    for (int l = 0; l < EB_KEY_LEVELS + 2; ++l) {
      lo.v[l] = t.lev_off[l];
      lo.rinv[l] = (float)((double)(1u << std::min(l, 30)) / t.W);
    }
    const size_t sm = sizeof(float2) * ((size_t)EB_CHUNK * (p + 1) + (E == 2 ? 3 : 1) * (EB_CHUNK + 2 * (size_t)p));
    k_p2m_chunks<E><<<t.nchunk, 128, sm, st>>>(lo, first2, t.blev.as<unsigned char>(), t.plev.as<unsigned char>(),
                                              t.chunk_box.as<int>(), t.cstart.as<int>(),
                                              t.keys.as<unsigned long long>(), t.pt0.as<int>(), t.pt1.as<int>(),
                                              t.wdf.as<float4>(), reinterpret_cast<const float2*>(w.qa.p),
                                              reinterpret_cast<const float2*>(w.qb.p), t.W, p,
                                              w.mpart.as<float2>(), t.cdone.as<int>(),
                                              reinterpret_cast<float2*>(w.mpole.p));
    eb_count_launch(ctx);
    for (int l = lmin - 1; l >= 2; --l) {
      int nb = t.lev_off[l + 1] - t.lev_off[l];
      size_t sm2 = sizeof(float2) * 4 * (size_t)nout;
      k_m2m_f32<E><<<nb, std::max(128, round32(nout)), sm2, st>>>(
          t.lev_off[l], t.bkey.as<unsigned long long>(), t.child0.as<int>(), t.nchild.as<int>(), p,
          reinterpret_cast<const float*>(tb.binom.p), ldb, reinterpret_cast<const float2*>(tb.epow.p),
          reinterpret_cast<const float2*>(tb.einv.p), reinterpret_cast<float2*>(w.mpole.p));
      eb_count_launch(ctx);
    }
  } else {
    size_t sm = sizeof(c_t<T>) * (32 * (size_t)(p + 1) + 96);
    k_p2m<T, E><<<t.nleaf, 64, sm, st>>>(t.leaves.as<int>(), t.bkey.as<unsigned long long>(),
                                          t.blev.as<unsigned char>(), t.pt0.as<int>(),
                                          t.pt1.as<int>(), t.zs.as<double2>(), w.qa.as<c_t<T>>(),
                                          w.qb.as<c_t<T>>(), t.x0, t.y0, t.W, p,
                                          w.mpole.as<c_t<T>>());
    eb_count_launch(ctx);
    for (int l = L - 1; l >= 2; --l) {
      int nb = t.lev_off[l + 1] - t.lev_off[l];
      size_t sm2 = sizeof(c_t<T>) * E * p;
      k_m2m<T, E><<<nb, round32(E * p), sm2, st>>>(t.lev_off[l], t.bkey.as<unsigned long long>(),
                                                   t.child0.as<int>(), t.nchild.as<int>(), p,
                                                   tb.binom.as<T>(), ldb, tb.epow.as<c_t<T>>(),
                                                   tb.einv.as<c_t<T>>(), w.mpole.as<c_t<T>>());
      eb_count_launch(ctx);
    }
  }
  {
    int first = t.lev_off[2], nt = t.nbox - first;
    size_t c2 = (sizeof(T) * (size_t)p * (p + 1) + 15) & ~(size_t)15;
    size_t sm = c2 + sizeof(c_t<T>) * 4 * E * (size_t)(2 * p + 1);
    if (sm > 48 * 1024)
      EB_CUDA_TRY(cudaFuncSetAttribute(k_m2l<T, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    ProfScope ps(ctx, 1, st);
    if (nt > 0 && sizeof(T) == 4 && p == 20 && ctx->opts.m2l_tc > 0) {
      EB_TRY(eb_m2l_tc(ctx, E, first, nt, t.vlist.as<int>(), t.vcode.as<unsigned char>(), t.vcount.as<int>(),
                       reinterpret_cast<const float*>(tb.binom.p), ldb, reinterpret_cast<const float2*>(tb.dinv.p),
                       tb.pd.as<int>(), reinterpret_cast<const float2*>(w.mpole.p),
                       reinterpret_cast<float2*>(w.local.p), st));
    } else if (nt > 0 && sizeof(T) == 4 && p == 20) {
      k_m2l_f32p<E, 20><<<nt, 128, 0, st>>>(first, t.vlist.as<int>(), t.vcode.as<unsigned char>(),
                                            t.vcount.as<int>(), reinterpret_cast<const float*>(tb.binom.p), ldb,
                                            reinterpret_cast<const float2*>(tb.dinv.p), tb.pd.as<int>(),
                                            reinterpret_cast<const float2*>(w.mpole.p),
                                            reinterpret_cast<float2*>(w.local.p), 0);
      eb_count_launch(ctx);
    } else if (nt > 0) {
      k_m2l<T, E><<<nt, 128, sm, st>>>(first, t.vlist.as<int>(), t.vcode.as<unsigned char>(),
                                       t.vcount.as<int>(), p, tb.binom.as<T>(), ldb,
                                       tb.dinv.as<c_t<T>>(), tb.pd.as<int>(), w.mpole.as<c_t<T>>(),
                                       w.local.as<c_t<T>>(), 0);
      eb_count_launch(ctx);
    }
    if (E == 2 && t.wall && t.ld >= 2) {  // the wall's reflected boxes
      const int nimg = t.lev_off[t.ld + 1], nbi = nimg - first;
      EB_TRY(w.mimg.ensure(sizeof(c_t<T>) * (size_t)nimg * E * p));
      k_reflect<T><<<nblk((long long)nbi * p, 128), 128, 0, st>>>(first, nbi, t.bkey.as<unsigned long long>(), p,
                                                                 w.mpole.as<c_t<T>>(), w.mimg.as<c_t<T>>());
      if (sizeof(T) == 4 && p == 20)
        k_m2l_f32p<E, 20><<<nbi, 128, 0, st>>>(first, t.ilist.as<int>(), t.icode.as<unsigned char>(),
                                               t.icount.as<int>(), reinterpret_cast<const float*>(tb.binom.p), ldb,
                                               reinterpret_cast<const float2*>(tb.dinv.p), tb.pd.as<int>(),
                                               reinterpret_cast<const float2*>(w.mimg.p),
                                               reinterpret_cast<float2*>(w.local.p), 1);
      else
        k_m2l<T, E><<<nbi, 128, sm, st>>>(first, t.ilist.as<int>(), t.icode.as<unsigned char>(), t.icount.as<int>(),
                                          p, tb.binom.as<T>(), ldb, tb.dinv.as<c_t<T>>(), tb.pd.as<int>(),
                                          w.mimg.as<c_t<T>>(), w.local.as<c_t<T>>(), 1);
      ctx->launches += 2;
    }
    ps.done();
  }
  // Downward pass. FP64: L2L level by level. FP32: L2L only into the level lend, the
  // coarsest of the EB_FAR_LEVELS finest levels; the far-field kernel evaluates the M2L
  // expansions of the levels below it directly (cheap FP32 work instead of a dependent
  // chain of shifts).
  {
    const int lend = sizeof(T) == 8 ? L : t.lend;
    for (int l = 3; l <= lend; ++l) {
      int nb = t.lev_off[l + 1] - t.lev_off[l];
      size_t sm = sizeof(c_t<T>) * E * (p + 1);
      k_l2l<T, E><<<nb, round32(E * (p + 1)), sm, st>>>(t.lev_off[l], t.bkey.as<unsigned long long>(),
                                                       t.parent.as<int>(), p, tb.binom.as<T>(), ldb,
                                                       tb.epow.as<c_t<T>>(), tb.einv.as<c_t<T>>(),
                                                       w.local.as<c_t<T>>());
      eb_count_launch(ctx);
    }
  }
  return EB_OK;
}

// The direct path of a small problem: the FMM's charges, k_direct64 / k_direct32, and
// the post-processing. FP64-class requests (native or double-float) run in native FP64.
template <int E>
int direct_run(eb_ctx* ctx, EbTree& t, bool f32, int sign, const double2* dens, const double2* dz,
               const double* hpt, const double2* q, double2* out, const EbPost* postp, cudaEvent_t join) {
  EbPost post{};
  if (postp) post = *postp;
  cudaStream_t st = eb_stream(ctx);
  const int n = t.n;
  EbFmmWork& w = f32 ? ctx->work32 : ctx->work64;
  const size_t cs = f32 ? sizeof(float2) : sizeof(double2);
  EB_TRY(w.qa.ensure(cs * (size_t)n));
  EB_TRY(w.qb.ensure(cs * (size_t)n));
  EB_TRY(w.pq.ensure(cs * 2 * (size_t)n));
  EB_TRY(w.aa.ensure(cs * (size_t)n));
  const int g = n;  // one block of 128 threads per target
  if (f32) {
    if (E == 2)
      k_charges_stokes<float><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), dens, dz, hpt, (double)sign,
                                                            w.qa.as<float2>(), w.qb.as<float2>(),
                                                            w.pq.as<float2>(), w.aa.as<float2>());
    else
      k_charges_cauchy<float><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), q, post.u, post.dz, post.hpt,
                                                            w.qa.as<float2>());
    if (join) EB_CUDA_TRY(cudaStreamWaitEvent(st, join, 0));
    k_direct32<E><<<g, 128, 0, st>>>(n, t.zhl.as<float4>(), reinterpret_cast<const float4*>(w.pq.p),
                                     w.aa.as<float2>(), w.qa.as<float2>(), t.perm.as<int>(), out, post);
  } else {
    if (E == 2)
      k_charges_stokes<double><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), dens, dz, hpt, (double)sign,
                                                             w.qa.as<double2>(), w.qb.as<double2>(),
                                                             w.pq.as<double2>(), w.aa.as<double2>());
    else
      k_charges_cauchy<double><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), q, post.u, post.dz, post.hpt,
                                                             w.qa.as<double2>());
    if (join) EB_CUDA_TRY(cudaStreamWaitEvent(st, join, 0));
    k_direct64<E><<<g, 128, 0, st>>>(n, t.zs.as<double2>(), w.pq.as<double2>(), w.aa.as<double2>(),
                                     w.qa.as<double2>(), t.perm.as<int>(), out, post);
  }
  ctx->launches += 2;
  return eb_check_launch(ctx, "direct sum");
}

template <typename T, int E>
int fmm_run(eb_ctx* ctx, EbTree& t, int sign, const double2* dens, const double2* dz,
            const double* hpt, const double2* q, double2* out, const EbPost* postp,
            cudaEvent_t join, bool df_req) {
  // a direct tree (eb_tree_build: at most eb_opts.direct_max points, one problem -- a
  // batch's forest keeps its simulations apart through the tree -- and no wall)
  if (t.direct) return direct_run<E>(ctx, t, sizeof(T) == 4, sign, dens, dz, hpt, q, out, postp, join);
  EbPost post{};
  if (postp) post = *postp;
  cudaStream_t st = eb_stream(ctx);
  const bool f64 = sizeof(T) == 8;
  EbTables& tb = f64 ? ctx->tab64 : ctx->tab32;
  EbFmmWork& w = f64 ? ctx->work64 : ctx->work32;
  const int n = t.n;
  const bool df = f64 && df_req;
  if (df) {
    EB_TRY(w.pqdf.ensure(sizeof(float4) * 2 * (size_t)n));
    EB_TRY(w.aadf.ensure(sizeof(float4) * (size_t)n));
    EB_TRY(w.qdf.ensure(sizeof(float4) * 2 * (size_t)n));
  } else {
    EB_TRY(w.qa.ensure(sizeof(c_t<T>) * (size_t)n));
    EB_TRY(w.qb.ensure(sizeof(c_t<T>) * (size_t)n));
    EB_TRY(w.pq.ensure(sizeof(c_t<T>) * 2 * (size_t)n));
    EB_TRY(w.aa.ensure(sizeof(c_t<T>) * (size_t)n));
  }
  if (df && E == 2) {
    k_charges_stokes_df<<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), dens, dz, hpt, (double)sign,
                                                      1.0 / t.W, t.plev.as<unsigned char>(), w.qdf.as<float4>(),
                                                      w.pqdf.as<float4>(), w.aadf.as<float4>());
  } else if (df) {
    k_charges_cauchy_df<<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), q, post.u, post.dz, post.hpt,
                                                      1.0 / t.W, t.plev.as<unsigned char>(), w.pqdf.as<float4>());
  } else if (E == 2) {
    k_charges_stokes<T><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), dens, dz, hpt, (double)sign,
                                                      w.qa.as<c_t<T>>(), w.qb.as<c_t<T>>(),
                                                      w.pq.as<c_t<T>>(), w.aa.as<c_t<T>>());
  } else {
    k_charges_cauchy<T><<<nblk(n, 256), 256, 0, st>>>(n, t.perm.as<int>(), q, post.u, post.dz, post.hpt,
                                                      w.qa.as<c_t<T>>());
  }
  eb_count_launch(ctx);
  const int has_far = t.L >= 2;
  int blocks = nblk((long long)t.ngroup * 32, 128);
  // FP32 and double-float: the near field runs on the side stream while the expansion
  // passes run on the main stream, and the far-field kernel adds both. Measured up to
  // 2^20 nodes it pays at every size (the expansion passes' coarse levels stay
  // latency-bound): against a limit of 2^18, the 285,440-node batch's RK2 step 35.1 →
  // 33.6 ms and the 1,048,576-node refined solve 45.7 → 44.3 ms. The per-kernel profiling
  // timer times the combined kernel.
  const bool split = has_far && (df || !f64) && !ctx->profiling && n <= (1 << 20);
  if (split) {
    EB_TRY(w.nearbuf.ensure(sizeof(double2) * (size_t)n));
    EB_CUDA_TRY(cudaEventRecord(ctx->ev_c, st));
    EB_CUDA_TRY(cudaStreamWaitEvent(ctx->side_stream, ctx->ev_c, 0));
    cudaStream_t ss = ctx->side_stream;
    if (df) {
      k_leaf_df<E, 1><<<blocks, 128, 0, ss>>>(
          t.ngroup, t.gleaf.as<int>(), t.gfirst.as<int>(), t.leaves.as<int>(), 0, t.bkey.as<unsigned long long>(),
          t.blev.as<unsigned char>(), t.pt0.as<int>(), t.pt1.as<int>(), t.ustart.as<int>(), t.ulist.as<int>(),
          t.wstart.as<int>(), t.wlist.as<int>(), w.mpole_df.as<float4>(), t.perm.as<int>(),
          t.wdf.as<float4>(), t.wdf_lo.as<float2>(), w.pqdf.as<float4>(), w.aadf.as<float4>(), tb.p,
          (double)sign, w.local_df.as<float4>(), out, post, w.nearbuf.as<double2>());
    } else {
      k_near32<E><<<t.ntile, 128, 0, ss>>>(t.tiles.as<int4>(), t.leaves.as<int>(), t.pt0.as<int>(), t.pt1.as<int>(),
                                           t.ustart.as<int>(), t.ulist.as<int>(), t.zhl.as<float4>(),
                                           w.pq.as<float2>(), w.aa.as<float2>(), w.qa.as<float2>(),
                                           w.nearbuf.as<double2>());
    }
    eb_count_launch(ctx);
    if (E == 2 && t.wall && dz) {  // the wall's reflected near field joins the near-field sums
      const int ld = t.ld, nbl = t.lev_off[ld + 1] - t.lev_off[ld];
      k_img_near<<<nbl, IMG_TILE, 0, ss>>>(t.lev_off[ld], nbl, ld, t.bkey.as<unsigned long long>(), t.pt0.as<int>(),
                                           t.pt1.as<int>(), t.zs.as<double2>(), t.perm.as<int>(), dens, dz, hpt,
                                           (double)sign, w.nearbuf.as<double2>(), 1);
      eb_count_launch(ctx);
    }
    EB_CUDA_TRY(cudaEventRecord(ctx->ev_p2p, ss));
  }
  if (has_far && df) EB_TRY(fmm_expansions_df<E>(ctx, t, tb, w));
  else if (has_far) EB_TRY((fmm_expansions<T, E>(ctx, t, tb, w)));
  if (!has_far) {
    EB_TRY(w.local.ensure(sizeof(c_t<T>) * (size_t)(E * (tb.p + 1))));
    EB_TRY(w.local_df.ensure(sizeof(float4) * (size_t)(E * (tb.p + 1))));
  }
  const int far_lev = has_far ? std::min(t.L - 1, EB_FAR_LEVELS) : 0;  // far boxes per leaf, at most
  const size_t far_sm = sizeof(float2) * (size_t)far_lev * E * (tb.p + 1);
  if (split) EB_CUDA_TRY(cudaStreamWaitEvent(st, ctx->ev_p2p, 0));
  if (join) EB_CUDA_TRY(cudaStreamWaitEvent(st, join, 0));
  if (!split && !f64) {
    // FP32 without the split: the near-field kernel, then the far field on the same stream
    EB_TRY(w.nearbuf.ensure(sizeof(double2) * (size_t)n));
    ProfScope pn(ctx, 2, st);
    k_near32<E><<<t.ntile, 128, 0, st>>>(t.tiles.as<int4>(), t.leaves.as<int>(), t.pt0.as<int>(), t.pt1.as<int>(),
                                         t.ustart.as<int>(), t.ulist.as<int>(), t.zhl.as<float4>(),
                                         w.pq.as<float2>(), w.aa.as<float2>(), w.qa.as<float2>(),
                                         w.nearbuf.as<double2>());
    eb_count_launch(ctx);
    pn.done();
  }
  ProfScope ps(ctx, 0, st);
  if (df && split) {
    k_leaf_df<E, 2><<<blocks, 128, 0, st>>>(
        t.ngroup, t.gleaf.as<int>(), t.gfirst.as<int>(), t.leaves.as<int>(), has_far, t.bkey.as<unsigned long long>(),
        t.blev.as<unsigned char>(), t.pt0.as<int>(), t.pt1.as<int>(), t.ustart.as<int>(), t.ulist.as<int>(),
        t.wstart.as<int>(), t.wlist.as<int>(), w.mpole_df.as<float4>(), t.perm.as<int>(),
        t.wdf.as<float4>(), t.wdf_lo.as<float2>(), w.pqdf.as<float4>(), w.aadf.as<float4>(), tb.p,
        (double)sign, w.local_df.as<float4>(), out, post, w.nearbuf.as<double2>());
  } else if (split) {
    k_far32<E><<<t.ntile, 128, far_sm, st>>>(t.tiles.as<int4>(), t.leaves.as<int>(),
                                             t.bkey.as<unsigned long long>(), t.blev.as<unsigned char>(),
                                             t.anc.as<int>(), t.wstart.as<int>(), t.wlist.as<int>(), t.perm.as<int>(),
                                             t.wdf.as<float4>(), tb.p, (float)sign, w.local.as<float2>(),
                                             w.mpole.as<float2>(), out, post, w.nearbuf.as<double2>());
  } else if (df) {
    k_leaf_df<E, 0><<<blocks, 128, 0, st>>>(
        t.ngroup, t.gleaf.as<int>(), t.gfirst.as<int>(), t.leaves.as<int>(), has_far, t.bkey.as<unsigned long long>(),
        t.blev.as<unsigned char>(), t.pt0.as<int>(), t.pt1.as<int>(), t.ustart.as<int>(), t.ulist.as<int>(),
        t.wstart.as<int>(), t.wlist.as<int>(), w.mpole_df.as<float4>(), t.perm.as<int>(),
        t.wdf.as<float4>(), t.wdf_lo.as<float2>(), w.pqdf.as<float4>(), w.aadf.as<float4>(), tb.p,
        (double)sign,
        w.local_df.as<float4>(), out, post, nullptr);
  } else if (f64) {
    k_leaf64<E><<<blocks, 128, 0, st>>>(
        t.ngroup, t.gleaf.as<int>(), t.gfirst.as<int>(), t.leaves.as<int>(), has_far, t.bkey.as<unsigned long long>(),
        t.blev.as<unsigned char>(), t.pt0.as<int>(), t.pt1.as<int>(), t.ustart.as<int>(), t.ulist.as<int>(),
        t.wstart.as<int>(), t.wlist.as<int>(), t.perm.as<int>(),
        t.zs.as<double2>(), w.pq.as<double2>(), w.aa.as<double2>(), w.qa.as<double2>(), t.x0, t.y0,
        t.W, tb.p, (double)sign, w.local.as<double2>(), w.mpole.as<double2>(), out, post);
  } else {
    k_far32<E><<<t.ntile, 128, far_sm, st>>>(t.tiles.as<int4>(), t.leaves.as<int>(),
                                             t.bkey.as<unsigned long long>(), t.blev.as<unsigned char>(),
                                             t.anc.as<int>(), t.wstart.as<int>(), t.wlist.as<int>(), t.perm.as<int>(),
                                             t.wdf.as<float4>(), tb.p, (float)sign, w.local.as<float2>(),
                                             w.mpole.as<float2>(), out, post, w.nearbuf.as<double2>());
  }
  eb_count_launch(ctx);
  if (E == 2 && t.wall && dz && !split) {  // the reflected near field, after the output is written
    const int ld = t.ld, nb = t.lev_off[ld + 1] - t.lev_off[ld];
    double2* dst = post.kind == 1 ? reinterpret_cast<double2*>(post.y) : out;
    k_img_near<<<nb, IMG_TILE, 0, st>>>(t.lev_off[ld], nb, ld, t.bkey.as<unsigned long long>(), t.pt0.as<int>(),
                                        t.pt1.as<int>(), t.zs.as<double2>(), t.perm.as<int>(), dens, dz, hpt,
                                        (double)sign, dst, 0);
    eb_count_launch(ctx);
  }
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
                 const double2* dens, const double2* dz, const double* hpt, double2* out,
                 const EbPost* post, cudaEvent_t join) {
  if (!t.valid) return EB_ERR_NOGEOM;
  if (kernel != 0) return EB_ERR_ARG;
  const bool df = precision == EB_PREC_DF || ctx->opts.df64 > 0;
  if (precision != EB_FP32) return fmm_run<double, 2>(ctx, t, sign, dens, dz, hpt, nullptr, out, post, join, df);
  return fmm_run<float, 2>(ctx, t, sign, dens, dz, hpt, nullptr, out, post, join, false);
}

int eb_fmm_apply_cauchy(eb_ctx* ctx, EbTree& t, int precision, const double2* q, double2* out,
                        const EbPost* post) {
  if (!t.valid) return EB_ERR_NOGEOM;
  const bool df = precision == EB_PREC_DF || ctx->opts.df64 > 0;
  if (precision != EB_FP32) return fmm_run<double, 1>(ctx, t, 0, nullptr, nullptr, nullptr, q, out, post, nullptr, df);
  return fmm_run<float, 1>(ctx, t, 0, nullptr, nullptr, nullptr, q, out, post, nullptr, false);
}
