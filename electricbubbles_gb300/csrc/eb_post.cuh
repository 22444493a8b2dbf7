// Post-processing of an FMM sum at one node, fused into the epilogue of the leaf
// kernels so that an operator apply writes its result directly.
#pragma once

#include "eb_common.cuh"

struct EbPost {
  int kind;               // 0: store the sum; 1: FASMVP; 2: FASMVP_LAP
  const double2* dens;    // kind 1: complex density
  const double* u;        // kind 2: real density
  const double2* z;
  const double2* dz;      // Cauchy charges from u (kind 2)
  const double* hpt;      // per-node weight 2 pi / nd of the node's drop
  const double* c1;       // per node (eb_post_coefs): kind 1 h s' kappa / (2 pi); kind 2 the diagonal
  const double2* c2;      // kind 1, per node: c1 n^2 with n = -i dz / s'
  const int* drop_of;
  const double2* za;      // kind 1: per-drop h sum(dens)
  const double* pk;       // kind 1: per-drop singular-term sums
  double* y;              // kind 1: complex w (interleaved); kind 2: real w
  const float* c1f;       // float copies of c1 and c2 for the FP32 operator
  const float2* c2f;
  const int* pinf_drop;   // kind 1: per drop, the drop whose pressure is pinf (the first
                          // drop of its simulation); null: drop 0
};

// Per-node coefficients of the post-processing, formed once per geometry (they hold the
// FP64 divisions): FASMVP c1 = h s' kappa / (2 pi), c2 = c1 n^2 (stokesbubb.f:592-594);
// FASMVP_LAP d = 1 + 2 (h kappa s' / (4 pi)) - 2 h s' (laplace.f:233-241).
__device__ __forceinline__ void eb_post_coefs(int t, const double2* dz, const double* dsda,
                                              const double* kappa, const double* hpt, double* c1,
                                              double2* c2, double* d, float* c1f, float2* c2f,
                                              float* df) {
  const double qwi = hpt[t], s = dsda[t], kap = kappa[t];
  const double2 zn = make_double2(dz[t].y / s, -dz[t].x / s);  // -i dz / s'
  const double a = qwi * s * 0.5 * kap / EB_PI;
  const double2 b = cscale<double>(cmul<double>(zn, zn), a);
  const double dd = 1.0 + 2.0 * (0.25 * qwi * kap * s / EB_PI) - 2.0 * (qwi * s);
  c1[t] = a;
  c2[t] = b;
  d[t] = dd;
  c1f[t] = (float)a;
  c2f[t] = make_float2((float)b.x, (float)b.y);
  df[t] = (float)dd;
}

// The same post-processing for the FP32 operator: everything but the identity term in
// FP32 (the operator's own error is ~1e-6), so that the FP64 pipe sees two additions.
__device__ __forceinline__ void eb_post_store_f32(const EbPost& P, int t, float2 g, double2* out) {
  if (P.kind == 0) {
    out[t] = make_double2((double)g.x, (double)g.y);
  } else if (P.kind == 1) {
    const int b = P.drop_of[t];
    const double2 ud = P.dens[t];
    const float2 u = make_float2((float)ud.x, (float)ud.y);
    const float c1 = P.c1f[t];
    const float2 c2 = P.c2f[t];
    const float2 zself = make_float2(c1 * u.x - (u.x * c2.x + u.y * c2.y), c1 * u.y - (u.x * c2.y - u.y * c2.x));
    const float pinf = -(float)P.pk[P.pinf_drop ? P.pinf_drop[b] : 0];
    const float pkb = (float)P.pk[b] + pinf;
    const float f = -0.5f * (pinf - pkb);
    const double2 zz = P.z[t];
    const double2 zab = P.za[b];
    const float rx = (float)zab.x + g.x + zself.x - f * (float)zz.y;
    const float ry = (float)zab.y + g.y + zself.y + f * (float)zz.x;
    reinterpret_cast<double2*>(P.y)[t] = make_double2(ud.x + (double)rx, ud.y + (double)ry);
  } else {
    const double ut = P.u[t];
    const float r = (P.c1f[t] - 1.0f) * (float)ut - g.y * 0.318309886f;
    P.y[t] = ut + (double)r;
  }
}

// kind 1: identity, self and singular terms of FASMVP (stokesbubb.f:585-612) added to
// the CADAPDR sum `stress`; kind 2: the discrete operator of FASMVP_LAP
// (laplace.f:225-243) from the Cauchy sum cf: w = d u - Im(cf) / pi.
__device__ __forceinline__ void eb_post_store(const EbPost& P, int t, double2 g, double2* out) {
  if (P.kind == 0) {
    out[t] = g;
  } else if (P.kind == 1) {
    const int b = P.drop_of[t];
    const double2 u = P.dens[t];
    const double c1 = P.c1[t];
    // zself = c1 u - c1 conj(u) n^2
    const double2 zself = csub<double>(cscale<double>(u, c1), cmul<double>(cconj<double>(u), P.c2[t]));
    const double pinf = -P.pk[P.pinf_drop ? P.pinf_drop[b] : 0];
    const double pkb = P.pk[b] + pinf;
    const double f = -0.5 * (pinf - pkb);  // times i z
    const double2 zz = P.z[t];
    double2 st = g;
    st.x += zself.x - f * zz.y;
    st.y += zself.y + f * zz.x;
    const double2 zab = P.za[b];
    reinterpret_cast<double2*>(P.y)[t] = make_double2(u.x + zab.x + st.x, u.y + zab.y + st.y);
  } else {
    constexpr double inv_pi = 0.318309886183790671537767526745028724;
    P.y[t] = fma(P.c1[t], P.u[t], -g.y * inv_pi);
  }
}
