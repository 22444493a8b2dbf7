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
};

// Per-node coefficients of the post-processing, formed once per geometry (they hold the
// FP64 divisions): FASMVP c1 = h s' kappa / (2 pi), c2 = c1 n^2 (stokesbubb.f:592-594);
// FASMVP_LAP d = 1 + 2 (h kappa s' / (4 pi)) - 2 h s' (laplace.f:233-241).
__device__ __forceinline__ void eb_post_coefs(int t, const double2* dz, const double* dsda,
                                              const double* kappa, const double* hpt, double* c1,
                                              double2* c2, double* d) {
  const double qwi = hpt[t], s = dsda[t], kap = kappa[t];
  const double2 zn = make_double2(dz[t].y / s, -dz[t].x / s);  // -i dz / s'
  const double a = qwi * s * 0.5 * kap / EB_PI;
  c1[t] = a;
  c2[t] = cscale<double>(cmul<double>(zn, zn), a);
  d[t] = 1.0 + 2.0 * (0.25 * qwi * kap * s / EB_PI) - 2.0 * (qwi * s);
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
    const double pinf = -P.pk[0];
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
