// Post-processing of an FMM sum at one node, fused into the epilogue of the leaf
// kernels so that an operator apply writes its result directly.
#pragma once

#include "eb_common.cuh"

struct EbPost {
  int kind;               // 0: store the sum; 1: FASMVP; 2: FASMVP_LAP
  const double2* dens;    // kind 1: complex density
  const double* u;        // kind 2: real density
  const double2* z;
  const double2* dz;
  const double* dsda;
  const double* kappa;
  const double* hpt;      // per-node weight 2 pi / nd of the node's drop
  const int* drop_of;
  const double2* za;      // kind 1: per-drop h sum(dens)
  const double* pk;       // kind 1: per-drop singular-term sums
  double* y;              // kind 1: complex w (interleaved); kind 2: real w
};

// kind 1: identity, self and singular terms of FASMVP (stokesbubb.f:585-612) added to
// the CADAPDR sum `stress`; kind 2: the discrete operator of FASMVP_LAP
// (laplace.f:225-243) from the Cauchy sum cf.
__device__ __forceinline__ void eb_post_store(const EbPost& P, int t, double2 g, double2* out) {
  if (P.kind == 0) {
    out[t] = g;
  } else if (P.kind == 1) {
    const int b = P.drop_of[t];
    const double2 u = P.dens[t];
    const double qwi = P.hpt[t], s = P.dsda[t], kap = P.kappa[t];
    const double2 zn = make_double2(P.dz[t].y / s, -P.dz[t].x / s);  // -i dz / s'
    const double c1 = qwi * s * 0.5 * kap / EB_PI;
    const double2 zn2 = cmul<double>(zn, zn);
    double2 zself = cscale<double>(u, c1);
    zself = csub<double>(zself, cscale<double>(cmul<double>(cconj<double>(u), zn2), c1));
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
    const double hs = P.hpt[t], ut = P.u[t];
    const double self = 0.25 * hs * P.kappa[t] * P.dsda[t] / EB_PI;
    // Re(cf / (2 pi i)) = Im(cf) / (2 pi)
    const double zc = self * ut - g.y / (2.0 * EB_PI);
    P.y[t] = ut + 2.0 * zc - 2.0 * (hs * ut * P.dsda[t]);
  }
}
