// Transposed (adjoint) operators of the two solves, for reverse-mode gradients of what a
// solve produces with respect to its right-hand side. The reference has no adjoint; these
// are the exact transposes (for the real inner product of the solver's unknowns) of
// FASMVP (stokesbubb.f:496-614) and FASMVP_LAP (laplace.f:159-262) as this library
// applies them, built from the same FMM.
//
// Stokes. FASMVP maps the complex density u to w = u + za_k + GW(u) + zself(u)
// + (i/2) raw_k z with za_k = h_k sum_{drop k} u, zself = c1 u - c2 conj(u),
// raw_k = sum_{drop k} Re(u pkw) (pinf cancels: pinf - pk_k = -raw_k), and the sum
// GW_i = sum_{j != i} a_ij u_j + b_ij conj(u_j) with, for D = z_j - z_i and
// alpha_j = dz_j h_j / (2 pi i),
//   a_ij = alpha_j / D + conj(alpha_j) / conj(D),
//   b_ij = -alpha_j / conj(D) + D conj(alpha_j / D^2)      (the CADAPDR sign s = -1).
// A map u -> a u + b conj(u) has the transpose v -> conj(a) v + b conj(v), so
//   (GW^T v)_j = 2 alpha_j Re(S1_j) - conj(alpha_j) X_j,
// where S1_j = sum_{i != j} v_i / (z_j - z_i) (a Cauchy sum with charges v) and X_j is
// z conj(phi') + conj(psi) of the Stokes sum with charges qa = -v, qb = conj(v) at the
// nodes (its phi is S1, so X = GW_+1 - S1 with the CADAPMOD sign). The remaining terms
// transpose to h_k sum_{drop k} v, c1 v - c2 conj(v) and conj(pkw_j) R_k with
// R_k = sum_{drop k} Re(conj(v) (i/2) z).
//
// Laplace. FASMVP_LAP maps the real density u to w_i = d_i u_i - Im(F_i) / pi with
// F_i = sum_{j != i} u_j h_j dz_j / (z_i - z_j); its transpose is
//   (A^T v)_j = d_j v_j + (h_j / pi) Im(dz_j F'_j),  F'_j = sum_{i != j} v_i / (z_j - z_i).
//
// Both are FP64 sums of FMM results (native, double-float or FP32 FMMs, as the
// precision asks). The wall's images are not part of the transposes.
#include <algorithm>
#include <cmath>

#include "eb_internal.h"

namespace {

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

// Per drop: sv_k = sum v and R_k = sum Re(conj(v) (i/2) z). One block per drop.
__global__ void k_adj_drop_reduce(const int* __restrict__ start, const double2* __restrict__ v,
                                  const double2* __restrict__ z, double2* __restrict__ sv,
                                  double* __restrict__ rk) {
  __shared__ double s[3][256];
  const int b = blockIdx.x, i0 = start[b], i1 = start[b + 1];
  double ax = 0.0, ay = 0.0, rr = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double2 u = v[i], zz = z[i];
    ax += u.x;
    ay += u.y;
    rr = fma(0.5 * u.y, zz.x, fma(-0.5 * u.x, zz.y, rr));  // Re(conj(v) i z / 2)
  }
  s[0][threadIdx.x] = ax;
  s[1][threadIdx.x] = ay;
  s[2][threadIdx.x] = rr;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s[0][threadIdx.x] += s[0][threadIdx.x + o];
      s[1][threadIdx.x] += s[1][threadIdx.x + o];
      s[2][threadIdx.x] += s[2][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    sv[b] = make_double2(s[0][0], s[1][0]);
    rk[b] = s[2][0];
  }
}

__global__ void k_stokes_adj_post(int n, const int* __restrict__ drop_of, const double2* __restrict__ v,
                                  const double2* __restrict__ dz, const double* __restrict__ hpt,
                                  const double* __restrict__ c1, const double2* __restrict__ c2,
                                  const double2* __restrict__ pkw, const double2* __restrict__ s1,
                                  const double2* __restrict__ gwp, const double2* __restrict__ sv,
                                  const double* __restrict__ rk, double2* __restrict__ y) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int k = drop_of[j];
  const double2 u = v[j], d = dz[j], S1 = s1[j];
  const double h = hpt[j], f = h / (2.0 * EB_PI);
  const double2 al = make_double2(d.y * f, -d.x * f);  // dz h / (2 pi i)
  const double2 X = csub<double>(gwp[j], S1);
  double2 r = u;
  r = cadd<double>(r, cscale<double>(sv[k], h));                                             // za^T
  r = cadd<double>(r, csub<double>(cscale<double>(u, c1[j]), cmul<double>(c2[j], cconj<double>(u))));  // zself^T
  r = cadd<double>(r, csub<double>(cscale<double>(al, 2.0 * S1.x), cmul<double>(cconj<double>(al), X)));  // GW^T
  r = cadd<double>(r, cscale<double>(cconj<double>(pkw[j]), rk[k]));                      // pressure^T
  y[j] = r;
}

__global__ void k_real_to_cplx(int n, const double* __restrict__ v, double2* __restrict__ q) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[i] = make_double2(v[i], 0.0);
}

__global__ void k_lap_adj_post(int n, const double* __restrict__ v, const double2* __restrict__ dz,
                               const double* __restrict__ hpt, const double* __restrict__ d,
                               const double2* __restrict__ f, double* __restrict__ y) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double2 a = dz[j], F = f[j];
  y[j] = fma(d[j], v[j], hpt[j] * (a.x * F.y + a.y * F.x) * (1.0 / EB_PI));
}

int check_adj(eb_ctx* ctx) {
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (ctx->iwall) {
    eb_set_last_error_msg("the transposed operators do not include the wall's images");
    return EB_ERR_ARG;
  }
  return EB_OK;
}

}  // namespace

int eb_stokes_matvec_adj_dev(eb_ctx* ctx, const double* x, double* y, int prec) {
  EB_TRY(check_adj(ctx));
  cudaStream_t s = ctx->stream;
  const int n = ctx->nbk, k = ctx->k;
  const double2* v = reinterpret_cast<const double2*>(x);
  EB_TRY(ctx->adj_a.ensure(sizeof(double2) * (size_t)n));
  EB_TRY(ctx->adj_b.ensure(sizeof(double2) * (size_t)n));
  EB_TRY(ctx->adj_s.ensure((sizeof(double2) + sizeof(double)) * (size_t)k));
  double2* s1 = ctx->adj_a.as<double2>();
  double2* gwp = ctx->adj_b.as<double2>();
  double2* sv = ctx->adj_s.as<double2>();
  double* rk = reinterpret_cast<double*>(sv + k);
  k_adj_drop_reduce<<<k, 256, 0, s>>>(ctx->start.as<int>(), v, ctx->z.as<double2>(), sv, rk);
  eb_count_launch(ctx);
  EB_TRY(eb_fmm_apply_cauchy(ctx, ctx->tree, prec, v, s1, nullptr));
  EB_TRY(eb_fmm_apply(ctx, ctx->tree, 0, +1, prec, v, nullptr, nullptr, gwp));
  k_stokes_adj_post<<<nblk(n, 256), 256, 0, s>>>(n, ctx->drop_of.as<int>(), v, ctx->dz.as<double2>(),
                                                 ctx->hpt.as<double>(), ctx->pc1.as<double>(),
                                                 ctx->pc2.as<double2>(), ctx->pkw.as<double2>(), s1, gwp, sv, rk,
                                                 reinterpret_cast<double2*>(y));
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "stokes matvec adjoint");
}

int eb_laplace_matvec_adj_dev(eb_ctx* ctx, const double* x, double* y, int prec) {
  EB_TRY(check_adj(ctx));
  cudaStream_t s = ctx->stream;
  const int n = ctx->nbk;
  EB_TRY(ctx->adj_a.ensure(sizeof(double2) * (size_t)n));
  EB_TRY(ctx->adj_b.ensure(sizeof(double2) * (size_t)n));
  double2* q = ctx->adj_a.as<double2>();
  double2* f = ctx->adj_b.as<double2>();
  k_real_to_cplx<<<nblk(n, 256), 256, 0, s>>>(n, x, q);
  eb_count_launch(ctx);
  EB_TRY(eb_fmm_apply_cauchy(ctx, ctx->tree, prec, q, f, nullptr));
  k_lap_adj_post<<<nblk(n, 256), 256, 0, s>>>(n, x, ctx->dz.as<double2>(), ctx->hpt.as<double>(),
                                              ctx->plap.as<double>(), f, y);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "laplace matvec adjoint");
}

namespace {
template <typename F>
int run_adj(eb_ctx* ctx, const double* x, double* y, size_t nd, int mem, F f) {
  if (mem == EB_DEVICE) return f(x, y);
  if (mem != EB_HOST) return EB_ERR_ARG;
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->vin.ensure(sizeof(double) * nd));
  EB_TRY(ctx->vout.ensure(sizeof(double) * nd));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, x, sizeof(double) * nd, cudaMemcpyHostToDevice, s));
  EB_TRY(f(ctx->vin.as<double>(), ctx->vout.as<double>()));
  EB_CUDA_TRY(cudaMemcpyAsync(y, ctx->vout.p, sizeof(double) * nd, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}
}  // namespace

int eb_stokes_matvec_adjoint(eb_ctx* ctx, int n, const double* x, double* y, int prec, int mem) {
  if (!ctx || !x || !y) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != 2 * ctx->nbk || (prec != EB_FP64 && prec != EB_FP32)) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return run_adj(ctx, x, y, (size_t)n, mem,
                 [&](const double* xd, double* yd) { return eb_stokes_matvec_adj_dev(ctx, xd, yd, prec); });
}

int eb_laplace_matvec_adjoint(eb_ctx* ctx, int n, const double* x, double* y, int prec, int mem) {
  if (!ctx || !x || !y) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != ctx->nbk || (prec != EB_FP64 && prec != EB_FP32)) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return run_adj(ctx, x, y, (size_t)n, mem,
                 [&](const double* xd, double* yd) { return eb_laplace_matvec_adj_dev(ctx, xd, yd, prec); });
}
