// GMRES on the GPU with the semantics of SLATEC DGMRES as SOLVEI / SOLVE_LAPL call it
// (stokesbubb.f:330-350, laplace.f:361-382): x0 = rhs, MAXL Krylov vectors, no
// restart, no preconditioner (JPRE = 0; the deflated Laplace solve below is the one
// option that adds one), stop when the Givens estimate of ||b - A x|| / ||b||
// (DPIGMR's RHO, dpigmr.f:340-355) is at most TOL (ISDGMR with ITOL = 0).
//
// The Krylov basis, residuals and the solution update stay FP64 in HBM. The Arnoldi
// step orthogonalises with classical Gram-Schmidt applied twice (two batched
// projections V^T w and w -= V h) instead of DORTH's modified Gram-Schmidt
// (dorth.f:90-123): the same basis in exact arithmetic, orthogonal to working
// precision, and 4 launches per step instead of 2*ll dependent ones. The
// (MAXL+1) x MAXL Hessenberg matrix, its Givens rotations (DHEQR, dheqr.f:82-176) and
// the triangular solve (DHELS, dhels.f:77-96) are O(MAXL^2) and run on the host.
//
// Refined mode (FP32 inner operator): iterative refinement with FP64 residuals from
// x = 0 (so r = b needs no apply),
//   solve A32 d = r to inner_tol with the same GMRES;  x += d;  r = b - A64 x,
// until ||r|| / ||b|| <= TOL; the reported error is the true FP64 residual. Steps after
// the first tighten the inner tolerance (to at most a tenth) when that is expected to
// end the solve (inner_tolerance below). The inner cycle orthogonalises with one
// Gram-Schmidt pass (its tolerance is far above the loss of orthogonality) and takes
// the new vector's norm by Pythagoras, ||w - V h||^2 = w.w - h.h, from the reduction
// that forms h = V^T w, so that a step is the apply, one reduction and one update.
//
// Deflated Laplace solve (eb_opts.lap_deflate): the same GMRES, both modes, on the
// right-preconditioned operator A M^-1 in the variable t = M x (k_deflate below), from
// t0 = M rhs; x = M^-1 t at the end. Its residual b - A M^-1 t is b - A x, so the
// stopping test and the reported error are those of the unpreconditioned solve.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#include "eb_internal.h"

namespace {

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }
constexpr int RBS = 256;   // reduction block size
// Reduction grids: at most two blocks per SM of the context's GPU.
inline int rmaxb(const eb_ctx* ctx) { return 2 * ctx->nsm; }

__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum<double>(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
    r = warp_sum<double>(r);
  }
  __syncthreads();
  return r;
}

// Sums part[blk * ncol + j] over the blocks into out[j] (one warp per column, fixed
// order); run by the last block of a kernel to finish, which also resets the ticket.
// Returns true in that block.
__device__ bool finish_columns(int nb, int ncol, const double* part, double* out,
                               unsigned int* ticket) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j = w; j < ncol; j += nw) {
    double s = 0.0;
    for (int b = lane; b < nb; b += 32) s += __ldcg(part + (size_t)b * ncol + j);
    s = warp_sum<double>(s);
    if (lane == 0) out[j] = s;
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// The block's partial sums of V[:, j] . w for j < ncol, and with with_w of w . w as
// column ncol, into part[blockIdx.x * (ncol + with_w) + j]. Each block takes a
// contiguous range of rows and each of its warps a subset of the columns.
__device__ __forceinline__ void vtw_partials(int n, int ncol, int with_w, const double* __restrict__ V,
                                             size_t ldv, const double* __restrict__ w,
                                             double* __restrict__ part) {
  const int nc = ncol + with_w;
  const int rows = (n + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * rows, r1 = min(n, r0 + rows);
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j = wi; j < nc; j += nw) {
    const double* v = j < ncol ? V + (size_t)j * ldv : w;
    double s = 0.0;
    for (int i = r0 + lane; i < r1; i += 32) s = fma(v[i], w[i], s);
    s = warp_sum<double>(s);
    if (lane == 0) part[(size_t)blockIdx.x * nc + j] = s;
  }
}

// out[j] = V[:, j] . w for j < ncol (and out[ncol] = w . w with with_w); partial sums
// per block go to `part` and the last block to finish adds them in block order.
__global__ void k_vtw(int n, int ncol, const int* __restrict__ ncol_dev, const double* __restrict__ V,
                      size_t ldv, const double* __restrict__ w, double* __restrict__ part,
                      double* __restrict__ out, unsigned int* __restrict__ ticket, int with_w = 0) {
  if (ncol_dev) ncol = *ncol_dev;
  vtw_partials(n, ncol, with_w, V, ldv, w, part);
  finish_columns(gridDim.x, ncol + with_w, part, out, ticket);
}

// Norm of the new Arnoldi vector w - V h of one Gram-Schmidt pass, from h = V^T w and
// s = w . w (Pythagoras, V orthonormal): ||w - V h||^2 = s - sum h_i^2. The same
// explicit fma sequence on the host and the device. With the difference at most 1e-12 s
// (the new direction is lost in rounding) the vector counts as zero: the Krylov space
// is invariant to working precision (DPIGMR's SNORMW = 0).
__host__ __device__ inline double pyth_norm2(const double* h, int ncol, double s) {
  double t = s;
  for (int i = 0; i < ncol; ++i) t = fma(-h[i], h[i], t);
  return t > 1e-12 * s ? t : 0.0;
}

// dst = (w - V[:, 0:ncol] h) * scale, and xin = the same when xin != nullptr (dst may be w).
__device__ __forceinline__ void sub_scale_store(int n, int ncol, const double* __restrict__ V, size_t ldv,
                                                const double* __restrict__ h, const double* w, double scale,
                                                double* dst, double* __restrict__ xin) {
  __shared__ double hs[128];
  for (int j = threadIdx.x; j < ncol; j += blockDim.x) hs[j] = h[j];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < ncol; ++j) acc = fma(V[(size_t)j * ldv + i], hs[j], acc);
    const double v = (w[i] - acc) * scale;
    dst[i] = v;
    if (xin) xin[i] = v;
  }
}

__global__ void k_sub_scale(int n, int ncol, const double* __restrict__ V, size_t ldv,
                            const double* __restrict__ h, double* w, double scale) {
  sub_scale_store(n, ncol, V, ldv, h, w, scale, w, nullptr);
}

// Pass-1 update fused with the pass-2 projection of classical Gram-Schmidt: each block
// updates its contiguous range of rows, w -= V[:, 0:ncol] hin, and then forms the
// block's partial V^T w for those rows exactly as k_vtw does (warps over columns, lanes
// over rows); the last block adds the partials in block order.
__global__ void k_update_vtw(int n, int ncol, const int* __restrict__ ncol_dev, const double* __restrict__ V,
                             size_t ldv, const double* __restrict__ hin, double* w,
                             double* __restrict__ part, double* __restrict__ out,
                             unsigned int* __restrict__ ticket) {
  __shared__ double hs[128];
  if (ncol_dev) ncol = *ncol_dev;
  for (int j = threadIdx.x; j < ncol; j += blockDim.x) hs[j] = hin[j];
  __syncthreads();
  const int rows = (n + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * rows, r1 = min(n, r0 + rows);
  for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < ncol; ++j) acc = fma(V[(size_t)j * ldv + i], hs[j], acc);
    w[i] -= acc;
  }
  __syncthreads();
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j = wi; j < ncol; j += nw) {
    const double* v = V + (size_t)j * ldv;
    double sum = 0.0;
    for (int i = r0 + lane; i < r1; i += 32) sum = fma(v[i], w[i], sum);
    sum = warp_sum<double>(sum);
    if (lane == 0) part[(size_t)blockIdx.x * ncol + j] = sum;
  }
  finish_columns(gridDim.x, ncol, part, out, ticket);
}

// w -= V[:, 0:ncol] h; if part != nullptr also ||w||^2 of the new w into *out (returns
// true in the block that wrote it).
__device__ bool gemv_sub(int n, int ncol, const int* __restrict__ ncol_dev, const double* __restrict__ V,
                         size_t ldv, const double* __restrict__ h, double* __restrict__ w,
                         double* __restrict__ part, double* __restrict__ out,
                         unsigned int* __restrict__ ticket) {
  __shared__ double hs[128];
  if (ncol_dev) ncol = *ncol_dev;
  __shared__ double red[32];
  for (int j = threadIdx.x; j < ncol; j += blockDim.x) hs[j] = h[j];
  __syncthreads();
  double sq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < ncol; ++j) acc = fma(V[(size_t)j * ldv + i], hs[j], acc);
    double v = w[i] - acc;
    w[i] = v;
    sq = fma(v, v, sq);
  }
  if (!part) return false;
  sq = block_sum(sq, red);
  if (threadIdx.x == 0) part[blockIdx.x] = sq;
  return finish_columns(gridDim.x, 1, part, out, ticket);
}

__global__ void k_gemv_sub(int n, int ncol, const int* __restrict__ ncol_dev, const double* __restrict__ V,
                           size_t ldv, const double* __restrict__ h, double* __restrict__ w,
                           double* __restrict__ part, double* __restrict__ out,
                           unsigned int* __restrict__ ticket) {
  gemv_sub(n, ncol, ncol_dev, V, ldv, h, w, part, out, ticket);
}

// x += V[:, 0:ncol] y
__global__ void k_gemv_add(int n, int ncol, const double* __restrict__ V, size_t ldv,
                           const double* __restrict__ y, double* __restrict__ x) {
  __shared__ double ys[128];
  for (int j = threadIdx.x; j < ncol; j += blockDim.x) ys[j] = y[j];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < ncol; ++j) acc = fma(V[(size_t)j * ldv + i], ys[j], acc);
    x[i] += acc;
  }
}

// out = a - y (residual; y may be out), with ||out||^2 into *nrm2.
__global__ void k_resid(int n, const double* __restrict__ a, const double* y, double* out,
                        double* __restrict__ part, double* __restrict__ nrm2,
                        unsigned int* __restrict__ ticket) {
  __shared__ double red[32];
  double sq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = a[i] - y[i];
    out[i] = v;
    sq = fma(v, v, sq);
  }
  sq = block_sum(sq, red);
  if (threadIdx.x == 0) part[blockIdx.x] = sq;
  finish_columns(gridDim.x, 1, part, nrm2, ticket);
}

__global__ void k_scale(int n, double s, double* __restrict__ v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] *= s;
}

__global__ void k_axpy(int n, double s, const double* __restrict__ a, double* __restrict__ v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] += s * a[i];
}

typedef int (*op_fn)(eb_ctx*, const double*, double*, int);

struct Gm {
  eb_ctx* ctx;
  int n;
  int nb;  // reduction blocks
  cudaStream_t s;
  unsigned int* ticket;  // last-block counter of the reduction kernels
};

// ||v||^2 into host
int dev_sumsq(Gm& g, const double* v, double* out) {
  eb_ctx* ctx = g.ctx;
  double* part = ctx->gPart.as<double>();
  k_vtw<<<g.nb, RBS, 0, g.s>>>(g.n, 1, nullptr, v, (size_t)g.n, v, part, ctx->gH.as<double>(), g.ticket);
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemcpyAsync(out, ctx->gH.p, sizeof(double), cudaMemcpyDeviceToHost, g.s));
  EB_CUDA_TRY(cudaStreamSynchronize(g.s));
  return EB_OK;
}

// DHEQR column update (IJOB > 1 form; identical to IJOB = 1 for the first column).
// Runs on the host (host-driven loop) and in the device Arnoldi kernel (graph mode).
__host__ __device__ inline int dheqr_col(double* hes, int ldh, int ll, double* q) {
  double* a = hes + (size_t)(ll - 1) * ldh;
  for (int k = 0; k < ll - 1; ++k) {
    double c = q[2 * k], s = q[2 * k + 1], t1 = a[k], t2 = a[k + 1];
    a[k] = c * t1 - s * t2;
    a[k + 1] = s * t1 + c * t2;
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

void dhels(const double* hes, int ldh, int ll, const double* q, double* b) {
  for (int k = 0; k < ll; ++k) {
    double c = q[2 * k], s = q[2 * k + 1], t1 = b[k], t2 = b[k + 1];
    b[k] = c * t1 - s * t2;
    b[k + 1] = s * t1 + c * t2;
  }
  for (int kb = 0; kb < ll; ++kb) {
    int k = ll - 1 - kb;
    b[k] /= hes[(size_t)k * ldh + k];
    double t = -b[k];
    for (int r = 0; r < k; ++r) b[r] += t * hes[(size_t)k * ldh + r];
  }
}

// Deflation of each drop's constant density for the Laplace solve. FASMVP_LAP
// (laplace.f:159-262) maps the constant 1 on drop k to -2 h_k s'_i on that drop and to
// zero elsewhere (the double layer of a constant vanishes off its curve and cancels the
// identity on it, leaving the -2 h u s' term of laplace.f:235-236), so with nodes
// equispaced in arclength the k constants are eigenvectors with the small, distinct
// eigenvalues mu_k = -2 h_k mean_k(s'), and unpreconditioned GMRES spends about one
// iteration on each. With P_k the mean over drop k spread over its nodes,
//   M^-1 = I + sum_k (1/mu_k - 1) P_k,   M = I + sum_k (mu_k - 1) P_k,
// and A M^-1 maps those modes to about 1 while leaving vectors of zero drop means alone.
// The coefficients are formed once per solve (k_deflate_coef: coef_k = (1/mu_k - 1,
// mu_k - 1), zero for a drop whose mu_k is not negative and finite); every application
// is then one block per drop: y = x + c_k mean_k(x) with c_k = coef_k.x (inverse = 1, M^-1)
// or coef_k.y (inverse = 0, M). y may alias x: every read of the drop precedes the writes.
constexpr int DEFL_BS = 256;
__global__ void __launch_bounds__(DEFL_BS) k_deflate_coef(const int* __restrict__ start,
                                                          const double* __restrict__ dsda,
                                                          double2* __restrict__ coef) {
  __shared__ double red[DEFL_BS / 32];
  const int b = blockIdx.x, i0 = start[b], i1 = start[b + 1];
  double ss = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += DEFL_BS) ss += dsda[i];
  ss = block_sum(ss, red);
  if (threadIdx.x == 0) {
    const int n = i1 - i0;
    double2 c = make_double2(0.0, 0.0);
    if (n > 0) {
      const double mu = -4.0 * EB_PI * ss / ((double)n * (double)n);  // -2 (2 pi / n) (ss / n)
      if (mu < 0.0 && isfinite(mu)) c = make_double2(1.0 / mu - 1.0, mu - 1.0);
    }
    coef[b] = c;
  }
}

__global__ void __launch_bounds__(DEFL_BS) k_deflate(const int* __restrict__ start,
                                                     const double2* __restrict__ coef, const double* x,
                                                     double* y, int inverse) {
  __shared__ double red[DEFL_BS / 32];
  __shared__ double s_add;
  const int b = blockIdx.x, i0 = start[b], i1 = start[b + 1];
  double sx = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += DEFL_BS) sx += x[i];
  sx = block_sum(sx, red);
  if (threadIdx.x == 0) {
    const int n = i1 - i0;
    const double2 c = coef[b];
    s_add = n > 0 ? (inverse ? c.x : c.y) * (sx / n) : 0.0;
  }
  __syncthreads();
  const double a = s_add;
  for (int i = i0 + threadIdx.x; i < i1; i += DEFL_BS) y[i] = x[i] + a;
}

int deflate(eb_ctx* ctx, const double* x, double* y, int inverse) {
  k_deflate<<<ctx->k, DEFL_BS, 0, ctx->stream>>>(ctx->start.as<int>(), ctx->gDeflC.as<double2>(), x, y, inverse);
  eb_count_launch(ctx);
  return EB_OK;
}

// y = A M^-1 x: the operator of the deflated Laplace solve
int laplace_matvec_deflated(eb_ctx* ctx, const double* x, double* y, int prec) {
  double* t = ctx->gDefl.as<double>();
  EB_TRY(deflate(ctx, x, t, 1));
  return eb_laplace_matvec_dev(ctx, t, y, prec);
}

// One GMRES cycle (DGMRES with NRMAX = 0). x holds x0 on entry unless x0_zero.
// Returns the DGMRES IERR convention in *ierr.
int gmres_cycle(Gm& g, op_fn op, int prec, const double* b, double* x, bool x0_zero,
                double tol, int maxl, int* iters, double* err, int* ierr, int* nmv,
                double bnrm_in) {
  eb_ctx* ctx = g.ctx;
  const int n = g.n;
  if (maxl > n) maxl = n;
  const size_t ldv = (size_t)n;
  const int ldh = maxl + 1;
  // classical Gram-Schmidt twice for the FP64 solve; once for the inner FP32 cycle of
  // the refined solve, whose tolerance (1e-5) is far above the loss of orthogonality
  const bool cgs2 = prec == EB_FP64;
  EB_TRY(ctx->gV.ensure(sizeof(double) * ldv * (maxl + 1)));
  double* V = ctx->gV.as<double>();
  double* part = ctx->gPart.as<double>();
  double* hdev = ctx->gH.as<double>();
  std::vector<double> hes((size_t)ldh * maxl, 0.0), q(2 * maxl, 0.0), y(maxl + 1, 0.0);
  std::vector<double> hbuf(3 * (maxl + 2), 0.0);
  double bnrm = bnrm_in;
  if (bnrm < 0) {
    double ss;
    EB_TRY(dev_sumsq(g, b, &ss));
    bnrm = std::sqrt(ss);
  }
  *iters = 0;
  *ierr = 0;
  if (!(bnrm > 0.0) || !std::isfinite(bnrm)) {
    *err = 0.0;
    if (!std::isfinite(bnrm)) {
      eb_set_last_error_msg("non-finite right-hand side");
      return EB_ERR_NAN;
    }
    // b = 0: the solution is x = 0 (DGMRES would divide by zero)
    EB_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, g.s));
    return EB_OK;
  }
  // r0 = b - A x0
  if (x0_zero) {
    EB_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, g.s));
    EB_CUDA_TRY(cudaMemcpyAsync(V, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, g.s));
  } else {
    EB_TRY(op(ctx, x, V, prec));
    (*nmv)++;
    k_resid<<<g.nb, RBS, 0, g.s>>>(n, b, V, V, part, hdev, g.ticket);
    eb_count_launch(ctx);
  }
  double ss;
  if (x0_zero) {
    EB_TRY(dev_sumsq(g, V, &ss));
  } else {
    EB_CUDA_TRY(cudaMemcpyAsync(&ss, hdev, sizeof(double), cudaMemcpyDeviceToHost, g.s));
    EB_CUDA_TRY(cudaStreamSynchronize(g.s));
  }
  double r0nrm = std::sqrt(ss);
  *err = r0nrm / bnrm;
  if (!std::isfinite(r0nrm)) {
    eb_set_last_error_msg("non-finite residual");
    return EB_ERR_NAN;
  }
  if (*err <= tol) return EB_OK;
  k_scale<<<g.nb, RBS, 0, g.s>>>(n, 1.0 / r0nrm, V);
  eb_count_launch(ctx);
  double prod = 1.0, rho = r0nrm;
  int ll, iflag = 1, lgmr = 0;
  for (ll = 1; ll <= maxl; ++ll) {
    lgmr = ll;
    double* w = V + (size_t)ll * ldv;
    EB_TRY(op(ctx, V + (size_t)(ll - 1) * ldv, w, prec));
    (*nmv)++;
    double* col = hes.data() + (size_t)(ll - 1) * ldh;
    double snormw;
    if (cgs2) {
      // pass 1: h1 = V^T w; w -= V h1; pass 2: h2 = V^T w; w -= V h2 with ||w||^2
      k_vtw<<<g.nb, RBS, 0, g.s>>>(n, ll, nullptr, V, ldv, w, part, hdev, g.ticket);
      k_update_vtw<<<g.nb, RBS, 0, g.s>>>(n, ll, nullptr, V, ldv, hdev, w, part, hdev + (maxl + 2), g.ticket);
      k_gemv_sub<<<g.nb, RBS, 0, g.s>>>(n, ll, nullptr, V, ldv, hdev + (maxl + 2), w, part,
                                        hdev + 2 * (maxl + 2), g.ticket);
      ctx->launches += 3;
      EB_CUDA_TRY(cudaMemcpyAsync(hbuf.data(), hdev, sizeof(double) * 3 * (maxl + 2),
                                  cudaMemcpyDeviceToHost, g.s));
      EB_CUDA_TRY(cudaStreamSynchronize(g.s));
      for (int i = 0; i < ll; ++i) col[i] = hbuf[i] + hbuf[(maxl + 2) + i];
      snormw = std::sqrt(std::max(hbuf[2 * (maxl + 2)], 0.0));
    } else {
      // one pass: h = V^T w and w . w; the update waits for the decision below
      k_vtw<<<g.nb, RBS, 0, g.s>>>(n, ll, nullptr, V, ldv, w, part, hdev, g.ticket, 1);
      eb_count_launch(ctx);
      EB_CUDA_TRY(cudaMemcpyAsync(hbuf.data(), hdev, sizeof(double) * (ll + 1), cudaMemcpyDeviceToHost, g.s));
      EB_CUDA_TRY(cudaStreamSynchronize(g.s));
      for (int i = 0; i < ll; ++i) col[i] = hbuf[i];
      snormw = std::sqrt(pyth_norm2(hbuf.data(), ll, hbuf[ll]));
    }
    col[ll] = snormw;
    if (!std::isfinite(snormw)) {
      eb_set_last_error_msg("non-finite Arnoldi vector");
      return EB_ERR_NAN;
    }
    if (dheqr_col(hes.data(), ldh, ll, q.data()) == ll) { iflag = 2; break; }
    prod *= q[2 * (ll - 1) + 1];
    rho = std::fabs(prod * r0nrm);
    *iters = ll;
    *err = rho / bnrm;
    if (*err <= tol) { iflag = 0; break; }
    if (ll == maxl) break;
    if (snormw == 0.0) { iflag = 2; break; }
    if (cgs2) {
      k_scale<<<g.nb, RBS, 0, g.s>>>(n, 1.0 / snormw, w);
    } else {
      k_sub_scale<<<g.nb, RBS, 0, g.s>>>(n, ll, V, ldv, hdev, w, 1.0 / snormw);
    }
    eb_count_launch(ctx);
  }
  if (iflag != 0 && iflag != 2) iflag = (rho < r0nrm) ? 1 : 2;
  if (iflag != 2) {
    for (int i = 0; i <= lgmr; ++i) y[i] = 0.0;
    y[0] = r0nrm;
    dhels(hes.data(), ldh, lgmr, q.data(), y.data());
    EB_CUDA_TRY(cudaMemcpyAsync(hdev, y.data(), sizeof(double) * lgmr, cudaMemcpyHostToDevice, g.s));
    k_gemv_add<<<g.nb, RBS, 0, g.s>>>(n, lgmr, V, ldv, hdev, x);
    eb_count_launch(ctx);
  }
  *ierr = iflag;
  return eb_check_launch(ctx, "gmres");
}


// =================================================================================
// Graph mode. One GMRES cycle (plain mode) or one refinement step (refined mode) is a
// single CUDA graph launch: the Arnoldi steps run inside a conditional WHILE node whose
// condition the device-side Arnoldi kernel sets after its DHEQR update, and DHELS and
// the solution update run on the device too. The host waits once per launch instead
// of once per Krylov step. Operator launches depend only on the installed geometry,
// so a captured graph is reused until the geometry or a work buffer changes.
// =================================================================================

struct GmCtl {
  int ll;         // Krylov column the next Arnoldi step produces (DPIGMR's LL)
  int maxl;
  int iters;
  int iflag;      // DGMRES IERR convention
  int lgmr;       // columns of the least-squares problem (= Arnoldi steps taken)
  int cont;       // the WHILE node iterates while this is 1
  int status;     // EB_OK or EB_ERR_NAN
  int store_col;  // column k_gm_store writes
  int nadd;       // columns k_gm_add adds to x
  int zero_x;     // b = 0: the solution is x = 0
  int pad[2];
  double tol, bnrm, r0nrm, prod, rho, err, scale, rnrm2;  // rnrm2: refinement ||r||^2
  double q[2 * EB_GM_MAXL];
  double hes[(EB_GM_MAXL + 1) * EB_GM_MAXL];
};
constexpr size_t GM_HEAD = offsetof(GmCtl, q);

// slots of the reduction output buffer (gH)
// (GM_TOL: the inner tolerance of the next refinement step, written by the host)
constexpr int GM_H1 = 0, GM_H2 = EB_GM_MAXL + 2, GM_NW = 2 * (EB_GM_MAXL + 2), GM_BN = GM_NW + 1,
              GM_R0 = GM_NW + 2, GM_Y = GM_NW + 4, GM_TOL = GM_Y + EB_GM_MAXL + 2, GM_HSIZE = GM_TOL + 1;

// tol_dev (if not null) holds the tolerance instead of `tol`
__global__ void k_gm_init(GmCtl* c, const double* __restrict__ hdev, cudaGraphConditionalHandle h,
                          double tol, const double* __restrict__ tol_dev, int maxl, int r0_is_b) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (tol_dev) tol = *tol_dev;
  c->tol = tol;
  c->maxl = maxl;
  c->iters = 0;
  c->iflag = 0;
  c->lgmr = 0;
  c->cont = 0;
  c->status = EB_OK;
  c->store_col = 0;
  c->nadd = 0;
  c->zero_x = 0;
  c->ll = 1;
  c->err = 0.0;
  const double bnrm = sqrt(hdev[GM_BN]);
  c->bnrm = bnrm;
  if (!isfinite(bnrm)) {
    c->status = EB_ERR_NAN;
  } else if (!(bnrm > 0.0)) {
    c->zero_x = 1;  // b = 0 (DGMRES would divide by zero)
  } else {
    const double r0 = r0_is_b ? bnrm : sqrt(hdev[GM_R0]);
    c->r0nrm = r0;
    c->err = r0 / bnrm;
    if (!isfinite(r0)) {
      c->status = EB_ERR_NAN;
    } else if (c->err > tol) {
      c->scale = 1.0 / r0;
      c->prod = 1.0;
      c->rho = r0;
      c->iflag = 1;
      c->cont = 1;
    }
  }
  cudaGraphSetConditional(h, c->cont ? 1u : 0u);
}

// V[:, store_col] = xin = scale * src while the iteration continues (src may alias V).
__global__ void k_gm_store(int n, const GmCtl* __restrict__ c, const double* src, double* V, size_t ldv,
                           double* __restrict__ xin) {
  if (!c->cont) return;
  const double sc = c->scale;
  double* dst = V + (size_t)c->store_col * ldv;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = src[i] * sc;
    dst[i] = v;
    xin[i] = v;
  }
}

// End of an Arnoldi step (DPIGMR, dpigmr.f:333-380): the Hessenberg column from the two
// Gram-Schmidt passes, its Givens update (DHEQR), the residual estimate and the decision.
__device__ void gm_arnoldi_warp(GmCtl* c, const double* __restrict__ hdev, cudaGraphConditionalHandle h) {
  const int lane = threadIdx.x;
  const int ll = c->ll, ldh = c->maxl + 1;
  double* col = c->hes + (size_t)(ll - 1) * ldh;
  for (int i = lane; i < ll; i += 32) col[i] = hdev[GM_H1 + i] + hdev[GM_H2 + i];
  __syncwarp();
  if (lane != 0) return;
  const double snormw = sqrt(fmax(hdev[GM_NW], 0.0));
  col[ll] = snormw;
  int cont = 0;
  c->lgmr = ll;
  if (!isfinite(snormw)) {
    c->status = EB_ERR_NAN;
  } else if (dheqr_col(c->hes, ldh, ll, c->q) == ll) {
    c->iflag = 2;
  } else {
    c->prod *= c->q[2 * (ll - 1) + 1];
    c->rho = fabs(c->prod * c->r0nrm);
    c->iters = ll;
    c->err = c->rho / c->bnrm;
    if (c->err <= c->tol) {
      c->iflag = 0;
    } else if (ll >= c->maxl) {
      // MAXL reached; IERR is resolved by k_gm_finish
    } else if (snormw == 0.0) {
      c->iflag = 2;
    } else {
      c->scale = 1.0 / snormw;
      c->store_col = ll;
      c->ll = ll + 1;
      cont = 1;
    }
  }
  c->cont = cont;
  cudaGraphSetConditional(h, cont ? 1u : 0u);
}

// The last Gram-Schmidt update (w -= V h with ||w||^2 into hdev[GM_NW]); the block that
// finishes the norm then ends the Arnoldi step with its first warp.
__global__ void k_gm_sub_arnoldi(int n, const int* __restrict__ ncol_dev, const double* __restrict__ V,
                                 size_t ldv, const double* __restrict__ hcol, double* __restrict__ w,
                                 double* __restrict__ part, double* hdev,
                                 unsigned int* __restrict__ ticket, GmCtl* c,
                                 cudaGraphConditionalHandle h) {
  if (!gemv_sub(n, 0, ncol_dev, V, ldv, hcol, w, part, hdev + GM_NW, ticket)) return;
  __syncthreads();
  if (threadIdx.x < 32) gm_arnoldi_warp(c, hdev, h);
}

// One-pass Arnoldi step of the refined inner cycle: h = V^T w and w . w in one
// reduction; the last block forms the norm of w - V h by Pythagoras (pyth_norm2) and
// ends the step with its first warp. k_gm_sub_store then forms the new column.
__global__ void k_gm_vtw_arnoldi(int n, const int* __restrict__ ncol_dev, const double* __restrict__ V,
                                 size_t ldv, const double* __restrict__ w, double* __restrict__ part,
                                 double* hdev, unsigned int* __restrict__ ticket, GmCtl* c,
                                 cudaGraphConditionalHandle h) {
  const int ncol = *ncol_dev;
  vtw_partials(n, ncol, 1, V, ldv, w, part);
  if (!finish_columns(gridDim.x, ncol + 1, part, hdev + GM_H1, ticket)) return;
  __syncthreads();
  if (threadIdx.x == 0) hdev[GM_NW] = pyth_norm2(hdev + GM_H1, ncol, hdev[GM_H1 + ncol]);
  __syncthreads();
  if (threadIdx.x < 32) gm_arnoldi_warp(c, hdev, h);
}

// V[:, store_col] = xin = (w - V[:, 0:store_col] h) * scale while the iteration continues
__global__ void k_gm_sub_store(int n, const GmCtl* __restrict__ c, double* V, size_t ldv,
                               const double* __restrict__ h, const double* __restrict__ w,
                               double* __restrict__ xin) {
  if (!c->cont) return;
  const int col = c->store_col;  // columns 0..col-1 are read, column col written
  sub_scale_store(n, col, V, ldv, h, w, c->scale, V + (size_t)col * ldv, xin);
}

// DHELS (dhels.f:77-96) on the device: y = R^-1 Q^T (r0nrm e1), into ydev.
__global__ void k_gm_finish(GmCtl* c, double* __restrict__ ydev) {
  __shared__ double y[EB_GM_MAXL + 1];
  __shared__ int s_n;
  const int tid = threadIdx.x;
  if (tid == 0) {
    int n = 0;
    if (c->status == EB_OK && !c->zero_x && c->lgmr > 0) {
      if (c->iflag != 0 && c->iflag != 2) c->iflag = (c->rho < c->r0nrm) ? 1 : 2;
      if (c->iflag != 2) n = c->lgmr;
    }
    c->nadd = n;
    s_n = n;
    if (n > 0) {
      for (int i = 0; i <= n; ++i) y[i] = 0.0;
      y[0] = c->r0nrm;
      for (int k = 0; k < n; ++k) {
        double cc = c->q[2 * k], ss = c->q[2 * k + 1], t1 = y[k], t2 = y[k + 1];
        y[k] = cc * t1 - ss * t2;
        y[k + 1] = ss * t1 + cc * t2;
      }
    }
  }
  __syncthreads();
  const int n = s_n;
  if (n == 0) return;
  const int ldh = c->maxl + 1;
  for (int kb = 0; kb < n; ++kb) {
    const int k = n - 1 - kb;
    if (tid == 0) y[k] /= c->hes[(size_t)k * ldh + k];
    __syncthreads();
    const double t = -y[k];
    for (int r = tid; r < k; r += blockDim.x) y[r] += t * c->hes[(size_t)k * ldh + r];
    __syncthreads();
  }
  for (int i = tid; i < n; i += blockDim.x) ydev[i] = y[i];
}

// x += V[:, 0:nadd] y, or x = 0 when b = 0.
__global__ void k_gm_add(int n, const GmCtl* __restrict__ c, const double* __restrict__ V, size_t ldv,
                         const double* __restrict__ y, double* __restrict__ x) {
  __shared__ double ys[EB_GM_MAXL + 1];
  const int stride = gridDim.x * blockDim.x;
  if (c->zero_x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] = 0.0;
    return;
  }
  const int ncol = c->nadd;
  if (ncol == 0) return;
  for (int j = threadIdx.x; j < ncol; j += blockDim.x) ys[j] = y[j];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double acc = 0.0;
    for (int j = 0; j < ncol; ++j) acc = fma(V[(size_t)j * ldv + i], ys[j], acc);
    x[i] += acc;
  }
}

// refinement: x += d unless the inner solve failed
__global__ void k_gm_axpy(int n, const GmCtl* __restrict__ c, const double* __restrict__ d,
                          double* __restrict__ x) {
  if (c->status != EB_OK) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += d[i];
}

// The inner tolerance of refinement step 2 from step 1's control block, formed as
// inner_tolerance() forms it on the host (the same operations, so the same value). A
// step 1 that ended the solve (converged, b = 0, a non-finite value) makes step 2 a
// no-op: tolerance 1e300, so no inner iteration and x += 0.
__global__ void k_gm_next_tol(const GmCtl* __restrict__ c, double* __restrict__ tol_out, double inner_tol,
                              double gmres_tol) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t = 1e300;
  if (c->status == EB_OK && !c->zero_x) {
    const double err = sqrt(fmax(c->rnrm2, 0.0)) / c->bnrm;
    if (err > gmres_tol) t = fmin(inner_tol, fmax(0.1 * inner_tol, 0.5 * gmres_tol / err));
  }
  *tol_out = t;
}

enum { GM_PLAIN = 0, GM_REFINE = 1 };
constexpr int GM_BUILD_FAILED = -100;  // internal: fall back to the host-driven loop

// Builds the graph of one plain GMRES cycle (x0 = x, tolerance gmres_tol) or of one
// refinement step (inner FP32 cycle on r from x0 = 0 to inner_tol, x += d, r = b - A x).
int build_graph(eb_ctx* ctx, GmGraph& G, int kind, op_fn op, int n, int maxl) {
  G.destroy();
  EB_CUDA_TRY(cudaGraphCreate(&G.graph, 0));
  cudaGraphConditionalHandle h;
  EB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, G.graph, 0, cudaGraphCondAssignDefault));
  const int nb = std::min(nblk(n, RBS), rmaxb(ctx));
  const size_t ldv = (size_t)n;
  double* V = ctx->gV.as<double>();
  double* part = ctx->gPart.as<double>();
  double* hdev = ctx->gH.as<double>();
  GmCtl* ctl = ctx->gCtl.as<GmCtl>();
  double* xin = ctx->gXin.as<double>();
  double* wbuf = ctx->gWbuf.as<double>();
  unsigned int* ticket = ctx->gTicket.as<unsigned int>();
  const bool refine = kind == GM_REFINE;
  const int prec = refine ? EB_FP32 : EB_FP64;
  const double tol = refine ? ctx->opts.inner_tol : ctx->opts.gmres_tol;
  double* bb = refine ? ctx->gZ.as<double>() : ctx->gR.as<double>();  // right-hand side of the cycle
  double* xx = refine ? ctx->gD.as<double>() : ctx->gX.as<double>();  // its solution
  std::vector<cudaGraphNode_t> sinks;
  // pre: norms, r0, V[:, 0]
  bool lost = false;
  auto fail = [&](int st) {
    if (lost) G.graph = nullptr;  // not destroyed by G.destroy()
    return st;
  };
  int cst = eb_capture_into(ctx, G.graph, nullptr, 0, &sinks, &G.n_pre, &lost, [&]() -> int {
    cudaStream_t s = ctx->stream;
    k_vtw<<<nb, RBS, 0, s>>>(n, 1, nullptr, bb, ldv, bb, part, hdev + GM_BN, ticket);
    eb_count_launch(ctx);
    if (refine) {
      EB_CUDA_TRY(cudaMemsetAsync(xx, 0, sizeof(double) * n, s));
      EB_CUDA_TRY(cudaMemcpyAsync(V, bb, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    } else {
      EB_CUDA_TRY(cudaMemcpyAsync(xin, xx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      EB_TRY(op(ctx, xin, wbuf, prec));
      k_resid<<<nb, RBS, 0, s>>>(n, bb, wbuf, V, part, hdev + GM_R0, ticket);
      eb_count_launch(ctx);
    }
    if (refine) EB_CUDA_TRY(cudaMemsetAsync(hdev + GM_H2, 0, sizeof(double) * (EB_GM_MAXL + 2), s));
    k_gm_init<<<1, 32, 0, s>>>(ctl, hdev, h, tol, refine ? hdev + GM_TOL : nullptr, maxl, refine ? 1 : 0);
    k_gm_store<<<nb, RBS, 0, s>>>(n, ctl, V, V, ldv, xin);
    ctx->launches += 2;
    return eb_check_launch(ctx, "gmres graph (pre)");
  });
  if (cst != EB_OK) return fail(cst);
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t ncond;
  EB_CUDA_TRY(cudaGraphAddNode(&ncond, G.graph, sinks.data(), nullptr, sinks.size(), &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  // body: one Arnoldi step
  const int* lld = &ctl->ll;
  bool body_lost = false;
  cst = eb_capture_into(ctx, body, nullptr, 0, nullptr, &G.n_body, &body_lost, [&]() -> int {
    cudaStream_t s = ctx->stream;
    EB_TRY(op(ctx, xin, wbuf, prec));
    if (refine) {
      // one Gram-Schmidt pass for the inner FP32 cycle (the H2 slots stay zero), its
      // norm by Pythagoras from the same reduction, the update fused with the store
      k_gm_vtw_arnoldi<<<nb, RBS, 0, s>>>(n, lld, V, ldv, wbuf, part, hdev, ticket, ctl, h);
      k_gm_sub_store<<<nb, RBS, 0, s>>>(n, ctl, V, ldv, hdev + GM_H1, wbuf, xin);
    } else {
      k_vtw<<<nb, RBS, 0, s>>>(n, 0, lld, V, ldv, wbuf, part, hdev + GM_H1, ticket);
      k_update_vtw<<<nb, RBS, 0, s>>>(n, 0, lld, V, ldv, hdev + GM_H1, wbuf, part, hdev + GM_H2, ticket);
      k_gm_sub_arnoldi<<<nb, RBS, 0, s>>>(n, lld, V, ldv, hdev + GM_H2, wbuf, part, hdev, ticket, ctl, h);
      k_gm_store<<<nb, RBS, 0, s>>>(n, ctl, wbuf, V, ldv, xin);
    }
    ctx->launches += refine ? 2 : 4;
    return eb_check_launch(ctx, "gmres graph (body)");
  });
  if (body_lost) lost = true;  // the body belongs to the graph; leave the whole graph alone
  if (cst != EB_OK) return fail(cst);
  // post: DHELS, x update; refined: x += d, r = b - A64 x with ||r||^2
  cst = eb_capture_into(ctx, G.graph, &ncond, 1, nullptr, &G.n_post, &lost, [&]() -> int {
    cudaStream_t s = ctx->stream;
    k_gm_finish<<<1, 128, 0, s>>>(ctl, hdev + GM_Y);
    k_gm_add<<<nb, RBS, 0, s>>>(n, ctl, V, ldv, hdev + GM_Y, xx);
    ctx->launches += 2;
    if (refine) {
      double* x = ctx->gX.as<double>();
      k_gm_axpy<<<nb, RBS, 0, s>>>(n, ctl, xx, x);
      eb_count_launch(ctx);
      EB_TRY(op(ctx, x, bb, eb_resid_prec(ctx)));
      k_resid<<<nb, RBS, 0, s>>>(n, ctx->gR.as<double>(), bb, bb, part, &ctl->rnrm2, ticket);
      eb_count_launch(ctx);
    }
    return eb_check_launch(ctx, "gmres graph (post)");
  });
  if (cst != EB_OK) return fail(cst);
  EB_CUDA_TRY(cudaGraphInstantiate(&G.exec, G.graph, cudaGraphInstantiateFlagUseNodePriority));
  G.valid = true;
  return EB_OK;
}

GmGraph* find_graph(eb_ctx* ctx, const unsigned long long* key) {
  for (GmGraph& g : ctx->gcache)
    if (g.valid && std::equal(key, key + 8, g.key)) return &g;
  return nullptr;
}

// Runs one graph launch (building it on first use) and reads the control block back:
// into head after a synchronisation; with wait = false into head (page-locked) without
// one, the caller synchronising and adding the launches (*base + *per_step * lgmr).
int run_graph(eb_ctx* ctx, int kind, op_fn op, int n, int maxl, GmCtl* head, bool wait = true,
              long long* base = nullptr, long long* per_step = nullptr) {
  unsigned long long key[8];
  auto fill_key = [&](unsigned long long epoch) {
    double t1 = ctx->opts.gmres_tol, t2 = ctx->opts.inner_tol;
    key[0] = (unsigned long long)kind;
    key[1] = (unsigned long long)(uintptr_t)op;
    key[2] = (unsigned long long)n;
    key[3] = (unsigned long long)maxl;
    key[4] = ctx->geom_shape;
    key[5] = epoch;
    memcpy(&key[6], &t1, 8);
    memcpy(&key[7], &t2, 8);
  };
  fill_key(eb_devbuf_epoch());
  GmGraph* G = find_graph(ctx, key);
  if (!G) {
    G = &ctx->gcache[ctx->gcache_next];
    ctx->gcache_next = (ctx->gcache_next + 1) % EB_GRAPH_CACHE;
    // A buffer that grows during the capture moves: nodes captured before the growth
    // hold its old address, which eb_devbuf_collect later frees. Such a graph is never
    // kept; it is captured again once every buffer has its final size (a buffer's
    // first allocation does not move it, so a second capture sees no growth).
    int st = EB_OK;
    for (int attempt = 0; attempt < 3; ++attempt) {
      const unsigned long long e0 = eb_devbuf_epoch();
      st = build_graph(ctx, *G, kind, op, n, maxl);
      if (st != EB_OK || eb_devbuf_epoch() == e0) break;
      G->destroy();
      st = GM_BUILD_FAILED;
    }
    if (st != EB_OK) {
      G->destroy();
      cudaGetLastError();
      return GM_BUILD_FAILED;
    }
    fill_key(eb_devbuf_epoch());
    memcpy(G->key, key, sizeof(key));
  }
  cudaStream_t s = ctx->stream;
  EB_CUDA_TRY(cudaGraphLaunch(G->exec, s));
  if (!head) {  // deferred: the control block goes to the next page-locked slot
    const int slot = ctx->ndefer++;
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->h_defer + (size_t)slot * GM_HEAD, ctx->gCtl.p, GM_HEAD,
                                cudaMemcpyDeviceToHost, s));
    ctx->launches += G->n_pre + G->n_post;
    ctx->defer_body[slot] = G->n_body;
    return EB_OK;
  }
  EB_CUDA_TRY(cudaMemcpyAsync(head, ctx->gCtl.p, GM_HEAD, cudaMemcpyDeviceToHost, s));
  if (!wait) {
    *base = G->n_pre + G->n_post;
    *per_step = G->n_body;
    return EB_OK;
  }
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  ctx->launches += G->n_pre + G->n_post + G->n_body * (long long)head->lgmr;
  return EB_OK;
}

// Inner tolerance of refinement step `outer` given the outer relative residual `err`
// before it: the configured inner tolerance for the first step; later steps solve far
// enough (by half a margin) that the step is expected to end the solve, since the
// residual contracts by about the inner tolerance per step, but never below a tenth of
// the configured value (the FP32 operator's own error sets the floor).
double inner_tolerance(const eb_ctx* ctx, int outer, double err) {
  const double t = ctx->opts.inner_tol;
  if (outer <= 1 || !(err > 0.0)) return t;
  return std::min(t, std::max(0.1 * t, 0.5 * ctx->opts.gmres_tol / err));
}

int solve_graph(eb_ctx* ctx, int n, op_fn op, int mode, int maxl, eb_solve_info* inf) {
  cudaStream_t s = ctx->stream;
  if (maxl > n) maxl = n;
  EB_TRY(ctx->gCtl.ensure(sizeof(GmCtl)));
  EB_TRY(ctx->gXin.ensure(sizeof(double) * n));
  EB_TRY(ctx->gWbuf.ensure(sizeof(double) * n));
  EB_TRY(ctx->gV.ensure(sizeof(double) * (size_t)n * (maxl + 1)));
  EB_TRY(ctx->gD.ensure(sizeof(double) * n));
  EB_TRY(ctx->gZ.ensure(sizeof(double) * n));
  GmCtl head;
  if (mode == EB_SOLVE_FP64 && ctx->defer && ctx->ndefer < EB_DEFER_SLOTS) {
    // inside an RK call: no wait here; eb_defer_info reads the control block later
    if (!ctx->h_defer)
      EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&ctx->h_defer), GM_HEAD * (size_t)EB_DEFER_SLOTS));
    EB_TRY(run_graph(ctx, GM_PLAIN, op, n, maxl, nullptr));
    inf->outer = 1;
    return EB_OK;
  }
  if (mode == EB_SOLVE_FP64) {
    EB_TRY(run_graph(ctx, GM_PLAIN, op, n, maxl, &head));
    if (head.status != EB_OK) {
      eb_set_last_error_msg("non-finite value in GMRES");
      return head.status;
    }
    inf->iters = head.iters;
    inf->err = head.err;
    inf->ierr = head.lgmr > 0 ? head.iflag : 0;
    inf->outer = 1;
    inf->matvecs64 = 1 + head.lgmr;
    return EB_OK;
  }
  double* x = ctx->gX.as<double>();
  EB_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->gZ.p, ctx->gR.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  inf->ierr = 1;
  double bnrm = 0.0;
  double err_prev = 1.0;
  // the host's part of refinement step `outer` once its control block is read: returns
  // EB_OK with *done set when the solve ended, or an error
  auto step_done = [&](int outer, const GmCtl& h, bool* done) -> int {
    *done = false;
    inf->outer = outer;
    if (h.status != EB_OK) {
      eb_set_last_error_msg("non-finite value in GMRES");
      return h.status;
    }
    inf->iters += h.iters;
    inf->matvecs32 += h.lgmr;
    inf->matvecs64 += 1;
    if (outer == 1) {
      bnrm = h.bnrm;  // the first inner right-hand side is b itself
      if (h.zero_x) {
        inf->err = 0.0;
        inf->ierr = 0;
        *done = true;
        return EB_OK;
      }
    }
    inf->err = std::sqrt(std::max(h.rnrm2, 0.0)) / bnrm;
    err_prev = inf->err;
    if (!std::isfinite(inf->err)) {
      eb_set_last_error_msg("non-finite residual");
      return EB_ERR_NAN;
    }
    if (inf->err <= ctx->opts.gmres_tol) {
      inf->ierr = 0;
      *done = true;
    }
    return EB_OK;
  };
  int first = 1;
  if (ctx->opts.max_outer >= 2) {
    // steps 1 and 2 back to back with one wait: step 2's inner tolerance is formed on the
    // device from step 1's residual (k_gm_next_tol), and a step 1 that ended the solve
    // leaves step 2 nothing to do
    if (!ctx->h_spec) EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&ctx->h_spec), 2 * GM_HEAD));
    GmCtl* h1 = reinterpret_cast<GmCtl*>(ctx->h_spec);
    GmCtl* h2 = reinterpret_cast<GmCtl*>(ctx->h_spec + GM_HEAD);
    const double itol = inner_tolerance(ctx, 1, err_prev);
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->gH.as<double>() + GM_TOL, &itol, sizeof(double), cudaMemcpyHostToDevice, s));
    long long b1 = 0, p1 = 0, b2 = 0, p2 = 0;
    EB_TRY(run_graph(ctx, GM_REFINE, op, n, maxl, h1, false, &b1, &p1));
    k_gm_next_tol<<<1, 32, 0, s>>>(ctx->gCtl.as<GmCtl>(), ctx->gH.as<double>() + GM_TOL, ctx->opts.inner_tol,
                                   ctx->opts.gmres_tol);
    eb_count_launch(ctx);
    EB_TRY(run_graph(ctx, GM_REFINE, op, n, maxl, h2, false, &b2, &p2));
    EB_CUDA_TRY(cudaStreamSynchronize(s));
    GmCtl hd1, hd2;
    memcpy(&hd1, h1, GM_HEAD);
    memcpy(&hd2, h2, GM_HEAD);
    ctx->launches += b1 + p1 * (long long)hd1.lgmr + b2 + p2 * (long long)hd2.lgmr;
    bool done = false;
    EB_TRY(step_done(1, hd1, &done));
    if (done) return EB_OK;
    EB_TRY(step_done(2, hd2, &done));
    if (done) return EB_OK;
    first = 3;
  }
  for (int outer = first; outer <= ctx->opts.max_outer; ++outer) {
    const double itol = inner_tolerance(ctx, outer, err_prev);
    EB_CUDA_TRY(cudaMemcpyAsync(ctx->gH.as<double>() + GM_TOL, &itol, sizeof(double), cudaMemcpyHostToDevice, s));
    EB_TRY(run_graph(ctx, GM_REFINE, op, n, maxl, &head));
    bool done = false;
    EB_TRY(step_done(outer, head, &done));
    if (done) break;
  }
  return EB_OK;
}

int solve(eb_ctx* ctx, int n, op_fn op, const double* rhs, double* soln, int mode,
          eb_solve_info* info, int mem) {
  if (ctx->nsim > 0)  // a batch of simulations: GMRES per simulation, in lockstep
    return eb_batch_solve(ctx, n, op, op == eb_stokes_matvec_dev || op == eb_stokes_matvec_adj_dev, rhs, soln,
                          mode, info, mem);
  cudaStream_t s = ctx->stream;
  Gm g{ctx, n, std::min(nblk(n, RBS), rmaxb(ctx)), s, nullptr};
  const int maxl = ctx->opts.maxl;
  if (maxl > 126) {
    eb_set_last_error_msg("maxl above 126 is not supported");
    return EB_ERR_WORKSPACE;
  }
  EB_TRY(ctx->gPart.ensure(sizeof(double) * (size_t)rmaxb(ctx) * (maxl + 2)));
  EB_TRY(ctx->gH.ensure(sizeof(double) * std::max(3 * (maxl + 2), (int)GM_HSIZE)));
  EB_TRY(ctx->gTicket.ensure(sizeof(unsigned int)));
  EB_CUDA_TRY(cudaMemsetAsync(ctx->gTicket.p, 0, sizeof(unsigned int), s));
  g.ticket = ctx->gTicket.as<unsigned int>();
  EB_TRY(ctx->gR.ensure(sizeof(double) * n));
  EB_TRY(ctx->gX.ensure(sizeof(double) * n));
  double* b = ctx->gR.as<double>();
  double* x = ctx->gX.as<double>();
  const bool defl = op == eb_laplace_matvec_dev && ctx->opts.lap_deflate > 0;
  if (defl) {
    EB_TRY(ctx->gDefl.ensure(sizeof(double) * n));
    EB_TRY(ctx->gDeflC.ensure(sizeof(double2) * (size_t)ctx->k));
    k_deflate_coef<<<ctx->k, DEFL_BS, 0, s>>>(ctx->start.as<int>(), ctx->dsda.as<double>(),
                                              ctx->gDeflC.as<double2>());
    eb_count_launch(ctx);
    op = laplace_matvec_deflated;
  }
  // SOLVEI / SOLVE_LAPL: soln = rhs as the initial guess (stokesbubb.f:346-349); the
  // deflated solve starts from t0 = M rhs, which is x0 = rhs.
  cudaMemcpyKind kin = mem == EB_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  auto init_x = [&]() -> int {
    EB_CUDA_TRY(cudaMemcpyAsync(x, rhs, sizeof(double) * n, kin, s));
    if (defl) EB_TRY(deflate(ctx, x, x, 0));
    return EB_OK;
  };
  EB_CUDA_TRY(cudaMemcpyAsync(b, rhs, sizeof(double) * n, kin, s));
  EB_TRY(init_x());
  eb_solve_info inf{};
  int st = EB_OK;
  bool eager = true;
  if (ctx->opts.graphs > 0 && !ctx->profiling) {
    st = solve_graph(ctx, n, op, mode, maxl, &inf);
    if (st == GM_BUILD_FAILED) {
      // graphs with conditional nodes are unavailable: use the host-driven loop from now on
      ctx->opts.graphs = -1;
      inf = eb_solve_info{};
      st = EB_OK;
      EB_TRY(init_x());
    } else {
      inf.graph = 1;
      eager = false;
    }
  }
  if (eager && mode == EB_SOLVE_FP64) {
    int nmv = 0;
    st = gmres_cycle(g, op, EB_FP64, b, x, false, ctx->opts.gmres_tol, maxl, &inf.iters, &inf.err,
                     &inf.ierr, &nmv, -1.0);
    inf.outer = 1;
    inf.matvecs64 = nmv;
  } else if (eager) {
    EB_TRY(ctx->gD.ensure(sizeof(double) * n));
    EB_TRY(ctx->gZ.ensure(sizeof(double) * n));
    double* r = ctx->gZ.as<double>();
    double* d = ctx->gD.as<double>();
    // Refinement starts from x = 0, so the first residual is b itself and costs no
    // FP64 apply; every step is one inner FP32 solve plus one FP64 residual.
    double bss;
    EB_TRY(dev_sumsq(g, b, &bss));
    double bnrm = std::sqrt(bss), rnrm = bnrm;
    EB_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
    EB_CUDA_TRY(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    inf.ierr = 1;
    inf.err = bnrm > 0 ? 1.0 : 0.0;
    if (!(bnrm > 0)) inf.ierr = 0;
    for (int outer = 1; outer <= ctx->opts.max_outer && inf.ierr != 0; ++outer) {
      inf.outer = outer;
      int it = 0, ie = 0, nmv = 0;
      double e2 = 0;
      st = gmres_cycle(g, op, EB_FP32, r, d, true, inner_tolerance(ctx, outer, inf.err), maxl, &it, &e2,
                       &ie, &nmv, rnrm);
      inf.iters += it;
      inf.matvecs32 += nmv;
      if (st != EB_OK) break;
      k_axpy<<<g.nb, RBS, 0, s>>>(n, 1.0, d, x);
      eb_count_launch(ctx);
      EB_TRY(op(ctx, x, r, eb_resid_prec(ctx)));
      inf.matvecs64++;
      double* part = ctx->gPart.as<double>();
      k_resid<<<g.nb, RBS, 0, s>>>(n, b, r, r, part, ctx->gH.as<double>(), g.ticket);
      ctx->launches += 1;
      double rss;
      EB_CUDA_TRY(cudaMemcpyAsync(&rss, ctx->gH.p, sizeof(double), cudaMemcpyDeviceToHost, s));
      EB_CUDA_TRY(cudaStreamSynchronize(s));
      rnrm = std::sqrt(rss);
      inf.err = rnrm / bnrm;
      if (!std::isfinite(inf.err)) {
        eb_set_last_error_msg("non-finite residual");
        st = EB_ERR_NAN;
        break;
      }
      if (inf.err <= ctx->opts.gmres_tol) inf.ierr = 0;
    }
  }
  if (st == EB_OK) {
    if (defl) EB_TRY(deflate(ctx, x, x, 1));  // x = M^-1 t
    cudaMemcpyKind kout = mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    EB_CUDA_TRY(cudaMemcpyAsync(soln, x, sizeof(double) * n, kout, s));
    // the info is already on the host; a device solution is ready in stream order
    if (mem == EB_HOST) EB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (info) *info = inf;
  return st;
}

}  // namespace

int eb_defer_info(eb_ctx* ctx, int slot, eb_solve_info* inf) {
  if (slot < 0 || slot >= ctx->ndefer) return EB_ERR_ARG;
  GmCtl head;
  memcpy(&head, ctx->h_defer + (size_t)slot * GM_HEAD, GM_HEAD);
  ctx->launches += ctx->defer_body[slot] * (long long)head.lgmr;
  if (head.status != EB_OK) {
    eb_set_last_error_msg("non-finite value in GMRES");
    return head.status;
  }
  inf->iters = head.iters;
  inf->err = head.err;
  inf->ierr = head.lgmr > 0 ? head.iflag : 0;
  inf->outer = 1;
  inf->matvecs64 = 1 + head.lgmr;
  inf->graph = 1;
  return EB_OK;
}

void GmGraph::destroy() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
  valid = false;
}

int eb_stokes_solve(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                    eb_solve_info* info, int mem) {
  if (!ctx || !rhs || !soln) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != 2 * ctx->nbk || (mode != EB_SOLVE_FP64 && mode != EB_SOLVE_FP32_REFINED)) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return solve(ctx, n, eb_stokes_matvec_dev, rhs, soln, mode, info, mem);
}

int eb_laplace_solve(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                     eb_solve_info* info, int mem) {
  if (!ctx || !rhs || !soln) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != ctx->nbk || (mode != EB_SOLVE_FP64 && mode != EB_SOLVE_FP32_REFINED)) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return solve(ctx, n, eb_laplace_matvec_dev, rhs, soln, mode, info, mem);
}

// The same GMRES on the transposed operators (the adjoint solves).
int eb_stokes_solve_adjoint(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                            eb_solve_info* info, int mem) {
  if (!ctx || !rhs || !soln) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != 2 * ctx->nbk || (mode != EB_SOLVE_FP64 && mode != EB_SOLVE_FP32_REFINED)) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  if (ctx->iwall) {
    eb_set_last_error_msg("the transposed operators do not include the wall's images");
    return EB_ERR_ARG;
  }
  cudaSetDevice(ctx->device);
  return solve(ctx, n, eb_stokes_matvec_adj_dev, rhs, soln, mode, info, mem);
}

int eb_laplace_solve_adjoint(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                             eb_solve_info* info, int mem) {
  if (!ctx || !rhs || !soln) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != ctx->nbk || (mode != EB_SOLVE_FP64 && mode != EB_SOLVE_FP32_REFINED)) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  if (ctx->iwall) {
    eb_set_last_error_msg("the transposed operators do not include the wall's images");
    return EB_ERR_ARG;
  }
  cudaSetDevice(ctx->device);
  return solve(ctx, n, eb_laplace_matvec_adj_dev, rhs, soln, mode, info, mem);
}

// ---------------------------------------------------------------------------------
// FP64 FMA throughput calibration: the roofline denominator of the FP64 kernels
// (the FMM apply is bound by the FP64 pipe, not by HBM or the tensor cores).
// ---------------------------------------------------------------------------------
namespace {
__global__ void k_ffma_chain(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_dfma_chain(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

int eb_measure_fp64_peak(eb_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int sms = 0;
  EB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int blocks = sms * 8, threads = 256, iters = 2000;
  DevBuf out;
  EB_TRY(out.ensure(sizeof(double) * (size_t)blocks * threads));
  cudaStream_t s = ctx->stream;
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    EB_CUDA_TRY(cudaEventRecord(ctx->ev0, s));
    k_dfma_chain<<<blocks, threads, 0, s>>>(out.as<double>(), iters, 0.999, 1e-3);
    EB_CUDA_TRY(cudaEventRecord(ctx->ev1, s));
    EB_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    EB_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (ms < best) best = ms;
  }
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return eb_check_launch(ctx, "fp64 peak");
}

// FP32 FMA throughput: the roofline denominator of the FP32 and double-float kernels.
int eb_measure_fp32_peak(eb_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  int sms = 0;
  EB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int blocks = sms * 8, threads = 256, iters = 20000;
  DevBuf out;
  EB_TRY(out.ensure(sizeof(float) * (size_t)blocks * threads));
  cudaStream_t s = ctx->stream;
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    EB_CUDA_TRY(cudaEventRecord(ctx->ev0, s));
    k_ffma_chain<<<blocks, threads, 0, s>>>(out.as<float>(), iters, 0.9999f, 1e-4f);
    EB_CUDA_TRY(cudaEventRecord(ctx->ev1, s));
    EB_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
    float ms = 0.f;
    EB_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (ms < best) best = ms;
  }
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return eb_check_launch(ctx, "fp32 peak");
}
