// GMRES on the GPU with the semantics of SLATEC DGMRES as SOLVEI / SOLVE_LAPL call it
// (stokesbubb.f:330-350, laplace.f:361-382): x0 = rhs, MAXL Krylov vectors, no
// restart, no preconditioner, stop when the Givens estimate of ||b - A x|| / ||b||
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
// until ||r|| / ||b|| <= TOL; the reported error is the true FP64 residual.
#include <cmath>
#include <vector>

#include "eb_internal.h"

namespace {

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }
constexpr int RBS = 256;   // reduction block size
constexpr int RMAXB = 304; // 2 blocks per SM on 152 SMs

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
__device__ void finish_columns(int nb, int ncol, const double* part, double* out,
                               unsigned int* ticket) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j = w; j < ncol; j += nw) {
    double s = 0.0;
    for (int b = lane; b < nb; b += 32) s += __ldcg(part + (size_t)b * ncol + j);
    s = warp_sum<double>(s);
    if (lane == 0) out[j] = s;
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// out[j] = V[:, j] . w for j < ncol. Each block takes a contiguous range of rows and
// each of its warps a subset of the columns; partial sums per block go to `part` and
// the last block to finish adds them in block order.
__global__ void k_vtw(int n, int ncol, const double* __restrict__ V, size_t ldv,
                      const double* __restrict__ w, double* __restrict__ part,
                      double* __restrict__ out, unsigned int* __restrict__ ticket) {
  const int rows = (n + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * rows, r1 = min(n, r0 + rows);
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j = wi; j < ncol; j += nw) {
    const double* v = V + (size_t)j * ldv;
    double s = 0.0;
    for (int i = r0 + lane; i < r1; i += 32) s = fma(v[i], w[i], s);
    s = warp_sum<double>(s);
    if (lane == 0) part[(size_t)blockIdx.x * ncol + j] = s;
  }
  finish_columns(gridDim.x, ncol, part, out, ticket);
}

// w -= V[:, 0:ncol] h; if part != nullptr also ||w||^2 of the new w into *out.
__global__ void k_gemv_sub(int n, int ncol, const double* __restrict__ V, size_t ldv,
                           const double* __restrict__ h, double* __restrict__ w,
                           double* __restrict__ part, double* __restrict__ out,
                           unsigned int* __restrict__ ticket) {
  __shared__ double hs[128];
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
  if (part) {
    sq = block_sum(sq, red);
    if (threadIdx.x == 0) part[blockIdx.x] = sq;
    finish_columns(gridDim.x, 1, part, out, ticket);
  }
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

// out = a - out (residual), with ||out||^2 into *nrm2.
__global__ void k_resid(int n, const double* __restrict__ a, double* __restrict__ out,
                        double* __restrict__ part, double* __restrict__ nrm2,
                        unsigned int* __restrict__ ticket) {
  __shared__ double red[32];
  double sq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = a[i] - out[i];
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
  k_vtw<<<g.nb, RBS, 0, g.s>>>(g.n, 1, v, (size_t)g.n, v, part, ctx->gH.as<double>(), g.ticket);
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaMemcpyAsync(out, ctx->gH.p, sizeof(double), cudaMemcpyDeviceToHost, g.s));
  EB_CUDA_TRY(cudaStreamSynchronize(g.s));
  return EB_OK;
}

// DHEQR column update (IJOB > 1 form; identical to IJOB = 1 for the first column).
int dheqr_col(double* hes, int ldh, int ll, double* q) {
  double* a = hes + (size_t)(ll - 1) * ldh;
  for (int k = 0; k < ll - 1; ++k) {
    double c = q[2 * k], s = q[2 * k + 1], t1 = a[k], t2 = a[k + 1];
    a[k] = c * t1 - s * t2;
    a[k + 1] = s * t1 + c * t2;
  }
  double t1 = a[ll - 1], t2 = a[ll], c, s;
  if (t2 == 0.0) { c = 1.0; s = 0.0; }
  else if (std::fabs(t2) >= std::fabs(t1)) { double t = t1 / t2; s = -1.0 / std::sqrt(1.0 + t * t); c = -s * t; }
  else { double t = t2 / t1; c = 1.0 / std::sqrt(1.0 + t * t); s = -c * t; }
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
    k_resid<<<g.nb, RBS, 0, g.s>>>(n, b, V, part, hdev, g.ticket);
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
    // pass 1: h1 = V^T w; w -= V h1
    k_vtw<<<g.nb, RBS, 0, g.s>>>(n, ll, V, ldv, w, part, hdev, g.ticket);
    k_gemv_sub<<<g.nb, RBS, 0, g.s>>>(n, ll, V, ldv, hdev, w, nullptr, nullptr, nullptr);
    // pass 2: h2 = V^T w; w -= V h2 with ||w||^2
    k_vtw<<<g.nb, RBS, 0, g.s>>>(n, ll, V, ldv, w, part, hdev + (maxl + 2), g.ticket);
    k_gemv_sub<<<g.nb, RBS, 0, g.s>>>(n, ll, V, ldv, hdev + (maxl + 2), w, part,
                                      hdev + 2 * (maxl + 2), g.ticket);
    ctx->launches += 4;
    EB_CUDA_TRY(cudaMemcpyAsync(hbuf.data(), hdev, sizeof(double) * 3 * (maxl + 2),
                                cudaMemcpyDeviceToHost, g.s));
    EB_CUDA_TRY(cudaStreamSynchronize(g.s));
    double* col = hes.data() + (size_t)(ll - 1) * ldh;
    for (int i = 0; i < ll; ++i) col[i] = hbuf[i] + hbuf[(maxl + 2) + i];
    double snormw = std::sqrt(std::max(hbuf[2 * (maxl + 2)], 0.0));
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
    k_scale<<<g.nb, RBS, 0, g.s>>>(n, 1.0 / snormw, w);
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

int solve(eb_ctx* ctx, int n, op_fn op, const double* rhs, double* soln, int mode,
          eb_solve_info* info, int mem) {
  cudaStream_t s = ctx->stream;
  Gm g{ctx, n, std::min(nblk(n, RBS), RMAXB), s, nullptr};
  const int maxl = ctx->opts.maxl;
  if (maxl > 126) {
    eb_set_last_error_msg("maxl above 126 is not supported");
    return EB_ERR_WORKSPACE;
  }
  EB_TRY(ctx->gPart.ensure(sizeof(double) * (size_t)RMAXB * (maxl + 2)));
  EB_TRY(ctx->gH.ensure(sizeof(double) * 3 * (maxl + 2)));
  EB_TRY(ctx->gTicket.ensure(sizeof(unsigned int)));
  EB_CUDA_TRY(cudaMemsetAsync(ctx->gTicket.p, 0, sizeof(unsigned int), s));
  g.ticket = ctx->gTicket.as<unsigned int>();
  EB_TRY(ctx->gR.ensure(sizeof(double) * n));
  EB_TRY(ctx->gX.ensure(sizeof(double) * n));
  double* b = ctx->gR.as<double>();
  double* x = ctx->gX.as<double>();
  // SOLVEI / SOLVE_LAPL: soln = rhs as the initial guess (stokesbubb.f:346-349).
  cudaMemcpyKind kin = mem == EB_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  EB_CUDA_TRY(cudaMemcpyAsync(b, rhs, sizeof(double) * n, kin, s));
  EB_CUDA_TRY(cudaMemcpyAsync(x, rhs, sizeof(double) * n, kin, s));
  eb_solve_info inf{};
  int st = EB_OK;
  if (mode == EB_SOLVE_FP64) {
    int nmv = 0;
    st = gmres_cycle(g, op, EB_FP64, b, x, false, ctx->opts.gmres_tol, maxl, &inf.iters, &inf.err,
                     &inf.ierr, &nmv, -1.0);
    inf.outer = 1;
    inf.matvecs64 = nmv;
  } else {
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
      st = gmres_cycle(g, op, EB_FP32, r, d, true, ctx->opts.inner_tol, maxl, &it, &e2, &ie, &nmv,
                       rnrm);
      inf.iters += it;
      inf.matvecs32 += nmv;
      if (st != EB_OK) break;
      k_axpy<<<g.nb, RBS, 0, s>>>(n, 1.0, d, x);
      eb_count_launch(ctx);
      EB_TRY(op(ctx, x, r, EB_FP64));
      inf.matvecs64++;
      double* part = ctx->gPart.as<double>();
      k_resid<<<g.nb, RBS, 0, s>>>(n, b, r, part, ctx->gH.as<double>(), g.ticket);
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
    cudaMemcpyKind kout = mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    EB_CUDA_TRY(cudaMemcpyAsync(soln, x, sizeof(double) * n, kout, s));
    EB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (info) *info = inf;
  return st;
}

}  // namespace

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

// ---------------------------------------------------------------------------------
// FP64 FMA throughput calibration: the roofline denominator of the FP64 kernels
// (the FMM apply is bound by the FP64 pipe, not by HBM or the tensor cores).
// ---------------------------------------------------------------------------------
namespace {
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
