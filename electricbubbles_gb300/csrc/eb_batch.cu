// Many independent simulations in one context.
//
// The reference advances one simulation per process (electric.f:134-251): its GMRES
// solves (SOLVEI, stokesbubb.f:294-415; SOLVE_LAPL, laplace.f:335-425), layer sums and RK
// stages see one set of drops. Here a context can hold a batch of simulations of uneven
// sizes: their drops are concatenated, every kernel launch covers all of them, and
//  * the FMM tree is a forest: each simulation is moved into its own cell of a grid of
//    2^R x 2^R cells (a translation, under which the layer sums are invariant) and no
//    interaction list crosses a cell, so no sum mixes simulations;
//  * the GMRES of every solve runs per simulation: each simulation's segment of the
//    batch vector has its own Krylov basis, Hessenberg matrix, Givens rotations and
//    stopping test, all advanced in lockstep by one block per simulation, and a
//    simulation that has converged stops changing while the others go on;
//  * the per-simulation quantities of FASMVP and SETVELF (the far-field pressure of the
//    simulation's first drop, E0, the `alpha` of its last drop) are taken per drop.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "eb_internal.h"

namespace {

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }
constexpr int BBS = 256;   // threads per simulation block
constexpr int BCH = 1024;  // rows per work item of the inner Arnoldi steps

__device__ __forceinline__ double bblock_sum(double v, double* red) {
  v = warp_sum<double>(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
    r = warp_sum<double>(r);
    if (l == 0) red[32] = r;
  }
  __syncthreads();
  return red[32];
}

// A simulation's bounding box: (min x, max x, min y, max y).
struct SimBox {
  double x, y, z, w;
};

// Per-simulation bounding boxes (block per simulation over its node range).
__global__ void k_sim_bbox(const int* __restrict__ node0, const double2* __restrict__ z, SimBox* __restrict__ box) {
  const int s = blockIdx.x, i0 = node0[s], i1 = node0[s + 1];
  double mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double2 p = z[i];
    mnx = fmin(mnx, p.x);
    mxx = fmax(mxx, p.x);
    mny = fmin(mny, p.y);
    mxy = fmax(mxy, p.y);
  }
  // min / max through negated sums would lose exactness: use shuffles
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fmin(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mny = fmin(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxy = fmax(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  __shared__ SimBox wb[32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) wb[w] = SimBox{mnx, mxx, mny, mxy};
  __syncthreads();
  if (threadIdx.x == 0) {
    SimBox r = wb[0];
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
      r.x = fmin(r.x, wb[q].x);
      r.y = fmax(r.y, wb[q].y);
      r.z = fmin(r.z, wb[q].z);
      r.w = fmax(r.w, wb[q].w);
    }
    box[s] = r;
  }
}

// Moves every node of simulation s by shift[s] (the simulation's cell of the forest).
__global__ void k_translate(int n, const int* __restrict__ sim_of_node, const double2* __restrict__ shift,
                            const double2* __restrict__ z, double2* __restrict__ zt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 d = shift[sim_of_node[i]];
  zt[i] = make_double2(z[i].x + d.x, z[i].y + d.y);
}

// The same for the fine grid of PVINTEV: drop b's 2 nd points start at 2 start[b].
__global__ void k_translate_fine(const int* __restrict__ start, const int* __restrict__ sim_of_drop,
                                 const double2* __restrict__ shift, double2* __restrict__ zf) {
  const int b = blockIdx.x;
  const double2 d = shift[sim_of_drop[b]];
  for (int i = 2 * start[b] + threadIdx.x; i < 2 * start[b + 1]; i += blockDim.x)
    zf[i] = make_double2(zf[i].x + d.x, zf[i].y + d.y);
}

// ---------------------------------------------------------------------------------
// Batched GMRES. Per simulation s, segment [seg[s], seg[s+1]) of every batch vector.
// ---------------------------------------------------------------------------------
struct BCtl {
  double bnrm;    // ||b||
  double rho;     // Givens estimate of ||b - A x||
  double tol;     // relative tolerance of this cycle
  int active;     // the simulation still iterates
  int lgmr;       // Krylov columns in use
  int iflag;      // 0 converged, 1 MAXL reached, 2 non-finite
  int pad;
};

// Start of a cycle: r = b - w (w = A x0, or nothing when x0 = 0), beta = ||r||,
// V[:, 0] = r / beta, g = (beta, 0, ...); converged already when beta <= tol ||b||.
// ctl->tol holds the cycle's relative tolerance; a simulation whose `skip` flag is set
// (already converged in an earlier refinement step) does not take part.
__global__ void k_bg_init(const int* __restrict__ seg, const double* __restrict__ b, const double* __restrict__ w,
                          const double* __restrict__ bnorm_src, double* __restrict__ V, BCtl* __restrict__ ctl,
                          double* __restrict__ G, const int* __restrict__ skip, int maxl) {
  __shared__ double red[33];
  const int s = blockIdx.x, i0 = seg[s], i1 = seg[s + 1];
  double rr = 0.0, bb = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double r = w ? b[i] - w[i] : b[i];
    V[i] = r;
    rr = fma(r, r, rr);
    const double bv = bnorm_src ? bnorm_src[i] : b[i];
    bb = fma(bv, bv, bb);
  }
  rr = bblock_sum(rr, red);
  bb = bblock_sum(bb, red);
  const double beta = sqrt(rr), bn = sqrt(bb);
  BCtl& c = ctl[s];
  const bool off = skip && skip[s];
  const bool done = off || !(beta > c.tol * bn) || !(bn > 0.0);
  if (!done) {  // one reciprocal: an FP64 division per element is slow on this GPU
    const double rb = 1.0 / beta;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) V[i] *= rb;
  }
  if (threadIdx.x == 0) {
    c.bnrm = bn;
    c.rho = off ? 0.0 : beta;
    c.active = done ? 0 : 1;
    c.lgmr = 0;
    c.iflag = (isfinite(beta) && isfinite(bn)) ? 0 : 2;
    if (c.iflag) c.active = 0;
    double* g = G + (size_t)s * (maxl + 1);
    g[0] = beta;
  }
}

// The end of Arnoldi step j of simulation s (one thread): the Hessenberg column h (plus
// h2 when given) with ||w'|| = hn below it, DHEQR's Givens update (dheqr.f:82-176), the
// residual estimate and the stopping test (DPIGMR's RHO, dpigmr.f:340-355).
__device__ void bg_step_end(int s, int j, const double* h, const double* h2, double hn, BCtl& c,
                            double* __restrict__ Hh, double* __restrict__ G, double* __restrict__ CS, int maxl,
                            int* __restrict__ nact) {
  double* H = Hh + (size_t)s * (maxl + 1) * maxl;  // column-major, ld maxl + 1
  double* g = G + (size_t)s * (maxl + 1);
  double* cs = CS + (size_t)s * 2 * maxl;
  double* col = H + (size_t)j * (maxl + 1);
  for (int q = 0; q <= j; ++q) col[q] = h2 ? h[q] + h2[q] : h[q];
  col[j + 1] = hn;
  for (int q = 0; q < j; ++q) {  // earlier rotations
    const double cq = cs[2 * q], sq = cs[2 * q + 1];
    const double t1 = col[q], t2 = col[q + 1];
    col[q] = cq * t1 - sq * t2;
    col[q + 1] = sq * t1 + cq * t2;
  }
  const double d = hypot(col[j], col[j + 1]);
  const double cj = d > 0.0 ? col[j] / d : 1.0, sj = d > 0.0 ? -col[j + 1] / d : 0.0;
  cs[2 * j] = cj;
  cs[2 * j + 1] = sj;
  col[j] = d;
  col[j + 1] = 0.0;
  g[j + 1] = sj * g[j];
  g[j] = cj * g[j];
  c.rho = fabs(g[j + 1]);
  c.lgmr = j + 1;
  if (!isfinite(c.rho)) {
    c.iflag = 2;
    c.active = 0;
  } else if (c.rho <= c.tol * c.bnrm || !(hn > 0.0)) {
    c.active = 0;
  } else if (j + 1 >= maxl) {
    c.iflag = 1;
    c.active = 0;
  } else {
    atomicAdd(nact, 1);
  }
}

// One Arnoldi step j for every active simulation of an FP64 cycle: classical Gram-Schmidt
// applied twice on w = A V[:, j] against V[:, 0..j] within the simulation's segment, the
// new column of the Hessenberg matrix, DHEQR's Givens update (dheqr.f:82-176) and the
// stopping test on |g_(j+1)| (DPIGMR's RHO, dpigmr.f:340-355). nact counts the
// simulations still active after the step.
__global__ void __launch_bounds__(BBS) k_bg_arnoldi(const int* __restrict__ jdev, const int* __restrict__ seg,
                                                    double* __restrict__ V, size_t ldv, double* __restrict__ w,
                                                    BCtl* __restrict__ ctl, double* __restrict__ Hh,
                                                    double* __restrict__ G, double* __restrict__ CS, int maxl,
                                                    int* __restrict__ nact) {
  const int j = *jdev;
  __shared__ double red[33];
  __shared__ double h1[EB_GM_MAXL + 2];
  __shared__ double h2[EB_GM_MAXL + 2];
  const int s = blockIdx.x;
  BCtl& c = ctl[s];
  if (!c.active) return;
  const int i0 = seg[s], i1 = seg[s + 1];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double* vn = V + (size_t)(j + 1) * ldv;
  double* hp[2] = {h1, h2};
  for (int pass = 0; pass < 2; ++pass) {
    double* h = hp[pass];
    for (int q = wi; q <= j; q += nw) {
      const double* v = V + (size_t)q * ldv;
      double acc = 0.0;
      for (int i = i0 + lane; i < i1; i += 32) acc = fma(v[i], w[i], acc);
      acc = warp_sum<double>(acc);
      if (lane == 0) h[q] = acc;
    }
    __syncthreads();
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      double acc = 0.0;
      for (int q = 0; q <= j; ++q) acc = fma(V[(size_t)q * ldv + i], h[q], acc);
      w[i] -= acc;
    }
    __syncthreads();
  }
  double nn = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) nn = fma(w[i], w[i], nn);
  const double hn = sqrt(bblock_sum(nn, red));
  if (hn > 0.0) {
    const double rh = 1.0 / hn;  // one reciprocal: an FP64 division per element is slow on this GPU
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) vn[i] = w[i] * rh;
  }
  if (threadIdx.x == 0) bg_step_end(s, j, h1, h2, hn, c, Hh, G, CS, maxl, nact);
}

// The inner FP32 cycle's Arnoldi step j over work items (chunks of BCH rows of one
// simulation), so that a large simulation's FP64 reductions spread over several SMs
// instead of one block: partial sums of h_q = V[:, q] . w (q <= j) and of w . w per item;
// the last item of a simulation to finish (a per-simulation ticket) adds its items'
// partials in item order, forms ||w - V h|| by Pythagoras (within 1e-12 of w.w the
// vector counts as zero), the Hessenberg column, DHEQR's Givens update and the stopping
// test, as k_bg_arnoldi does, and leaves h and the norm in hbuf for k_bg_upd1.
__global__ void __launch_bounds__(BBS) k_bg_dots1(const int* __restrict__ jdev, const int4* __restrict__ items,
                                                  const int2* __restrict__ sitem, const double* __restrict__ V,
                                                  size_t ldv, const double* __restrict__ w, BCtl* __restrict__ ctl,
                                                  double* __restrict__ part, int* __restrict__ tick,
                                                  double* __restrict__ hbuf, double* __restrict__ Hh,
                                                  double* __restrict__ G, double* __restrict__ CS, int maxl,
                                                  int* __restrict__ nact) {
  const int j = *jdev;
  const int4 it = items[blockIdx.x];
  const int s = it.x;
  BCtl& c = ctl[s];
  if (!c.active) return;
  const int nc = j + 2, ldp = maxl + 2;
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int q = wi; q < nc; q += nw) {  // column j + 1: w . w
    const double* v = q <= j ? V + (size_t)q * ldv : w;
    double acc = 0.0;
    for (int i = it.y + lane; i < it.z; i += 32) acc = fma(v[i], w[i], acc);
    acc = warp_sum<double>(acc);
    if (lane == 0) part[(size_t)blockIdx.x * ldp + q] = acc;
  }
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  const int2 si = sitem[s];
  if (threadIdx.x == 0) s_last = atomicAdd(&tick[s], 1) == si.y - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  __shared__ double h1[EB_GM_MAXL + 2];
  for (int q = wi; q < nc; q += nw) {
    double acc = 0.0;
    for (int b = si.x + lane; b < si.x + si.y; b += 32) acc += __ldcg(part + (size_t)b * ldp + q);
    acc = warp_sum<double>(acc);
    if (lane == 0) h1[q] = acc;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  tick[s] = 0;
  const double ww = h1[j + 1];
  double t = ww;
  for (int q = 0; q <= j; ++q) t = fma(-h1[q], h1[q], t);
  const double hn = t > 1e-12 * ww ? sqrt(t) : 0.0;
  double* hb = hbuf + (size_t)s * ldp;
  for (int q = 0; q <= j; ++q) hb[q] = h1[q];
  hb[maxl + 1] = hn;
  bg_step_end(s, j, h1, nullptr, hn, c, Hh, G, CS, maxl, nact);
}

// V[:, j + 1] = (w - V[:, 0..j] h) / ||.|| over each work item of a simulation that
// continues (its h and norm from k_bg_dots1).
__global__ void __launch_bounds__(BBS) k_bg_upd1(const int* __restrict__ jdev, const int4* __restrict__ items,
                                                 double* __restrict__ V, size_t ldv, const double* __restrict__ w,
                                                 const BCtl* __restrict__ ctl, const double* __restrict__ hbuf,
                                                 int maxl) {
  const int j = *jdev;
  const int4 it = items[blockIdx.x];
  const int s = it.x;
  if (!ctl[s].active) return;
  __shared__ double hs[EB_GM_MAXL + 2];
  const double* hb = hbuf + (size_t)s * (maxl + 2);
  for (int q = threadIdx.x; q <= j; q += blockDim.x) hs[q] = hb[q];
  __syncthreads();
  const double rh = 1.0 / hb[maxl + 1];
  double* vn = V + (size_t)(j + 1) * ldv;
  for (int i = it.y + threadIdx.x; i < it.z; i += blockDim.x) {
    double acc = 0.0;
    for (int q = 0; q <= j; ++q) acc = fma(V[(size_t)q * ldv + i], hs[q], acc);
    vn[i] = (w[i] - acc) * rh;
  }
}

// End of a cycle: DHELS's triangular solve H y = g (dhels.f:77-96) and x += V y, per
// simulation over its segment (x = 0 first when zero_x).
__global__ void k_bg_finish(const int* __restrict__ seg, const double* __restrict__ V, size_t ldv,
                            const BCtl* __restrict__ ctl, const double* __restrict__ Hh,
                            const double* __restrict__ G, int maxl, int zero_x, const int* __restrict__ skip,
                            double* __restrict__ x) {
  __shared__ double y[EB_GM_MAXL + 1];
  const int s = blockIdx.x, i0 = seg[s], i1 = seg[s + 1];
  if (skip && skip[s]) return;
  const BCtl& c = ctl[s];
  const int m = c.lgmr;
  if (threadIdx.x == 0) {
    const double* H = Hh + (size_t)s * (maxl + 1) * maxl;
    const double* g = G + (size_t)s * (maxl + 1);
    for (int q = m - 1; q >= 0; --q) {
      double t = g[q];
      for (int r = q + 1; r < m; ++r) t -= H[(size_t)r * (maxl + 1) + q] * y[r];
      y[q] = t / H[(size_t)q * (maxl + 1) + q];
    }
  }
  __syncthreads();
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    double acc = zero_x ? 0.0 : x[i];
    for (int q = 0; q < m; ++q) acc = fma(V[(size_t)q * ldv + i], y[q], acc);
    x[i] = acc;
  }
}

// Refinement: x += d and r = b - A x (w = A x) with the relative residual per
// simulation; a simulation at or below tol is marked done (skip) for the next steps.
__global__ void k_br_update(const int* __restrict__ seg, const double* __restrict__ b, const double* __restrict__ w,
                            double* __restrict__ r, double* __restrict__ err, int* __restrict__ skip, double tol,
                            double itol0, double* __restrict__ itol, int* __restrict__ nleft) {
  __shared__ double red[33];
  const int s = blockIdx.x, i0 = seg[s], i1 = seg[s + 1];
  if (skip[s]) return;
  double rr = 0.0, bb = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double v = b[i] - w[i];
    r[i] = v;
    rr = fma(v, v, rr);
    bb = fma(b[i], b[i], bb);
  }
  rr = bblock_sum(rr, red);
  bb = bblock_sum(bb, red);
  if (threadIdx.x == 0) {
    const double e = bb > 0.0 ? sqrt(rr / bb) : 0.0;
    err[s] = e;
    if (!(e > tol)) {
      skip[s] = 1;
    } else {
      atomicAdd(nleft, 1);
      // the next inner tolerance: expected to end the solve, at most a tenth of the first
      itol[s] = fmin(itol0, fmax(0.1 * itol0, 0.5 * tol / e));
    }
  }
}

// Loop control of a cycle, in jdev = {j, continue}: j = 0 and continue = (a simulation is
// active) at the start; after each step j += 1 and continue = (still active, j < maxl),
// resetting the step's counter of active simulations. With use_h the WHILE node's
// condition is set to `continue` as well (the host-driven loop reads jdev[1]).
__global__ void k_bg_start(int nsim, const BCtl* __restrict__ ctl, int* __restrict__ jdev, int* __restrict__ nact,
                           cudaGraphConditionalHandle h, int use_h) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int any = 0;
  for (int s = 0; s < nsim; ++s) any |= ctl[s].active;
  jdev[0] = 0;
  jdev[1] = any;
  *nact = 0;
  if (use_h) cudaGraphSetConditional(h, any ? 1u : 0u);
}

__global__ void k_bg_next(int maxl, int* __restrict__ jdev, int* __restrict__ nact, cudaGraphConditionalHandle h,
                          int use_h) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int a = *nact;
  *nact = 0;
  const int j = jdev[0] + 1;
  const int cont = (a > 0 && j < maxl) ? 1 : 0;
  jdev[0] = j;
  jdev[1] = cont;
  if (use_h) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

// the operator's input: Krylov column j
__global__ void k_bg_col(int n, const int* __restrict__ jdev, const double* __restrict__ V, size_t ldv,
                         double* __restrict__ xin) {
  const double* v = V + (size_t)(*jdev) * ldv;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) xin[i] = v[i];
}

__global__ void k_bg_axpy(const int* __restrict__ seg, const int* __restrict__ skip, const double* __restrict__ d,
                          double* __restrict__ x) {
  const int s = blockIdx.x;
  if (skip[s]) return;
  for (int i = seg[s] + threadIdx.x; i < seg[s + 1]; i += blockDim.x) x[i] += d[i];
}

__global__ void k_bg_set_tol(int nsim, BCtl* __restrict__ ctl, double tol, const double* __restrict__ per_sim) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsim) ctl[s].tol = per_sim ? per_sim[s] : tol;
}

__global__ void k_bg_gather(int nsim, const BCtl* __restrict__ ctl, double* __restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsim) {
    out[3 * s] = ctl[s].rho / (ctl[s].bnrm > 0.0 ? ctl[s].bnrm : 1.0);
    out[3 * s + 1] = (double)ctl[s].lgmr;
    out[3 * s + 2] = (double)ctl[s].iflag;
  }
}

}  // namespace

// ---------------------------------------------------------------------------------
// Set-up of the batch (host) and of the forest geometry (device)
// ---------------------------------------------------------------------------------
int eb_batch_define(eb_ctx* ctx, int nsim, const int* sim_k, const double* e0) {
  if (!ctx || nsim < 0 || (nsim > 0 && !sim_k)) return EB_ERR_ARG;
  if (nsim > 0 && ctx->iwall) {
    eb_set_last_error_msg("a batch of simulations is not available in wall mode");
    return EB_ERR_ARG;
  }
  cudaSetDevice(ctx->device);
  ctx->geom_valid = false;
  ctx->tree.valid = false;
  ctx->tree_pv.valid = false;
  if (nsim == 0) {
    ctx->nsim = 0;
    ctx->sim_k.clear();
    ctx->sim_e0.clear();
    return EB_OK;
  }
  std::vector<int> k(sim_k, sim_k + nsim);
  for (int v : k)
    if (v <= 0) {
      eb_set_last_error_msg("eb_batch_define: every simulation needs at least one drop");
      return EB_ERR_ARG;
    }
  ctx->nsim = nsim;
  ctx->sim_k = k;
  ctx->sim_e0.assign(nsim, 0.0);
  if (e0) ctx->sim_e0.assign(e0, e0 + nsim);
  ctx->sim_has_e0 = e0 != nullptr;
  return EB_OK;
}

// Per-install batch data: drop -> simulation maps, segments, and the forest placement
// (a grid of 2^R x 2^R cells of side Wc, one simulation per cell, each simulation
// centred in its cell) with the translated nodes ctx->zt.
int eb_batch_install(eb_ctx* ctx) {
  cudaStream_t st = ctx->stream;
  const int S = ctx->nsim, k = ctx->k, nbk = ctx->nbk;
  int tot = 0;
  for (int v : ctx->sim_k) tot += v;
  if (tot != k) {
    eb_set_last_error_msg("batch: the simulations' drop counts do not add up to the drops installed");
    return EB_ERR_ARG;
  }
  std::vector<int> sod(k), node0(S + 1), pinf(k);
  std::vector<double> e0d(k), alpha(k);
  int d = 0;
  node0[0] = 0;
  for (int s = 0; s < S; ++s) {
    const int d0 = d;
    int nodes = 0;
    for (int q = 0; q < ctx->sim_k[s]; ++q, ++d) {
      sod[d] = s;
      pinf[d] = d0;
      nodes += ctx->nd_host[d];
    }
    node0[s + 1] = node0[s] + nodes;
    // SETVELF's electric-stress loop uses the alpha left by its last drop (stokesbubb.f:125)
    const int nlast = ctx->nd_host[d - 1];
    for (int q = d0; q < d; ++q) {
      e0d[q] = ctx->sim_e0[s];
      alpha[q] = 2.0 * EB_PI * (double)(nlast - 1) / (double)nlast;
    }
  }
  ctx->sim_node0 = node0;
  std::vector<int> sonode(nbk);
  for (int s = 0; s < S; ++s)
    for (int i = node0[s]; i < node0[s + 1]; ++i) sonode[i] = s;
  std::vector<int> seg2(S + 1);
  for (int s = 0; s <= S; ++s) seg2[s] = 2 * node0[s];
  EB_TRY(ctx->b_sim_of_drop.ensure(sizeof(int) * k));
  EB_TRY(ctx->b_pinf.ensure(sizeof(int) * k));
  EB_TRY(ctx->b_e0.ensure(sizeof(double) * k));
  EB_TRY(ctx->b_alpha.ensure(sizeof(double) * k));
  EB_TRY(ctx->b_seg1.ensure(sizeof(int) * (S + 1)));
  EB_TRY(ctx->b_seg2.ensure(sizeof(int) * (S + 1)));
  EB_TRY(ctx->b_sim_of_node.ensure(sizeof(int) * nbk));
  EB_TRY(ctx->b_box.ensure(sizeof(SimBox) * S));
  EB_TRY(ctx->b_shift.ensure(sizeof(double2) * S));
  EB_TRY(ctx->zt.ensure(sizeof(double2) * nbk));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_sim_of_drop.p, sod.data(), sizeof(int) * k, cudaMemcpyHostToDevice, st));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_pinf.p, pinf.data(), sizeof(int) * k, cudaMemcpyHostToDevice, st));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_e0.p, e0d.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_alpha.p, alpha.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_seg1.p, node0.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice, st));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_seg2.p, seg2.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice, st));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_sim_of_node.p, sonode.data(), sizeof(int) * nbk, cudaMemcpyHostToDevice, st));
  // work items of the inner Arnoldi steps: each simulation's segment in chunks of BCH rows
  for (int e = 1; e <= 2; ++e) {
    std::vector<int4> items;
    std::vector<int2> sitem(S);
    for (int sm = 0; sm < S; ++sm) {
      const int r0 = e * node0[sm], r1 = e * node0[sm + 1];
      sitem[sm].x = (int)items.size();
      for (int r = r0; r < r1; r += BCH) items.push_back(make_int4(sm, r, std::min(r1, r + BCH), 0));
      sitem[sm].y = (int)items.size() - sitem[sm].x;
    }
    DevBuf& bi = e == 1 ? ctx->b_items1 : ctx->b_items2;
    DevBuf& bs = e == 1 ? ctx->b_sitem1 : ctx->b_sitem2;
    EB_TRY(bi.ensure(sizeof(int4) * items.size()));
    EB_TRY(bs.ensure(sizeof(int2) * (size_t)S));
    EB_CUDA_TRY(cudaMemcpyAsync(bi.p, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, st));
    EB_CUDA_TRY(cudaMemcpyAsync(bs.p, sitem.data(), sizeof(int2) * (size_t)S, cudaMemcpyHostToDevice, st));
    (e == 1 ? ctx->b_nitem1 : ctx->b_nitem2) = (int)items.size();
  }
  k_sim_bbox<<<S, 256, 0, st>>>(ctx->b_seg1.as<int>(), ctx->z.as<double2>(), ctx->b_box.as<SimBox>());
  eb_count_launch(ctx);
  std::vector<SimBox> box(S);
  EB_CUDA_TRY(cudaMemcpyAsync(box.data(), ctx->b_box.p, sizeof(SimBox) * S, cudaMemcpyDeviceToHost, st));
  EB_CUDA_TRY(cudaStreamSynchronize(st));
  double wc = 0.0;
  for (const SimBox& b : box) {
    if (!std::isfinite(b.x) || !std::isfinite(b.y) || !std::isfinite(b.z) || !std::isfinite(b.w)) {
      eb_set_last_error_msg("non-finite node coordinate");
      return EB_ERR_NAN;
    }
    wc = std::max(wc, std::max(b.y - b.x, b.w - b.z));
  }
  if (!(wc > 0.0)) wc = 1.0;
  // a quarter of margin: PVINTEV's interpolated points between the nodes lie slightly
  // outside the nodes' box and must stay in their simulation's cell
  wc *= 1.25;
  int R = 0;
  while ((1 << R) * (1 << R) < S) ++R;
  const int G = 1 << R;
  std::vector<double2> shift(S);
  for (int s = 0; s < S; ++s) {
    const int gx = s % G, gy = s / G;
    const double cx = 0.5 * (box[s].x + box[s].y), cy = 0.5 * (box[s].z + box[s].w);
    shift[s] = make_double2((gx + 0.5) * wc - cx, (gy + 0.5) * wc - cy);
  }
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_shift.p, shift.data(), sizeof(double2) * S, cudaMemcpyHostToDevice, st));
  k_translate<<<nblk(nbk, 256), 256, 0, st>>>(nbk, ctx->b_sim_of_node.as<int>(), ctx->b_shift.as<double2>(),
                                              ctx->z.as<double2>(), ctx->zt.as<double2>());
  eb_count_launch(ctx);
  ctx->b_R = R;
  ctx->b_sq[0] = G * wc;
  ctx->b_sq[1] = 0.0;
  ctx->b_sq[2] = 0.0;
  return eb_check_launch(ctx, "batch install");
}

int eb_batch_translate_fine(eb_ctx* ctx, double2* zf) {
  k_translate_fine<<<ctx->k, 256, 0, ctx->stream>>>(ctx->start.as<int>(), ctx->b_sim_of_drop.as<int>(),
                                                    ctx->b_shift.as<double2>(), zf);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "batch fine translate");
}

// ---------------------------------------------------------------------------------
// Batched solves
// ---------------------------------------------------------------------------------
namespace {

struct BatchWork {
  eb_ctx* ctx;
  int n, S, maxl;
  const int* seg;
  const int4* items;  // work items of the inner Arnoldi steps
  const int2* sitem;
  int nitem;
  double *part, *hbuf;
  int* tick;
  double *V, *H, *G, *CS, *w, *xin;
  BCtl* ctl;
  int* nact;
  int* jdev;  // {step j, continue}
};

// One GMRES cycle on every simulation not marked in skip: solves A x = b per segment to
// the per-simulation relative tolerance in ctl (x0 = x when have_x0, else 0). The Arnoldi
// steps run until no simulation is active or MAXL is reached, each step one operator
// apply and one k_bg_arnoldi over all simulations.
int bg_enqueue_pre(BatchWork& B, eb_op_fn op, int prec, const double* b, double* x, bool have_x0,
                   const int* skip, cudaGraphConditionalHandle h, int use_h) {
  eb_ctx* ctx = B.ctx;
  cudaStream_t st = ctx->stream;
  if (have_x0) EB_TRY(op(ctx, x, B.w, prec));
  k_bg_init<<<B.S, BBS, 0, st>>>(B.seg, b, have_x0 ? B.w : nullptr, nullptr, B.V, B.ctl, B.G, skip, B.maxl);
  k_bg_start<<<1, 32, 0, st>>>(B.S, B.ctl, B.jdev, B.nact, h, use_h);
  ctx->launches += 2;
  return eb_check_launch(ctx, "batched gmres (start)");
}

int bg_enqueue_step(BatchWork& B, eb_op_fn op, int prec, cudaGraphConditionalHandle h, int use_h) {
  eb_ctx* ctx = B.ctx;
  cudaStream_t st = ctx->stream;
  const size_t ldv = (size_t)B.n;
  k_bg_col<<<std::min(nblk(B.n, 256), 2 * ctx->nsm), 256, 0, st>>>(B.n, B.jdev, B.V, ldv, B.xin);
  eb_count_launch(ctx);
  EB_TRY(op(ctx, B.xin, B.w, prec));
  if (prec == EB_FP32) {
    // one-pass step over work items: partial sums, then the update
    k_bg_dots1<<<B.nitem, BBS, 0, st>>>(B.jdev, B.items, B.sitem, B.V, ldv, B.w, B.ctl, B.part, B.tick, B.hbuf,
                                        B.H, B.G, B.CS, B.maxl, B.nact);
    k_bg_upd1<<<B.nitem, BBS, 0, st>>>(B.jdev, B.items, B.V, ldv, B.w, B.ctl, B.hbuf, B.maxl);
    ctx->launches += 2;
  } else {
    k_bg_arnoldi<<<B.S, BBS, 0, st>>>(B.jdev, B.seg, B.V, ldv, B.w, B.ctl, B.H, B.G, B.CS, B.maxl, B.nact);
    eb_count_launch(ctx);
  }
  k_bg_next<<<1, 32, 0, st>>>(B.maxl, B.jdev, B.nact, h, use_h);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "batched gmres (step)");
}

int bg_enqueue_post(BatchWork& B, bool have_x0, const int* skip, double* x) {
  eb_ctx* ctx = B.ctx;
  k_bg_finish<<<B.S, BBS, 0, ctx->stream>>>(B.seg, B.V, (size_t)B.n, B.ctl, B.H, B.G, B.maxl, have_x0 ? 0 : 1,
                                            skip, x);
  eb_count_launch(ctx);
  return eb_check_launch(ctx, "batched gmres (finish)");
}

// The cycle as one CUDA graph (pre, a conditional WHILE node over the steps, post),
// cached under the geometry's shape and the buffer epoch like the single solves' graphs.
int bg_cycle_graph(BatchWork& B, eb_op_fn op, int prec, const double* b, double* x, bool have_x0,
                   const int* skip, int slot) {
  eb_ctx* ctx = B.ctx;
  unsigned long long key[8] = {(unsigned long long)slot, (unsigned long long)(uintptr_t)op,
                               (unsigned long long)B.n, (unsigned long long)B.maxl, ctx->geom_shape,
                               eb_devbuf_epoch(), (unsigned long long)B.S, (unsigned long long)prec};
  GmGraph& G = ctx->bgraph[slot];
  if (!G.valid || !std::equal(key, key + 8, G.key)) {
    G.destroy();
    const unsigned long long e0 = eb_devbuf_epoch();
    EB_CUDA_TRY(cudaGraphCreate(&G.graph, 0));
    cudaGraphConditionalHandle h;
    EB_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, G.graph, 0, cudaGraphCondAssignDefault));
    std::vector<cudaGraphNode_t> sinks;
    bool lost = false;
    int st = eb_capture_into(ctx, G.graph, nullptr, 0, &sinks, &G.n_pre, &lost,
                             [&]() { return bg_enqueue_pre(B, op, prec, b, x, have_x0, skip, h, 1); });
    if (st != EB_OK) {
      if (lost) G.graph = nullptr;
      G.destroy();
      return st;
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t ncond;
    EB_CUDA_TRY(cudaGraphAddNode(&ncond, G.graph, sinks.data(), nullptr, sinks.size(), &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    bool body_lost = false;
    st = eb_capture_into(ctx, body, nullptr, 0, nullptr, &G.n_body, &body_lost,
                         [&]() { return bg_enqueue_step(B, op, prec, h, 1); });
    if (st == EB_OK)
      st = eb_capture_into(ctx, G.graph, &ncond, 1, nullptr, &G.n_post, &lost,
                           [&]() { return bg_enqueue_post(B, have_x0, skip, x); });
    if (st == EB_OK && eb_devbuf_epoch() != e0) st = EB_ERR_CUDA;  // a buffer moved: retry later
    if (st != EB_OK) {
      if (lost || body_lost) G.graph = nullptr;
      G.destroy();
      cudaGetLastError();
      return st;
    }
    EB_CUDA_TRY(cudaGraphInstantiate(&G.exec, G.graph, cudaGraphInstantiateFlagUseNodePriority));
    memcpy(G.key, key, sizeof(key));
    G.valid = true;
  }
  EB_CUDA_TRY(cudaGraphLaunch(G.exec, ctx->stream));
  return EB_OK;
}

// defer_iters: the cycle's iteration count is queued to ctx->b_host_act[2] without a wait
// (the caller reads it after its own synchronisation) instead of added to *total_iters.
int bg_cycle(BatchWork& B, eb_op_fn op, int prec, const double* b, double* x, bool have_x0,
             const int* skip, int* total_iters, int slot, bool defer_iters = false) {
  eb_ctx* ctx = B.ctx;
  cudaStream_t st = ctx->stream;
  const long long l0 = ctx->launches;
  bool done = false;
  if (ctx->opts.graphs > 0 && !ctx->profiling) {
    // a failed capture (a buffer grew while capturing) falls back to the host loop once
    done = bg_cycle_graph(B, op, prec, b, x, have_x0, skip, slot) == EB_OK;
  }
  if (!done) {
    ctx->launches = l0;
    cudaGraphConditionalHandle h0 = 0;
    EB_TRY(bg_enqueue_pre(B, op, prec, b, x, have_x0, skip, h0, 0));
    int* hact = ctx->b_host_act;
    for (int j = 0; j < B.maxl; ++j) {
      EB_CUDA_TRY(cudaMemcpyAsync(hact, B.jdev + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
      EB_CUDA_TRY(cudaStreamSynchronize(st));
      if (*hact == 0) break;
      EB_TRY(bg_enqueue_step(B, op, prec, h0, 0));
    }
    EB_TRY(bg_enqueue_post(B, have_x0, skip, x));
  }
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_host_act + 2, B.jdev, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (defer_iters) return EB_OK;
  EB_CUDA_TRY(cudaStreamSynchronize(st));
  *total_iters += ctx->b_host_act[2];
  return EB_OK;
}

}  // namespace

int eb_batch_solve(eb_ctx* ctx, int n, eb_op_fn op, bool stokes, const double* rhs, double* soln, int mode,
                   eb_solve_info* info, int mem) {
  cudaStream_t st = ctx->stream;
  const int S = ctx->nsim;
  int maxl = std::min(ctx->opts.maxl, EB_GM_MAXL);
  BatchWork B{};
  B.ctx = ctx;
  B.n = n;
  B.S = S;
  B.maxl = maxl;
  B.seg = stokes ? ctx->b_seg2.as<int>() : ctx->b_seg1.as<int>();
  B.items = stokes ? ctx->b_items2.as<int4>() : ctx->b_items1.as<int4>();
  B.sitem = stokes ? ctx->b_sitem2.as<int2>() : ctx->b_sitem1.as<int2>();
  B.nitem = stokes ? ctx->b_nitem2 : ctx->b_nitem1;
  EB_TRY(ctx->b_part.ensure(sizeof(double) * (size_t)std::max(ctx->b_nitem2, 1) * (maxl + 2)));
  EB_TRY(ctx->b_hbuf.ensure(sizeof(double) * (size_t)S * (maxl + 2)));
  EB_TRY(ctx->b_tick.ensure(sizeof(int) * (size_t)S));
  EB_CUDA_TRY(cudaMemsetAsync(ctx->b_tick.p, 0, sizeof(int) * (size_t)S, st));
  B.part = ctx->b_part.as<double>();
  B.hbuf = ctx->b_hbuf.as<double>();
  B.tick = ctx->b_tick.as<int>();
  EB_TRY(ctx->gV.ensure(sizeof(double) * (size_t)n * (maxl + 1)));
  EB_TRY(ctx->gH.ensure(sizeof(double) * (size_t)S * (maxl + 1) * (maxl + 1)));
  EB_TRY(ctx->b_G.ensure(sizeof(double) * (size_t)S * (maxl + 1)));
  EB_TRY(ctx->b_CS.ensure(sizeof(double) * (size_t)S * 2 * maxl));
  EB_TRY(ctx->b_ctl.ensure(sizeof(BCtl) * (size_t)S));
  EB_TRY(ctx->b_misc.ensure(sizeof(int) * (6 + (size_t)S) + sizeof(double) * 5 * (size_t)S));
  EB_TRY(ctx->gWbuf.ensure(sizeof(double) * n));
  EB_TRY(ctx->gXin.ensure(sizeof(double) * n));
  EB_TRY(ctx->gR.ensure(sizeof(double) * n));
  EB_TRY(ctx->gX.ensure(sizeof(double) * n));
  EB_TRY(ctx->gD.ensure(sizeof(double) * n));
  EB_TRY(ctx->gZ.ensure(sizeof(double) * n));
  if (!ctx->b_host_act) EB_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&ctx->b_host_act), sizeof(int) * 4));
  B.V = ctx->gV.as<double>();
  B.H = ctx->gH.as<double>();
  B.G = ctx->b_G.as<double>();
  B.CS = ctx->b_CS.as<double>();
  B.ctl = ctx->b_ctl.as<BCtl>();
  B.w = ctx->gWbuf.as<double>();
  B.xin = ctx->gXin.as<double>();
  int* misc = ctx->b_misc.as<int>();
  B.nact = misc;
  int* nleft = misc + 1;
  B.jdev = misc + 2;
  int* skip = misc + 4;
  double* err = reinterpret_cast<double*>(skip + S + (S & 1));  // 8-byte aligned
  double* itol = err + S;
  double* gat = itol + S;  // 3 per simulation
  double* b = ctx->gR.as<double>();
  double* x = ctx->gX.as<double>();
  cudaMemcpyKind kin = mem == EB_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  EB_CUDA_TRY(cudaMemcpyAsync(b, rhs, sizeof(double) * n, kin, st));
  eb_solve_info inf{};
  std::vector<double> hg(3 * (size_t)S);
  if (mode == EB_SOLVE_FP64) {
    // x0 = b as SOLVEI / SOLVE_LAPL set it (stokesbubb.f:346-349)
    EB_CUDA_TRY(cudaMemcpyAsync(x, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    k_bg_set_tol<<<nblk(S, 128), 128, 0, st>>>(S, B.ctl, ctx->opts.gmres_tol, nullptr);
    eb_count_launch(ctx);
    int its = 0;
    EB_TRY(bg_cycle(B, op, EB_FP64, b, x, true, nullptr, &its, 0));
    k_bg_gather<<<nblk(S, 128), 128, 0, st>>>(S, B.ctl, gat);
    EB_CUDA_TRY(cudaMemcpyAsync(hg.data(), gat, sizeof(double) * 3 * S, cudaMemcpyDeviceToHost, st));
    EB_CUDA_TRY(cudaStreamSynchronize(st));
    inf.outer = 1;
    inf.iters = its;
    inf.matvecs64 = its + 1;
    for (int s = 0; s < S; ++s) {
      inf.err = std::max(inf.err, hg[3 * s]);
      inf.ierr = std::max(inf.ierr, (int)hg[3 * s + 2]);
    }
  } else {
    // refinement from x = 0: inner FP32 cycles on r, x += d, r = b - A x in the FP64
    // arithmetic of the residuals, per simulation until its residual is at tol
    double* r = ctx->gZ.as<double>();
    double* dd = ctx->gD.as<double>();
    EB_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
    EB_CUDA_TRY(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    EB_CUDA_TRY(cudaMemsetAsync(skip, 0, sizeof(int) * S, st));
    int outer = 0, left = S;
    for (outer = 1; outer <= ctx->opts.max_outer && left > 0; ++outer) {
      k_bg_set_tol<<<nblk(S, 128), 128, 0, st>>>(S, B.ctl, ctx->opts.inner_tol, outer > 1 ? itol : nullptr);
      eb_count_launch(ctx);
      // the cycle's iteration count is read after this step's one wait (below)
      EB_TRY(bg_cycle(B, op, EB_FP32, r, dd, false, skip, nullptr, 1, true));
      // x += d on the simulations that took part
      k_bg_axpy<<<S, BBS, 0, st>>>(B.seg, skip, dd, x);
      eb_count_launch(ctx);
      EB_TRY(op(ctx, x, B.w, eb_resid_prec(ctx)));
      inf.matvecs64 += 1;
      EB_CUDA_TRY(cudaMemsetAsync(nleft, 0, sizeof(int), st));
      k_br_update<<<S, BBS, 0, st>>>(B.seg, b, B.w, r, err, skip, ctx->opts.gmres_tol, ctx->opts.inner_tol, itol,
                                     nleft);
      eb_count_launch(ctx);
      EB_CUDA_TRY(cudaMemcpyAsync(ctx->b_host_act + 1, nleft, sizeof(int), cudaMemcpyDeviceToHost, st));
      EB_CUDA_TRY(cudaStreamSynchronize(st));
      left = ctx->b_host_act[1];
      inf.iters += ctx->b_host_act[2];
      inf.matvecs32 += ctx->b_host_act[2];
    }
    std::vector<double> he(S);
    EB_CUDA_TRY(cudaMemcpyAsync(he.data(), err, sizeof(double) * S, cudaMemcpyDeviceToHost, st));
    EB_CUDA_TRY(cudaStreamSynchronize(st));
    inf.outer = outer - 1;
    for (double e : he) inf.err = std::max(inf.err, e);
    inf.ierr = left > 0 ? 1 : 0;
    if (!std::isfinite(inf.err)) {
      eb_set_last_error_msg("non-finite residual");
      return EB_ERR_NAN;
    }
  }
  cudaMemcpyKind kout = mem == EB_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  EB_CUDA_TRY(cudaMemcpyAsync(soln, x, sizeof(double) * n, kout, st));
  EB_CUDA_TRY(cudaStreamSynchronize(st));
  if (info) *info = inf;
  return EB_OK;
}
