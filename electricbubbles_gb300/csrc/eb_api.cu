// C ABI of libeb_gb300: context, geometry, operator applies and the Fortran shims.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "eb_internal.h"
#include "eb_post.cuh"

// ---------------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------------
static thread_local std::string g_last_error;

void eb_set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  g_last_error = buf;
}
void eb_set_last_error_msg(const char* msg) { g_last_error = msg; }

int eb_check_launch(eb_ctx* ctx, const char* name) {
  (void)ctx;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    eb_set_last_cuda_error(e, name, __FILE__, __LINE__);
    return EB_ERR_CUDA;
  }
  return EB_OK;
}

cudaStream_t eb_stream(eb_ctx* ctx) { return ctx->stream; }

namespace {

inline int nblk(long long n, int bs) { return (int)((n + bs - 1) / bs); }

// Per-drop reductions of FASMVP (stokesbubb.f:549-565): za_k = h sum dens,
// pk_k = sum 2 h Re(dens dz/(z - zk)^2) / pi = sum Re(dens w) with the per-node weights
// w = (2 h / pi) dz / (z - zk)^2 of k_pk_weights. One block per drop.
__global__ void k_drop_reduce_stokes(const int* __restrict__ start, const double2* __restrict__ dens,
                                     const double2* __restrict__ pkw, double2* __restrict__ za,
                                     double* __restrict__ pk) {
  __shared__ double s[3][256];
  int b = blockIdx.x;
  int i0 = start[b], i1 = start[b + 1];
  double h = 2.0 * EB_PI / (double)(i1 - i0);
  double ax = 0.0, ay = 0.0, pp = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double2 u = dens[i], w = pkw[i];
    pp = fma(u.x, w.x, fma(-u.y, w.y, pp));
    ax += u.x;
    ay += u.y;
  }
  s[0][threadIdx.x] = ax; s[1][threadIdx.x] = ay; s[2][threadIdx.x] = pp;
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
    za[b] = make_double2(h * s[0][0], h * s[1][0]);
    pk[b] = s[2][0];
  }
}

// Per-node weight of the singular-term sums, once per geometry.
__device__ __forceinline__ double2 pk_weight(int i, const int* __restrict__ drop_of,
                                             const double* __restrict__ hpt, const double2* __restrict__ z,
                                             const double2* __restrict__ dz, const double2* __restrict__ zk) {
  const double2 c = zk[drop_of[i]];
  const double2 d = make_double2(z[i].x - c.x, z[i].y - c.y);
  const double2 q = cdiv<double>(dz[i], cmul<double>(d, d));
  const double f = 2.0 * hpt[i] / EB_PI;
  return make_double2(f * q.x, f * q.y);
}

// Constraint sums the reference writes past YY(N) (laplace.f:252-259): h s' u per drop.
__global__ void k_lap_constraints(const int* __restrict__ start, const double* __restrict__ u,
                                  const double* __restrict__ dsda, double* __restrict__ sums) {
  __shared__ double s[256];
  int b = blockIdx.x;
  int i0 = start[b], i1 = start[b + 1];
  double h = 2.0 * EB_PI / (double)(i1 - i0), acc = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) acc += h * dsda[i] * u[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[b] = s[0];
}

__global__ void k_fill_drop(int k, const int* __restrict__ start, int* __restrict__ drop_of,
                            double* __restrict__ hpt) {
  int b = blockIdx.x;
  if (b >= k) return;
  int i0 = start[b], i1 = start[b + 1];
  double h = 2.0 * EB_PI / (double)(i1 - i0);
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    drop_of[i] = b;
    hpt[i] = h;
  }
}

// Per-node coefficients of the post-processing and the singular-sum weights.
__global__ void k_post_coefs(int nbk, const double2* __restrict__ dz, const double* __restrict__ dsda,
                             const double* __restrict__ kappa, const double* __restrict__ hpt,
                             double* __restrict__ c1, double2* __restrict__ c2, double* __restrict__ d,
                             float* __restrict__ c1f, float2* __restrict__ c2f, float* __restrict__ df,
                             const int* __restrict__ drop_of, const double2* __restrict__ z,
                             const double2* __restrict__ zk, double2* __restrict__ pkw) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbk) return;
  eb_post_coefs(t, dz, dsda, kappa, hpt, c1, c2, d, c1f, c2f, df);
  pkw[t] = pk_weight(t, drop_of, hpt, z, dz, zk);
}

int copy_in(eb_ctx* ctx, DevBuf& buf, const void* src, size_t bytes, int mem) {
  EB_TRY(buf.ensure(bytes));
  EB_CUDA_TRY(cudaMemcpyAsync(buf.p, src, bytes,
                              mem == EB_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                              ctx->stream));
  return EB_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------
// Context. The public functions are declared extern "C" in eb_gb300.h, which gives
// these definitions C linkage.
// ---------------------------------------------------------------------------------

int eb_version(void) { return EB_GB300_VERSION; }

const char* eb_status_string(int s) {
  switch (s) {
    case EB_OK: return "ok";
    case EB_ERR_ARG: return "invalid argument";
    case EB_ERR_CUDA: return "CUDA error";
    case EB_ERR_NOGEOM: return "no geometry installed";
    case EB_ERR_WORKSPACE: return "size exceeds capacity";
    case EB_ERR_TOL: return "tolerance needs too many expansion terms";
    case EB_ERR_NAN: return "non-finite value";
    case EB_ERR_NOT_CONVERGED: return "GMRES did not converge";
    case EB_ERR_NODEVICE: return "no CUDA device";
    case EB_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

const char* eb_last_error(void) { return g_last_error.c_str(); }

void eb_opts_default(eb_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->p64 = 44;
  o->p32 = 20;
  o->leaf64 = 32;
  o->leaf_cap = EB_LEAF_CAP;
  o->tol64 = 1e-15;
  o->tol32 = 1e-7;
  o->maxl = 100;
  o->gmres_tol = 1e-10;
  o->inner_tol = 1e-5;
  o->max_outer = 8;
  o->device = 0;
  o->graphs = 1;
  o->df64 = -1;
  o->resid_df = 1;
  o->m2l_tc = -1;
  o->lap_deflate = -1;
  o->direct_max = 1024;
  o->adj_df = 1;
}

int eb_ctx_create(eb_ctx** out, const eb_opts* opts) {
  if (!out) return EB_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= 0) {
    eb_set_last_error_msg("no CUDA device is available");
    return EB_ERR_NODEVICE;
  }
  eb_ctx* c = new eb_ctx();
  eb_opts_default(&c->opts);
  if (opts) {
    eb_opts o = *opts;
    eb_opts d;
    eb_opts_default(&d);
    if (o.p64 <= 0) o.p64 = d.p64;
    if (o.p32 <= 0) o.p32 = d.p32;
    if (o.leaf64 <= 0) o.leaf64 = d.leaf64;
    if (o.leaf_cap <= 0) o.leaf_cap = d.leaf_cap;
    if (o.tol64 <= 0) o.tol64 = d.tol64;
    if (o.tol32 <= 0) o.tol32 = d.tol32;
    if (o.maxl <= 0) o.maxl = d.maxl;
    if (o.gmres_tol <= 0) o.gmres_tol = d.gmres_tol;
    if (o.inner_tol <= 0) o.inner_tol = d.inner_tol;
    if (o.max_outer <= 0) o.max_outer = d.max_outer;
    if (o.graphs == 0) o.graphs = d.graphs;
    if (o.df64 == 0) o.df64 = d.df64;
    if (o.resid_df == 0) o.resid_df = d.resid_df;
    if (o.m2l_tc == 0) o.m2l_tc = d.m2l_tc;
    if (o.lap_deflate == 0) o.lap_deflate = d.lap_deflate;
    if (o.direct_max == 0) o.direct_max = d.direct_max;
    if (o.adj_df == 0) o.adj_df = d.adj_df;
    c->opts = o;
  }
  if (c->opts.device < 0 || c->opts.device >= ndev) {
    delete c;
    eb_set_last_error_msg("device ordinal out of range");
    return EB_ERR_ARG;
  }
  c->device = c->opts.device;
  e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  // The capture stream runs at the highest priority and the side stream (the near field,
  // concurrent with the latency-bound expansion chain) at the lowest, so that the
  // chain's blocks are scheduled first; captured graphs keep the per-node priorities.
  int prio_least = 0, prio_greatest = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->cap_stream, cudaStreamNonBlocking, prio_greatest);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->side_stream, cudaStreamNonBlocking, prio_least);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_c, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_p2p, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev_near0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev_near1);
  if (e != cudaSuccess) {
    eb_set_last_cuda_error(e, "context setup", __FILE__, __LINE__);
    delete c;
    return EB_ERR_CUDA;
  }
  c->stream = c->own_stream;
  int st = eb_tables_init(c);
  if (st != EB_OK) {
    eb_ctx_destroy(c);
    return st;
  }
  *out = c;
  return EB_OK;
}

int eb_ctx_destroy(eb_ctx* ctx) {
  if (!ctx) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev_near0) cudaEventDestroy(ctx->ev_near0);
  if (ctx->ev_near1) cudaEventDestroy(ctx->ev_near1);
  for (GmGraph& g : ctx->gcache) g.destroy();
  if (ctx->b_host_act) cudaFreeHost(ctx->b_host_act);
  if (ctx->h_flux) cudaFreeHost(ctx->h_flux);
  if (ctx->h_defer) cudaFreeHost(ctx->h_defer);
  if (ctx->h_spec) cudaFreeHost(ctx->h_spec);
  if (ctx->h_bad) cudaFreeHost(ctx->h_bad);
  for (GmGraph& g : ctx->bgraph) g.destroy();
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
  if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->ev_c) cudaEventDestroy(ctx->ev_c);
  if (ctx->ev_p2p) cudaEventDestroy(ctx->ev_p2p);
  delete ctx;
  eb_devbuf_collect();
  return EB_OK;
}

int eb_ctx_set_stream(eb_ctx* ctx, void* s) {
  if (!ctx) return EB_ERR_ARG;
  ctx->stream = s ? (cudaStream_t)s : ctx->own_stream;
  return EB_OK;
}

int eb_ctx_sync(eb_ctx* ctx) {
  if (!ctx) return EB_ERR_ARG;
  EB_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return EB_OK;
}

long long eb_ctx_launch_count(eb_ctx* ctx) { return ctx ? ctx->launches : -1; }

int eb_ctx_set_profiling(eb_ctx* ctx, int enable) {
  if (!ctx) return EB_ERR_ARG;
  ctx->profiling = enable != 0;
  for (int k = 0; k < 3; ++k) {
    ctx->prof_launch[k] = 0;
    ctx->prof_ms[k] = 0.0;
  }
  return EB_OK;
}

int eb_ctx_kernel_time(eb_ctx* ctx, int cls, long long* launches, double* total_ms) {
  if (!ctx || cls < 0 || cls > 2) return EB_ERR_ARG;
  if (launches) *launches = ctx->prof_launch[cls];
  if (total_ms) *total_ms = ctx->prof_ms[cls];
  return EB_OK;
}

int eb_ctx_tree_info(eb_ctx* ctx, eb_tree_info* info) {
  if (!ctx || !info) return EB_ERR_ARG;
  if (!ctx->tree.valid) return EB_ERR_NOGEOM;
  info->npoints = ctx->tree.n;
  info->levels = ctx->tree.L;
  info->nboxes = ctx->tree.nbox;
  info->nleaves = ctx->tree.nleaf;
  EB_TRY(eb_tree_pairs(ctx, ctx->tree));
  info->v_pairs = ctx->tree.v_pairs;
  info->u_pairs = ctx->tree.u_pairs;
  info->w_pairs = ctx->tree.w_pairs;
  info->p = ctx->last_p;
  return EB_OK;
}

// ---------------------------------------------------------------------------------
// Geometry
// ---------------------------------------------------------------------------------
int eb_set_geometry(eb_ctx* ctx, int k, const int* nd, const double* z, const double* dz,
                    const double* dsda, const double* kappa, const double* zk, int mem) {
  if (!ctx || k <= 0 || !nd || !z || !dz || !dsda || !kappa || !zk) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  std::vector<int> st(k + 1, 0);
  for (int b = 0; b < k; ++b) {
    if (nd[b] < 2) {
      eb_set_last_error_msg("every drop needs at least 2 nodes");
      return EB_ERR_ARG;
    }
    st[b + 1] = st[b] + nd[b];
  }
  int nbk = st[k];
  ctx->geom_valid = false;
  ctx->ckern_valid = false;
  ctx->k = k;
  ctx->nbk = nbk;
  ctx->nd_host.assign(nd, nd + k);
  ctx->start_host = st;
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->nd.ensure(sizeof(int) * k));
  EB_TRY(ctx->start.ensure(sizeof(int) * (k + 1)));
  EB_TRY(ctx->drop_of.ensure(sizeof(int) * nbk));
  EB_TRY(ctx->hpt.ensure(sizeof(double) * nbk));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->nd.p, nd, sizeof(int) * k, cudaMemcpyHostToDevice, s));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->start.p, st.data(), sizeof(int) * (k + 1), cudaMemcpyHostToDevice, s));
  EB_TRY(copy_in(ctx, ctx->z, z, sizeof(double2) * nbk, mem));
  EB_TRY(copy_in(ctx, ctx->dz, dz, sizeof(double2) * nbk, mem));
  EB_TRY(copy_in(ctx, ctx->dsda, dsda, sizeof(double) * nbk, mem));
  EB_TRY(copy_in(ctx, ctx->kappa, kappa, sizeof(double) * nbk, mem));
  EB_TRY(copy_in(ctx, ctx->zk, zk, sizeof(double2) * k, mem));
  k_fill_drop<<<k, 256, 0, s>>>(k, ctx->start.as<int>(), ctx->drop_of.as<int>(), ctx->hpt.as<double>());
  eb_count_launch(ctx);
  EB_TRY(ctx->pc1.ensure(sizeof(double) * nbk));
  EB_TRY(ctx->pc2.ensure(sizeof(double2) * nbk));
  EB_TRY(ctx->plap.ensure(sizeof(double) * nbk));
  EB_TRY(ctx->pc1f.ensure(sizeof(float) * nbk));
  EB_TRY(ctx->pc2f.ensure(sizeof(float2) * nbk));
  EB_TRY(ctx->plapf.ensure(sizeof(float) * nbk));
  EB_TRY(ctx->pkw.ensure(sizeof(double2) * nbk));
  k_post_coefs<<<nblk(nbk, 256), 256, 0, s>>>(nbk, ctx->dz.as<double2>(), ctx->dsda.as<double>(),
                                             ctx->kappa.as<double>(), ctx->hpt.as<double>(),
                                             ctx->pc1.as<double>(), ctx->pc2.as<double2>(),
                                             ctx->plap.as<double>(), ctx->pc1f.as<float>(),
                                             ctx->pc2f.as<float2>(), ctx->plapf.as<float>(),
                                             ctx->drop_of.as<int>(), ctx->z.as<double2>(),
                                             ctx->zk.as<double2>(), ctx->pkw.as<double2>());
  eb_count_launch(ctx);
  if (ctx->nsim > 0) EB_TRY(eb_batch_install(ctx));  // a batch: nodes moved into their cells
  EB_TRY(eb_geom_tree(ctx));
  ctx->geom_valid = true;
  ctx->geom_version++;
  eb_devbuf_collect();
  return EB_OK;
}

// The node tree of the installed geometry (a forest for a batch of simulations), and
// the hash of everything a captured solve graph takes from it by value.
int eb_geom_tree(eb_ctx* ctx) {
  const int nbk = ctx->nbk;
  if (ctx->nsim > 0)
    EB_TRY(eb_tree_build(ctx, ctx->tree, ctx->zt.as<double2>(), nbk, ctx->opts.leaf64, ctx->opts.leaf_cap,
                         ctx->b_sq, ctx->b_R));
  else
    EB_TRY(eb_tree_build(ctx, ctx->tree, ctx->z.as<double2>(), nbk, ctx->opts.leaf64, ctx->opts.leaf_cap,
                         nullptr, 0, ctx->iwall));
  ctx->tree_pv.valid = false;
  if (ctx->iwall) {  // EXTRACTDAT's xleft and slength (the root square without its 1e-9 margin)
    ctx->xleft = ctx->tree.x0;
    ctx->slength = ctx->tree.W / (1.0 + 1e-9);
  }
  {
    const EbTree& t = ctx->tree;
    unsigned long long h = 1469598103934665603ull;  // FNV-1a over the fields' bytes
    auto mix = [&h](const void* p, size_t nb) {
      const unsigned char* c = static_cast<const unsigned char*>(p);
      for (size_t i = 0; i < nb; ++i) h = (h ^ c[i]) * 1099511628211ull;
    };
    const int ints[] = {t.n, ctx->nbk, ctx->k, t.L, t.nbox, t.nleaf, t.ngroup, t.ntile, t.nchunk, t.chunk_lmin,
                        t.lend, t.cap, (int)t.nu, (int)t.nw, t.wall, t.ld};
    mix(ints, sizeof(ints));
    mix(t.lev_off, sizeof(int) * (size_t)(t.L + 2));
    const double dbl[] = {t.W, t.x0, t.y0};
    mix(dbl, sizeof(dbl));
    ctx->geom_shape = h;
  }
  return EB_OK;
}

int eb_set_wall(eb_ctx* ctx, int iwall) {
  if (!ctx) return EB_ERR_ARG;
  iwall = iwall ? 1 : 0;
  if (iwall && ctx->nsim > 0) {
    eb_set_last_error_msg("wall-bounded flow is not available for a batch of simulations");
    return EB_ERR_ARG;
  }
  if (iwall == ctx->iwall) return EB_OK;
  cudaSetDevice(ctx->device);
  ctx->iwall = iwall;
  if (ctx->geom_valid) {
    const int st = eb_geom_tree(ctx);
    if (st != EB_OK) {
      ctx->geom_valid = false;
      return st;
    }
    ctx->geom_version++;
    eb_devbuf_collect();
  }
  return EB_OK;
}

int eb_get_wall(eb_ctx* ctx, int* iwall, double* xleft, double* slength) {
  if (!ctx) return EB_ERR_ARG;
  if (iwall) *iwall = ctx->iwall;
  if (xleft) *xleft = ctx->xleft;
  if (slength) *slength = ctx->slength;
  return EB_OK;
}

// ---------------------------------------------------------------------------------
// Operators on device vectors
// ---------------------------------------------------------------------------------
int eb_stokes_sum_dev(eb_ctx* ctx, const double2* dens, int sign, double2* gradw, int prec) {
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  return eb_fmm_apply(ctx, ctx->tree, 0, sign, prec, dens, ctx->dz.as<double2>(),
                      ctx->hpt.as<double>(), gradw);
}

int eb_stokes_matvec_dev(eb_ctx* ctx, const double* x, double* y, int prec) {
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  cudaStream_t s = ctx->stream;
  const int k = ctx->k;
  const double2* dens = reinterpret_cast<const double2*>(x);
  EB_TRY(ctx->za.ensure(sizeof(double2) * k));
  EB_TRY(ctx->pk.ensure(sizeof(double) * k));
  // the per-drop sums run on the side stream, overlapping the FMM; the leaf kernel, whose
  // fused post-processing reads them, waits for them
  EB_CUDA_TRY(cudaEventRecord(ctx->ev_fork, s));
  EB_CUDA_TRY(cudaStreamWaitEvent(ctx->side_stream, ctx->ev_fork, 0));
  k_drop_reduce_stokes<<<k, 256, 0, ctx->side_stream>>>(ctx->start.as<int>(), dens, ctx->pkw.as<double2>(),
                                                       ctx->za.as<double2>(), ctx->pk.as<double>());
  eb_count_launch(ctx);
  EB_CUDA_TRY(cudaEventRecord(ctx->ev_join, ctx->side_stream));
  EbPost post{1, dens, nullptr, ctx->z.as<double2>(), ctx->dz.as<double2>(), ctx->hpt.as<double>(),
               ctx->pc1.as<double>(), ctx->pc2.as<double2>(), ctx->drop_of.as<int>(),
               ctx->za.as<double2>(), ctx->pk.as<double>(), y, ctx->pc1f.as<float>(),
               ctx->pc2f.as<float2>(), ctx->nsim > 0 ? ctx->b_pinf.as<int>() : nullptr};
  EB_TRY(eb_fmm_apply(ctx, ctx->tree, 0, -1, prec, dens, ctx->dz.as<double2>(), ctx->hpt.as<double>(),
                      nullptr, &post, ctx->ev_join));
  return eb_check_launch(ctx, "stokes matvec");
}

int eb_laplace_matvec_dev(eb_ctx* ctx, const double* x, double* y, int prec) {
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  // the Cauchy charges q = u dz h of FASMVP_LAP (laplace.f:190-200) are formed by the
  // FMM's charge kernel from u (EbPost::u)
  EbPost post{2, nullptr, x, nullptr, ctx->dz.as<double2>(), ctx->hpt.as<double>(),
               ctx->plap.as<double>(), nullptr, nullptr, nullptr, nullptr, y, ctx->plapf.as<float>(),
               nullptr, nullptr};
  EB_TRY(eb_fmm_apply_cauchy(ctx, ctx->tree, prec, nullptr, nullptr, &post));
  return eb_check_launch(ctx, "laplace matvec");
}

// Host/device dispatch for an operator y = A x with nin, nout doubles.
template <typename F>
static int run_op(eb_ctx* ctx, const double* x, size_t nin, double* y, size_t nout, int mem, F f) {
  if (mem == EB_DEVICE) return f(x, y);
  if (mem != EB_HOST) return EB_ERR_ARG;
  cudaStream_t s = ctx->stream;
  EB_TRY(ctx->vin.ensure(sizeof(double) * nin));
  EB_TRY(ctx->vout.ensure(sizeof(double) * nout));
  EB_CUDA_TRY(cudaMemcpyAsync(ctx->vin.p, x, sizeof(double) * nin, cudaMemcpyHostToDevice, s));
  EB_TRY(f(ctx->vin.as<double>(), ctx->vout.as<double>()));
  EB_CUDA_TRY(cudaMemcpyAsync(y, ctx->vout.p, sizeof(double) * nout, cudaMemcpyDeviceToHost, s));
  EB_CUDA_TRY(cudaStreamSynchronize(s));
  return EB_OK;
}

int eb_stokes_matvec(eb_ctx* ctx, int n, const double* x, double* y, int prec, int mem) {
  if (!ctx || !x || !y) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != 2 * ctx->nbk || (prec != EB_FP64 && prec != EB_FP32)) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return run_op(ctx, x, n, y, n, mem, [&](const double* xd, double* yd) {
    return eb_stokes_matvec_dev(ctx, xd, yd, prec);
  });
}

int eb_laplace_matvec(eb_ctx* ctx, int n, const double* x, double* y, int prec, int mem) {
  if (!ctx || !x || !y) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != ctx->nbk || (prec != EB_FP64 && prec != EB_FP32)) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return run_op(ctx, x, n, y, n, mem, [&](const double* xd, double* yd) {
    return eb_laplace_matvec_dev(ctx, xd, yd, prec);
  });
}

int eb_laplace_constraints(eb_ctx* ctx, int n, const double* x, double* sums, int mem) {
  if (!ctx || !x || !sums) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != ctx->nbk) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return run_op(ctx, x, n, sums, ctx->k, mem, [&](const double* xd, double* yd) {
    k_lap_constraints<<<ctx->k, 256, 0, ctx->stream>>>(ctx->start.as<int>(), xd, ctx->dsda.as<double>(), yd);
    eb_count_launch(ctx);
    return eb_check_launch(ctx, "laplace constraints");
  });
}

int eb_stokes_sum(eb_ctx* ctx, int n, const double* dens, int sign, double* gradw, int prec,
                  int mem) {
  if (!ctx || !dens || !gradw || (sign != 1 && sign != -1)) return EB_ERR_ARG;
  if (!ctx->geom_valid) return EB_ERR_NOGEOM;
  if (n != ctx->nbk || (prec != EB_FP64 && prec != EB_FP32)) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  return run_op(ctx, dens, 2 * (size_t)n, gradw, 2 * (size_t)n, mem, [&](const double* xd, double* yd) {
    return eb_stokes_sum_dev(ctx, reinterpret_cast<const double2*>(xd), sign,
                             reinterpret_cast<double2*>(yd), prec);
  });
}

int eb_cauchy_sum(eb_ctx* ctx, int n, const double* z, const double* q, double* field, int prec,
                  int mem) {
  if (!ctx || !z || !q || !field || n <= 0) return EB_ERR_ARG;
  if (prec != EB_FP64 && prec != EB_FP32) return EB_ERR_ARG;
  if (mem != EB_HOST && mem != EB_DEVICE) return EB_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const double2* zd = reinterpret_cast<const double2*>(z);
  const double2* qd = reinterpret_cast<const double2*>(q);
  double2* fd = reinterpret_cast<double2*>(field);
  if (mem == EB_HOST) {
    EB_TRY(copy_in(ctx, ctx->pvz, z, sizeof(double2) * n, mem));
    EB_TRY(copy_in(ctx, ctx->pvq, q, sizeof(double2) * n, mem));
    EB_TRY(ctx->pvout.ensure(sizeof(double2) * n));
    zd = ctx->pvz.as<double2>();
    qd = ctx->pvq.as<double2>();
    fd = ctx->pvout.as<double2>();
  }
  EB_TRY(eb_tree_build(ctx, ctx->tree_tmp, zd, n, ctx->opts.leaf64, ctx->opts.leaf_cap));
  EB_TRY(eb_fmm_apply_cauchy(ctx, ctx->tree_tmp, prec, qd, fd));
  if (mem == EB_HOST) {
    EB_CUDA_TRY(cudaMemcpyAsync(field, fd, sizeof(double2) * n, cudaMemcpyDeviceToHost, s));
    EB_CUDA_TRY(cudaStreamSynchronize(s));
  }
  return EB_OK;
}

// ---------------------------------------------------------------------------------
// gfortran shims: MATVEC(N, XX, YY, NELT, IA, JA, A, ISYM) as DPIGMR calls it.
// ---------------------------------------------------------------------------------
static eb_ctx* g_default_ctx = nullptr;

int eb_set_default_ctx(eb_ctx* ctx) {
  g_default_ctx = ctx;
  return EB_OK;
}

static void shim_fail(const char* who, int st) {
  fprintf(stderr, "%s: %s: %s\n", who, eb_status_string(st), eb_last_error());
  abort();
}

void matvec_(const int* n, const double* xx, double* yy, const int* nelt, const int* ia,
             const int* ja, const double* a, const int* isym) {
  (void)nelt; (void)ia; (void)ja; (void)a; (void)isym;
  if (!g_default_ctx) shim_fail("matvec_", EB_ERR_NOGEOM);
  int st = eb_stokes_matvec(g_default_ctx, *n, xx, yy, EB_FP64, EB_HOST);
  if (st != EB_OK) shim_fail("matvec_", st);
}

void matvec_lapl_(const int* n, const double* xx, double* yy, const int* nelt, const int* ia,
                  const int* ja, const double* a, const int* isym) {
  (void)nelt; (void)ia; (void)ja; (void)a; (void)isym;
  if (!g_default_ctx) shim_fail("matvec_lapl_", EB_ERR_NOGEOM);
  int st = eb_laplace_matvec(g_default_ctx, *n, xx, yy, EB_FP64, EB_HOST);
  if (st != EB_OK) shim_fail("matvec_lapl_", st);
}
