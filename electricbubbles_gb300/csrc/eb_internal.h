// Internal declarations shared by the translation units of libeb_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "eb_common.cuh"

// Deepest level of the point keys (2*EB_KEY_LEVELS bits of Morton code).
#define EB_KEY_LEVELS 20
#define EB_MAX_P 60
#define EB_VMAX 27
#define EB_UMAX 9
// M2L offset codes (dx + 3) + 7 (dy + 3) of the offset d = (c_t - c_s)/r in box units:
// dx, dy in [-3, 3] for the V lists, and dy up to 7 for the reflected boxes of a wall
// (a source box mirrored across the wall y = 0, at level 2 anywhere in the 4 x 4 grid)
#define EB_NCODE 77
#define EB_GROUP 8
#define EB_NTILE 32
// Internal precision value (beside EB_FP64 and EB_FP32): FP64-class arithmetic in
// double-float on the FP32 pipes whatever eb_opts.df64 says. The refined solver's FP64
// residuals use it when eb_opts.resid_df is on.
#define EB_PREC_DF 2

// ---------------------------------------------------------------------------------
// Device buffer that grows on demand (never shrinks) and frees itself. Every
// reallocation or release advances a process-wide epoch, which invalidates the cached
// CUDA graphs that captured the old addresses. While a stream capture is in progress
// on the calling thread, a buffer that must grow keeps its old allocation alive (freed
// by eb_devbuf_collect) instead of freeing it, since cudaFree synchronises the device.
// ---------------------------------------------------------------------------------
unsigned long long eb_devbuf_epoch();
void eb_devbuf_set_capturing(bool on);
void eb_devbuf_collect();

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t nbytes);
  void release();
  ~DevBuf() { release(); }
  template <typename X> X* as() const { return reinterpret_cast<X*>(p); }
};

// Page-locked host staging for the tree build's small device-to-host reads (so that one
// stream synchronisation covers several of them).
struct EbTreeHost {
  double sq[4];            // the bounding square: W, x0, y0, 2^20 / W
  int bad;                 // 1: a non-finite coordinate; 2: a node below the wall
  int lmax;                // deepest leaf level
  int lmin;                // the uniform floor level (no leaf above it)
  int hist[EB_KEY_LEVELS + 1];  // boxes per level (heads of existing boxes)
  int last[12];            // counts and scans of the last leaf or box (work items, lists)
  unsigned long long pairs[3];  // near-field, V-list and W-list (M2P) pair counts
};

// Adaptive quadtree over a point set, built on the GPU. Every box above a minimum level
// is split (for one problem the shallowest level of mean occupancy at most the leaf
// target; for a forest the level of its cells), and below it a box is split while it
// holds more than `cap` points (DAASSI's rule, dapif1.f:1165-1255, with NAPB = cap);
// only boxes whose parent is split exist, so leaves lie on any level up to L. Boxes of level
// l are stored in Morton order in the global box range [lev_off[l], lev_off[l+1]);
// every box owns a contiguous range of the sorted points, and the leaves, in point
// order, partition them.
struct EbTree {
  int n = 0;
  int L = 0;                 // deepest leaf level
  int cap = 32;              // points per leaf at most (unless at the deepest key level)
  int R = 0;                 // a forest of independent problems: the boxes of level R hold
                             // one problem each and no interaction list crosses them
  int nbox = 0;
  int nleaf = 0;
  int lend = 2;              // FP32 far field: levels <= lend hold L2L-accumulated locals
  int lev_off[EB_KEY_LEVELS + 2] = {0};
  double x0 = 0, y0 = 0, W = 1;  // root square [x0, x0+W] x [y0, y0+W]
  long long v_pairs = 0, u_pairs = 0, w_pairs = 0;  // read from host->pairs when first asked for
  long long nu = 0, nw = 0;  // lengths of the U and W lists
  bool pairs_read = false;
  bool valid = false;
  // a problem small enough for the direct sums (eb_opts.direct_max; one problem, no
  // wall): the points in their given order (perm, zs, zhl) and no boxes or lists
  bool direct = false;
  EbTreeHost* host = nullptr;  // page-locked (cudaMallocHost), freed with the tree
  ~EbTree();

  DevBuf perm;     // int[n]: sorted index -> original index
  DevBuf zs;       // double2[n]: sorted positions
  DevBuf zhl;      // float4[n]: sorted positions as float hi + lo, (hi.x, hi.y, lo.x, lo.y)
  DevBuf plev;     // unsigned char[n]: level of the leaf holding each sorted point
  DevBuf wdf;      // float4[n]: offset from the leaf centre in leaf units, (x.hi, y.hi, x.mid, y.mid)
  DevBuf wdf_lo;   // float2[n]: (x.lo, y.lo) of the same offset
  DevBuf keys, keys_alt, idx_alt;  // sort buffers
  DevBuf lcpw;     // unsigned char[n]: levels shared by the keys of points w and w + cap
  DevBuf bkey;     // unsigned long long[nbox]: Morton key of the box at its level
  DevBuf blev;     // unsigned char[nbox]: level of the box
  DevBuf pt0, pt1; // int[nbox]: point range
  DevBuf parent;   // int[nbox]
  DevBuf child0, nchild;  // int[nbox] (nchild = 0: a leaf)
  DevBuf vlist;    // int[nbox*EB_VMAX]
  DevBuf vcode;    // unsigned char[nbox*EB_VMAX]
  DevBuf vcount;   // int[nbox]
  DevBuf leaves;   // int[nleaf]: box of each leaf, in point order
  DevBuf lflag, lscan;   // int[n]: leaf heads among the points and their scan
  // U lists (leaves adjacent to the leaf, on any level: evaluated directly) and W lists
  // (boxes below an adjacent box of the leaf's level that are not adjacent to the leaf
  // but whose parent is: evaluated from their multipoles), CSR per leaf
  DevBuf ucnt, ustart, ulist;
  DevBuf wcnt, wstart, wlist;
  DevBuf tcount, tstart;  // int[nleaf]: near-field tiles per leaf and their scan
  // near-field work items: groups of up to EB_GROUP targets of one leaf
  int ngroup = 0;
  DevBuf gleaf;    // int[ngroup]: leaf index
  DevBuf gfirst;   // int[ngroup]: first sorted target of the group
  // shared-memory near-field work items: tiles of up to EB_NTILE targets of one leaf,
  // a leaf's targets split evenly over its tiles
  int ntile = 0;
  DevBuf tiles;    // int4[ntile]: (leaf index, first, end, 0)
  // FP32 far field: per leaf its boxes at levels lev(leaf), .., max(2, min(lev(leaf), lend)),
  // at most EB_FAR_LEVELS of them (the coarsest one holds the accumulated locals above)
  DevBuf anc;      // int[nleaf*EB_FAR_LEVELS]
  DevBuf gcount, gstart;  // groups per leaf and their scan
  DevBuf flags, scan, hist, bbox, partial, cubtmp, pairs;
  // FP32 direct multipoles: the boxes of levels chunk_lmin..L and the leaves above them,
  // split into chunks of EB_CHUNK points (other boxes by M2M)
  int nchunk = 0;
  int chunk_lmin = 2;
  DevBuf ccount;     // int[nbox - lev_off[2]]: chunks per box of levels >= 2
  DevBuf cstart;     // int[nbox - lev_off[2] + 1]: first chunk of each box
  DevBuf chunk_box;  // int[nchunk]: the box of each chunk
  DevBuf cdone;      // int[nbox - lev_off[2]]: chunks of the box finished in the
                     // current P2M (zero between launches: the box's last chunk resets it)
  // Wall-bounded flow (the wall is y = 0, the root square's bottom edge): the reflected
  // source boxes of every box of levels 2..ld (ilist/icode/icount, stride EB_VMAX, like
  // the V lists), whose multipoles are mirrored and translated by M2L; the pairs of
  // adjacent first-row boxes of level ld are summed directly. ld is the uniform floor
  // level (no leaf above it), or 0 when the tree has no level-2 expansions.
  int wall = 0;
  int ld = 0;
  DevBuf ilist;      // int[lev_off[ld+1] * EB_VMAX] (boxes below level 2 unused)
  DevBuf icode;      // unsigned char[same]
  DevBuf icount;     // int[lev_off[ld+1]]
};
#define EB_CHUNK 64
#define EB_DIRECT_LEVELS 3  // finest levels whose FP32 multipoles come directly from points
#define EB_FAR_LEVELS 6     // finest levels whose FP32 locals are evaluated at each target
                            // directly (coarser levels reach them by L2L)
#define EB_LEAF_CAP 96      // default maximum points per leaf

// Per-precision constant tables for the translation operators.
struct EbTables {
  int p = 0;
  DevBuf binom;   // T[(2p+2)*(2p+2)] binomial coefficients C(i, j) at [i*(2p+2)+j]
  DevBuf dinv;    // c_t<T>[EB_NCODE*(p+2)]: d^-j for the offset codes
  DevBuf pd;      // int[EB_NCODE]: per-offset truncation order
  DevBuf epow;    // c_t<T>[4*(p+2)]: e_q^j for the 4 child offsets (child units)
  DevBuf einv;    // c_t<T>[4*(p+2)]: e_q^-j
  // double-float copies (FP64 tables only) for the double-float M2L
  DevBuf binom_df;  // float2[(2p+2)*(2p+2)]
  DevBuf dinv_df;   // float4[EB_NCODE*(p+2)]
  DevBuf epow_df;   // float4[4*(p+2)]
  DevBuf einv_df;   // float4[4*(p+2)]
};

struct EbFmmWork {
  DevBuf qa, qb;     // c_t<T>[n] sorted charges (P2M)
  DevBuf pq, aa;     // near-field source data (P2P)
  DevBuf pqdf, aadf; // double-float near-field source data, scaled by 1/r_leaf (float4)
  DevBuf mpole_df;   // float4[nbox*E*p]: multipoles, double-float pipeline
  DevBuf local_df;   // float4[nbox*E*(p+1)]: local expansions, double-float pipeline
  DevBuf qdf;        // float4[2n]: qa/r, qb/r as double-float (P2M)
  DevBuf nearbuf;    // double2[n]: near-field sums (sorted order) when split from the far field
  DevBuf mpole;      // c_t<T>[nbox*E*p]
  DevBuf mpart;      // c_t<T>[nchunk*E*p]: per-chunk partial multipoles (FP32 direct P2M)
  DevBuf local;      // c_t<T>[nbox*E*(p+1)]
  DevBuf mimg;       // multipoles mirrored across the wall, in the pipeline's format
};

// A GMRES cycle (or refinement step) captured as one CUDA graph: the Arnoldi steps run
// inside a conditional WHILE node whose condition a device kernel sets.
struct GmGraph {
  bool valid = false;
  unsigned long long key[8] = {0};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long n_pre = 0, n_body = 0, n_post = 0;  // kernel launches per part
  void destroy();
};
#define EB_GRAPH_CACHE 4
#define EB_GM_MAXL 126
#define EB_DEFER_SLOTS 8

struct eb_ctx {
  eb_opts opts;
  int device = 0;
  int nsm = 1;      // streaming multiprocessors of the device
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  long long launches = 0;
  bool profiling = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_near0 = nullptr, ev_near1 = nullptr;  // kernel class 2 (nested in class 0)
  long long prof_launch[3] = {0, 0, 0};
  double prof_ms[3] = {0, 0, 0};
  int last_p = 0;

  // installed geometry (COMMON /inteqn/ and /problem/)
  int k = 0, nbk = 0;
  std::vector<int> nd_host;
  std::vector<int> start_host;
  DevBuf nd, start, drop_of;     // int[k], int[k+1], int[nbk]
  DevBuf z, dz, zk, ckern;       // double2
  DevBuf dsda, kappa, tha, hpt;  // double
  DevBuf pc1, pc2, plap;         // per-node post-processing coefficients (eb_post_coefs)
  DevBuf pc1f, pc2f, plapf;      // their float copies (FP32 operator)
  DevBuf pkw;                    // double2: weights of FASMVP's singular-term sums
  bool geom_valid = false;
  bool ckern_valid = false;       // ckern/tha filled by eb_extractdat
  // wall-bounded flow (COMMON /wallinfo/, electric.f:55): the Stokes sums add the images
  // across the wall y = 0; xleft and slength are EXTRACTDAT's (electric.f:710-711),
  // taken from the installed nodes by the tree build
  int iwall = 0;
  double xleft = 0.0, slength = 0.0;

  EbTree tree;      // tree over the nodes
  EbTree tree_pv;   // tree over the 2N fine points of PVINTEV
  EbTree tree_tmp;  // tree for eb_cauchy_sum on caller points
  EbTables tab64, tab32;
  EbFmmWork work64, work32;

  // operator scratch
  DevBuf za, pk, redpart;          // per-drop reductions
  DevBuf vin, vout, vtmp, vtmp2;   // host-path staging and temporaries
  DevBuf pvz, pvq, pvout;          // PVINTEV fine grid
  DevBuf fftbuf, fftbuf2;          // spectral scratch
  DevBuf ex_zk, ex_dz, ex_ds, ex_ka, ex_area;  // EXTRACTDAT outputs before install

  // RK stage F and the RK2 step
  DevBuf st_lap;                   // double[5*nbk]: Laplace rhs/Un, density, phi, psi, dphi/dn
  DevBuf st_rhs, st_u, st_zc;      // Stokes rhs and density (double2[nbk]), C_k (double2[k])
  DevBuf adj_a, adj_b, adj_s;      // transposed operators: two node sums, per-drop sums
  DevBuf aj, aj_part, aj_rk;       // adjoint of F: cotangents, per-drop partials, RK2 step state
  DevBuf aj_df;                    // adjoint of F: double-float positions, charges and cotangents
  DevBuf aj_ck;                    // eb_rk2_gradient: the checkpointed states and the cotangent
  DevBuf rk_y, rk_y1, rk_d0, rk_phi;  // RK state, predictor, derivative, dt * F(y)

  // GMRES workspace
  DevBuf gV, gW, gH, gPart, gX, gR, gD, gZ, gTicket;
  DevBuf gCtl, gXin, gWbuf;        // graph mode: control block, operator input and output
  DevBuf gDefl, gDeflC;            // deflated Laplace solve: M^-1 of the operator's input, coefficients
  std::vector<double> hH;
  unsigned long long geom_version = 0;  // advanced by every geometry install
  // hash of everything a captured solve graph takes from the geometry by value (counts,
  // level offsets, work-item counts, the root square): graphs are reused across installs
  // with the same hash (the device data they read is reloaded by every launch)
  unsigned long long geom_shape = 0;
  cudaStream_t cap_stream = nullptr;    // private stream for graph capture
  cudaStream_t side_stream = nullptr;   // second stream for work that overlaps the FMM
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_c = nullptr, ev_p2p = nullptr;  // FMM: near field forked after the charges
  GmGraph gcache[EB_GRAPH_CACHE];
  int gcache_next = 0;

  // a batch of independent simulations (eb_batch_define; nsim = 0: one problem)
  int nsim = 0;
  std::vector<int> sim_k;          // drops per simulation
  std::vector<double> sim_e0;      // E0 per simulation
  bool sim_has_e0 = false;
  std::vector<int> sim_node0;      // first node of each simulation (nsim + 1)
  DevBuf b_sim_of_drop, b_pinf, b_e0, b_alpha, b_seg1, b_seg2, b_sim_of_node, b_box, b_shift;
  DevBuf zt;                       // nodes moved into their simulation's cell of the forest
  int b_R = 0;                     // the forest's cells are the boxes of level b_R
  double b_sq[3] = {1, 0, 0};      // the forest's root square (W, x0, y0)
  DevBuf b_G, b_CS, b_ctl, b_misc; // batched GMRES state
  // inner FP32 Arnoldi steps over chunks of rows: work items (sim, row0, row1, 0) of the
  // Laplace (1) and Stokes (2) segments, per simulation its first item and count, the
  // partial sums per item, h and the norm per simulation, and per-simulation tickets
  DevBuf b_items1, b_items2, b_sitem1, b_sitem2, b_part, b_hbuf, b_tick;
  int b_nitem1 = 0, b_nitem2 = 0;
  DevBuf b_st1, b_st2, b_flag;     // GETFOURIER / DOUBLE: drop starts and flags
  int* b_host_act = nullptr;       // page-locked counters read back per cycle
  double* h_flux = nullptr;        // page-locked: an RK stage's FLUX, read after the step's synchronisation
  // Deferred waits inside an RK call in plain mode (eb_rk2_step, eb_rk_f): the GMRES graph
  // solves queue their control blocks to page-locked slots and the installs of direct
  // trees their finiteness flags to d_bad; the call reads both after its one
  // synchronisation (eb_defer_info)
  bool defer = false;
  int ndefer = 0;                  // slots used by this call
  unsigned char* h_defer = nullptr; // page-locked: EB_DEFER_SLOTS control-block heads
  unsigned char* h_spec = nullptr;  // page-locked: the heads of refinement steps 1 and 2 (one wait)
  long long defer_body[8] = {0};    // kernel launches per Arnoldi step of each slot's graph
  DevBuf d_bad;                    // int: a direct tree's non-finite node (deferred)
  int* h_bad = nullptr;            // page-locked copy of d_bad
  GmGraph bgraph[2];               // batched GMRES cycles as graphs (plain, refinement inner)
};

typedef int (*eb_op_fn)(eb_ctx*, const double*, double*, int);

// Enqueues `f` on the capture stream into graph `gr` after `deps`; records the sink
// nodes of the capture and the kernel launches it issued.
template <typename F>
inline int eb_capture_into(eb_ctx* ctx, cudaGraph_t gr, const cudaGraphNode_t* deps, size_t ndeps,
                 std::vector<cudaGraphNode_t>* sinks, long long* nlaunch, bool* graph_lost, F f) {
  cudaStream_t saved = ctx->stream;
  const long long l0 = ctx->launches;
  ctx->stream = ctx->cap_stream;
  eb_devbuf_set_capturing(true);
  int st = EB_OK;
  cudaError_t e = cudaStreamBeginCaptureToGraph(ctx->cap_stream, gr, deps, nullptr, ndeps,
                                                cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    eb_set_last_cuda_error(e, "cudaStreamBeginCaptureToGraph", __FILE__, __LINE__);
    st = EB_ERR_CUDA;
  } else {
    st = f();
    if (sinks) {
      cudaStreamCaptureStatus cs;
      const cudaGraphNode_t* d = nullptr;
      size_t nd = 0;
      e = cudaStreamGetCaptureInfo(ctx->cap_stream, &cs, nullptr, nullptr, &d, nullptr, &nd);
      if (e == cudaSuccess && d) sinks->assign(d, d + nd);
      else if (st == EB_OK) {
        eb_set_last_cuda_error(e, "cudaStreamGetCaptureInfo", __FILE__, __LINE__);
        st = EB_ERR_CUDA;
      }
    }
    cudaGraph_t out = nullptr;
    e = cudaStreamEndCapture(ctx->cap_stream, &out);
    if (e != cudaSuccess || out == nullptr) {
      // an invalidated capture: the graph is not ours to destroy any more
      if (graph_lost) *graph_lost = true;
      if (st == EB_OK) {
        eb_set_last_cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        st = EB_ERR_CUDA;
      }
    }
  }
  eb_devbuf_set_capturing(false);
  ctx->stream = saved;
  *nlaunch = ctx->launches - l0;
  ctx->launches = l0;
  return st;
}


// batch.cu
int eb_batch_install(eb_ctx* ctx);
int eb_batch_translate_fine(eb_ctx* ctx, double2* zf);
// solve.cu: the info of deferred plain solve `slot` (after the caller's synchronisation)
int eb_defer_info(eb_ctx* ctx, int slot, eb_solve_info* inf);
// One RK stage F (eb_spectral.cu) with synchronous solves; gout (device, optional)
// receives INTERFACENEW's full velocity sum g (Un = Re(-i g conj(zn))). ul_in / u_in
// (device, optional) stand in for the Laplace / Stokes solve with kept solutions; ul_out /
// u_out receive the solutions.
int eb_stage_f_keep(eb_ctx* ctx, int k, const int* nd, const double* rku, double* rkup, const eb_model* m,
                    eb_stage_info* info, double2* gout, const double* ul_in = nullptr,
                    const double* u_in = nullptr, double* ul_out = nullptr, double* u_out = nullptr);
// PVINTEV's fine points and charges of the Laplace density ul (charges of ul dz, as
// DIRICH_NEU_MAP forms them) into ctx->pvz / ctx->pvq, interleaved even/odd fine nodes.
int eb_pv_fine(eb_ctx* ctx, const double* ul);
int eb_batch_solve(eb_ctx* ctx, int n, eb_op_fn op, bool stokes, const double* rhs, double* soln, int mode,
                   eb_solve_info* info, int mem);

// Precision of the refined solver's FP64 residual applies (and of the refined RK stage's
// other FP64 sums): double-float when eb_opts.resid_df is on, else EB_FP64.
inline int eb_resid_prec(const eb_ctx* ctx) { return ctx->opts.resid_df > 0 ? EB_PREC_DF : EB_FP64; }

// tree.cu
// root_sq (W, x0, y0) and root_level: an explicit root square whose boxes of level
// root_level each hold one independent problem (null: the bounding square, one problem)
// wall != 0: the root square is [xmin, xmin + S] x [0, S], S = max(xmax - xmin, ymax)
// (EXTRACTDAT's xleft and slength, electric.f:710-711), its bottom edge the wall y = 0,
// and the tree gets the image lists of the wall (EbTree::ilist); a node below the wall
// is an error.
int eb_tree_build(eb_ctx* ctx, EbTree& t, const double2* z_dev, int n, int leaf_target, int leaf_cap,
                  const double* root_sq = nullptr, int root_level = 0, int wall = 0);
// The tree's pair counts (u_pairs, v_pairs), waiting for the build if it is in flight.
int eb_tree_pairs(eb_ctx* ctx, EbTree& t);

// fmm.cu
struct EbPost;
int eb_tables_init(eb_ctx* ctx);
// kernel: 0 = Stokes (sign from `sign`). `post` (may be null: store the sum into out)
// fuses an operator's post-processing into the leaf kernels.
// `join` (may be null): an event the leaf kernel waits for (work the caller forked onto
// another stream whose results the post-processing reads).
// The Stokes sum of FASMVP's charges qa = dens dz h/(2 pi i), qb = (dens conj(dz) -
// conj(dens) dz) h/(2 pi i); dz = null: the charges qa = -dens, qb = conj(dens) of the
// transposed operator's sums (never with a wall's images).
int eb_fmm_apply(eb_ctx* ctx, EbTree& t, int kernel, int sign, int precision,
                 const double2* dens, const double2* dz, const double* hpt, double2* out,
                 const EbPost* post = nullptr, cudaEvent_t join = nullptr);
int eb_fmm_apply_cauchy(eb_ctx* ctx, EbTree& t, int precision, const double2* q,
                        double2* out, const EbPost* post = nullptr);

// api.cu: operators on device vectors (x, y device pointers)
int eb_stokes_sum_dev(eb_ctx* ctx, const double2* dens, int sign, double2* gradw, int prec);
int eb_stokes_matvec_dev(eb_ctx* ctx, const double* x, double* y, int prec);
int eb_laplace_matvec_dev(eb_ctx* ctx, const double* x, double* y, int prec);
// adjoint.cu: the transposed operators
int eb_stokes_matvec_adj_dev(eb_ctx* ctx, const double* x, double* y, int prec);
int eb_laplace_matvec_adj_dev(eb_ctx* ctx, const double* x, double* y, int prec);

// m2l_tc.cu: the FP32 M2L of order 20 on the tensor cores
int eb_m2l_tc(eb_ctx* ctx, int E, int first, int ntarget, const int* vlist, const unsigned char* vcode,
              const int* vcount, const float* binom, int ldb, const float2* dinv, const int* pd,
              const float2* mpole, float2* local, cudaStream_t st);

// api.cu: (re)build the installed geometry's tree with the current eb_opts
int eb_geom_tree(eb_ctx* ctx);

// api.cu helpers
cudaStream_t eb_stream(eb_ctx* ctx);
inline void eb_count_launch(eb_ctx* ctx) { ctx->launches++; }
int eb_check_launch(eb_ctx* ctx, const char* name);
