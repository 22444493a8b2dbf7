/*
 * eb_gb300.h - C ABI of the GB300-native ElectricBubbles hot path.
 *
 * The reference (mcetal/ElectricBubbles, Fortran 77) applies its boundary-integral
 * operators through GMRES callbacks with the SLATEC signature
 *     MATVEC(N, X, Y, NELT, IA, JA, A, ISYM)
 * and passes the geometry through COMMON blocks. This library replaces that
 * operator apply (and the solves, spectral derivatives and principal-value
 * integrals around it) with CUDA kernels on one GPU. Plain C types only: pointers
 * and sizes, no CUDA or PyTorch types in any signature.
 *
 * Conventions
 *  - Complex arrays are interleaved (re, im) doubles, i.e. Fortran COMPLEX*16.
 *  - Nodes of k drops are concatenated in drop order (nd[0] nodes of drop 0, ...).
 *  - `mem` says whether the array arguments are host (EB_HOST) or device
 *    (EB_DEVICE, allocated on the context's GPU) pointers. Host calls copy in,
 *    compute, copy out, and return when the result is in host memory. Device calls
 *    return once their work is enqueued on the context's stream (waiting on the host
 *    only where sizes or loop decisions need it: tree builds, GMRES steps); a device
 *    result is ready in that stream's order (eb_ctx_sync waits for it). The RK calls
 *    (eb_rk_f, eb_rk2_step) return with their stage info, so after the stream's work.
 *  - Every function returns an eb_status; the library never calls exit().
 *    eb_last_error() describes the last failure of the calling thread.
 */
#ifndef EB_GB300_H
#define EB_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define EB_GB300_VERSION 6

/* Status codes. The reference prints and STOPs on FMM/GMRES errors
 * (stokesbubb.f:573-579, laplace.f:217-222, 395-398, pv_integral.f:183-188);
 * here every condition is returned to the caller. */
enum eb_status {
  EB_OK = 0,
  EB_ERR_ARG = 1,          /* invalid argument (size mismatch, null pointer, ...) */
  EB_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  EB_ERR_NOGEOM = 3,       /* no geometry installed in the context */
  EB_ERR_WORKSPACE = 4,    /* a size exceeds a fixed capacity */
  EB_ERR_TOL = 5,          /* requested tolerance needs more expansion terms than supported */
  EB_ERR_NAN = 6,          /* non-finite value detected in an input or a residual */
  EB_ERR_NOT_CONVERGED = 7,/* GMRES did not reach the tolerance (DGMRES IERR = 1 or 2) */
  EB_ERR_NODEVICE = 8,     /* no CUDA device available */
  EB_ERR_TIMEOUT = 9       /* a bounded device-side wait gave up */
};

enum eb_memspace { EB_HOST = 0, EB_DEVICE = 1 };

/* Arithmetic of a layer-potential sum: plain FP64, or FP32 expansions and near
 * field (compensated) for the inner operator of the refined solver. */
enum eb_precision { EB_FP64 = 0, EB_FP32 = 1 };

/* Solver mode: plain FP64 GMRES, or FP32-inner GMRES with FP64 iterative
 * refinement (outer residual, Arnoldi and least squares in FP64). */
enum eb_solve_mode { EB_SOLVE_FP64 = 0, EB_SOLVE_FP32_REFINED = 1 };

typedef struct eb_opts {
  int p64;          /* FP64 expansion order (0: default 44)                    */
  int p32;          /* FP32 expansion order (0: default 20)                    */
  int leaf64;       /* tree: mean points per leaf of its uniform floor (0: 32)  */
  int leaf_cap;     /* tree: maximum points per leaf below the floor (0: 96)   */
  double tol64;     /* M2L per-offset truncation tolerance, FP64 (0: 1e-15)    */
  double tol32;     /* M2L per-offset truncation tolerance, FP32 (0: 1e-7)     */
  int maxl;         /* GMRES Krylov dimension, MAXL (0: 100, electric.f:1011)  */
  double gmres_tol; /* GMRES relative residual tolerance (0: 1e-10)            */
  double inner_tol; /* refined mode: inner FP32 GMRES relative tolerance of the first
                     * refinement step (0: 1e-5); later steps tighten it, to at most a
                     * tenth, when that is expected to end the solve */
  int max_outer;    /* refined mode: maximum refinement steps (0: 8)           */
  int device;       /* CUDA device ordinal                                     */
  int graphs;       /* GMRES as CUDA graphs with a device-side Arnoldi loop:
                       0 default (on), 1 on, -1 off (host-driven loop)          */
  int df64;         /* plain FP64 operators in double-float arithmetic on the FP32
                       pipes (FP64-class, <= 4e-13 from FP64 direct sums):
                       0 default (off: native FP64 throughout), 1 on, -1 off    */
  int resid_df;     /* refined mode: the FP64 residual of every refinement step (and
                       the refined RK stage's PV and velocity sums) in double-float
                       arithmetic: 0 default (on), 1 on, -1 off (native FP64)   */
  int m2l_tc;       /* FP32 M2L (order 20) as a 3xTF32 contraction on the tensor
                       cores (tcgen05): 0 default (off), 1 on, -1 off          */
  int lap_deflate;  /* Laplace solves: GMRES right-preconditioned by the deflation of
                       each drop's constant density, an eigenvector of FASMVP_LAP with
                       eigenvalue -2 h mean(s'); same stopping test on ||b - A x||, far
                       fewer iterations with many drops. 0 default (off: DGMRES as the
                       reference runs it), 1 on, -1 off. Not applied to a batch of
                       simulations or to the adjoint solve. */
  int direct_max;   /* layer sums over at most this many points (one problem, no wall)
                       are direct O(N^2) sums in one kernel instead of the FMM: exact up
                       to rounding, and faster on few points (0: default 1024; -1: the
                       FMM always) */
  int adj_df;       /* reverse mode (eb_rk_f_vjp): the O(nbk^2) derivative sums in
                       double-float arithmetic on the FP32 pipes (about 48 bits; the
                       positions relative to the first node): 0 default (on), 1 on,
                       -1 off (native FP64) */
} eb_opts;

typedef struct eb_solve_info {
  int iters;        /* total Krylov iterations (inner iterations in refined mode) */
  int outer;        /* refinement steps (1 in plain mode)                     */
  int matvecs64;    /* FP64 operator applies                                  */
  int matvecs32;    /* FP32 operator applies                                  */
  double err;       /* final ||b - A x|| / ||b|| estimate (DGMRES ERR)        */
  int ierr;         /* DGMRES IERR convention: 0 converged, 1 MAXL reached, 2 stalled */
  int graph;        /* 1 if the solve ran as CUDA graphs with the device-side loop */
} eb_solve_info;

typedef struct eb_tree_info {
  int npoints;      /* points in the tree                                     */
  int levels;       /* deepest leaf level (root is level 0)                   */
  int nboxes;       /* boxes over all levels                                  */
  int nleaves;      /* leaves (on any level)                                  */
  long long v_pairs;/* M2L (source box, target box) pairs                     */
  long long u_pairs;/* near-field (target point, source point) pairs          */
  int p;            /* expansion order of the last apply                      */
  long long w_pairs;/* M2P (W-list box, target point) evaluations             */
} eb_tree_info;

/* Physical parameters of the RK right-hand side F (electric.f:968-1109), the values the
 * reference keeps in COMMON: cap (strain rate of the far field psi = -i cap z / 2,
 * stokesbubb.f:64-68), e0 (electric field strength, the E0 of the electric stress,
 * stokesbubb.f:110-128) and zbond (complex Bond number). zbond != 0 is the wall-bounded
 * flow of the reference (READINI sets iwall = 1, electric.f:321-326): the drops lie above
 * the wall y = 0, every Stokes sum adds the images across it, and SETVELF / INTERFACENEW
 * add the reflected log sources zc = i zbond area / (8 pi) (REFSING, reflect.f:28-86);
 * eb_rk_f and eb_rk2_step then set the context's wall mode as eb_set_wall does (and clear
 * it for zbond = 0). mode selects the solver of both GMRES solves. */
typedef struct eb_model {
  double cap;
  double e0;
  double zbond[2];
  int mode;         /* eb_solve_mode */
} eb_model;

/* Diagnostics of eb_rk_f / eb_rk2_step (summed over the stages of a step). */
typedef struct eb_stage_info {
  int lap_iters;    /* Krylov iterations of the Laplace solves (SOLVE_LAPL)   */
  int stokes_iters; /* Krylov iterations of the Stokes solves (SOLVEI)        */
  double lap_err;   /* last Laplace relative residual                         */
  double stokes_err;/* last Stokes relative residual                          */
  double flux;      /* FLUX of the last stage (electric.f:848-882)            */
  int lap_ierr;     /* DGMRES IERR of the last Laplace solve                  */
  int stokes_ierr;  /* DGMRES IERR of the last Stokes solve                   */
} eb_stage_info;

typedef struct eb_ctx eb_ctx;

int eb_version(void);
const char* eb_status_string(int status);
const char* eb_last_error(void);
void eb_opts_default(eb_opts* opts);

int eb_ctx_create(eb_ctx** out, const eb_opts* opts);
int eb_ctx_destroy(eb_ctx* ctx);
/* Run the context's work on an existing CUDA stream (a cudaStream_t passed as void*);
 * NULL restores the context's own stream. */
int eb_ctx_set_stream(eb_ctx* ctx, void* cuda_stream);
int eb_ctx_sync(eb_ctx* ctx);
/* Kernel launches issued by this context so far. */
long long eb_ctx_launch_count(eb_ctx* ctx);
/* When enabled, the dominant leaf and M2L kernels are bracketed by CUDA events on
 * the context's stream (and the near field runs on it, not concurrently);
 * eb_ctx_kernel_time reports launches and total milliseconds per kernel class
 * (0: the kernel that ends an apply: far-field L2P and post-processing, for the
 * FP64-class operators also the near field; 1: M2L; 2: the FP32 near-field kernel). */
int eb_ctx_set_profiling(eb_ctx* ctx, int enable);
int eb_ctx_kernel_time(eb_ctx* ctx, int kernel_class, long long* launches, double* total_ms);
int eb_ctx_tree_info(eb_ctx* ctx, eb_tree_info* info);
/* Autotuner of the tree's leaf sizes for the installed geometry; no counterpart in the
 * reference (its leaf rule is fixed: LEVMAX = 7 in CADAPDR, NAPB = 30 in DAPIF2). Each
 * candidate (eb_opts.leaf64, eb_opts.leaf_cap) is installed and the FP32 Stokes operator,
 * the refined solver's inner operator, is timed on the GPU; the fastest is kept in the
 * context's options (and used by later installs) and reported in info. */
#define EB_TUNE_MAX 8
typedef struct eb_tune_info {
  int leaf64, leaf_cap;           /* the chosen leaf sizes                         */
  int ncand;                      /* candidates timed                              */
  int leaf_target[EB_TUNE_MAX];   /* candidate i: eb_opts.leaf64                   */
  int leaf_cap_cand[EB_TUNE_MAX]; /* candidate i: eb_opts.leaf_cap                 */
  double apply_us[EB_TUNE_MAX];   /* candidate i: microseconds per FP32 apply      */
} eb_tune_info;
int eb_autotune(eb_ctx* ctx, eb_tune_info* info);

/* FP64 FMA throughput of the context's GPU in TFLOP/s (a short calibration kernel):
 * the roofline denominator of the FP64 FMM kernels. No counterpart in the reference. */
int eb_measure_fp64_peak(eb_ctx* ctx, double* tflops);
/* FP32 FMA throughput in TFLOP/s: the denominator of the FP32 and double-float kernels. */
int eb_measure_fp32_peak(eb_ctx* ctx, double* tflops);

/* Install the geometry of k drops: the data EXTRACTDAT (electric.f:636-716) leaves
 * in COMMON /inteqn/ dsdth, rkappa, z, dz and /problem/ zk, nd, k, nbk
 * (electric.f:1022-1023). z, dz, zk are complex; dsda, kappa real. Builds the
 * quadtree and interaction lists once; they stay valid until the next call. */
int eb_set_geometry(eb_ctx* ctx, int k, const int* nd, const double* z, const double* dz,
                    const double* dsda, const double* kappa, const double* zk, int mem);

/* EXTRACTDAT (electric.f:636-716) on the GPU: from the RK state rku (interleaved
 * x, y of all nodes) compute z, zk, dz, dsda, kappa, ckern, tha and the drop areas,
 * and install the geometry. Outputs may be NULL. zbond enters only zc. */
int eb_extractdat(eb_ctx* ctx, int k, const int* nd, const double* rku, double* zk,
                  double* dz, double* dsda, double* kappa, double* ckern, double* tha,
                  double* area, int mem);

/* Stokes operator FASMVP (stokesbubb.f:496-614), the body of MATVEC
 * (stokesbubb.f:419-465): x, y interleaved real vectors of length n = 2 nbk. */
int eb_stokes_matvec(eb_ctx* ctx, int n, const double* x, double* y, int precision, int mem);

/* Laplace operator FASMVP_LAP (laplace.f:159-262), the body of MATVEC_LAPL
 * (laplace.f:429-465): x, y of length n = nbk. The reference additionally writes k
 * constraint sums past y(n) (laplace.f:252-259); eb_laplace_constraints returns them. */
int eb_laplace_matvec(eb_ctx* ctx, int n, const double* x, double* y, int precision, int mem);
int eb_laplace_constraints(eb_ctx* ctx, int n, const double* x, double* sums, int mem);

/* The sum CADAPDR (sign = -1, cadapdrop.f:3-387, used by FASMVP) or CADAPMOD
 * (sign = +1, cadapmod.f:3-386, used by INTERFACENEW) evaluates at the installed
 * nodes, self excluded: dens complex density (n = nbk complex values), gradw out. */
int eb_stokes_sum(eb_ctx* ctx, int n, const double* dens, int sign, double* gradw,
                  int precision, int mem);

/* For callers that cannot allocate GPU memory; no counterpart in the reference.
 * Hosts that own every device buffer themselves, code running inside an allocator or
 * memory-pool callback, and loops that forbid allocation after start-up cannot use the
 * context-based entry points, which draw working memory from cudaMalloc. This one needs
 * no eb_ctx and allocates nothing: it evaluates the sum of eb_stokes_sum (CADAPDR for
 * sign = -1, CADAPMOD for sign = +1, self excluded) by direct FP64 summation for
 * n <= EB_NOALLOC_MAX_POINTS nodes, larger n returns EB_ERR_WORKSPACE. All arrays are
 * device pointers: z, dz, dens, gradw complex (n values, 16-byte aligned), h real (the
 * per-node weight 2 pi / nd of the node's drop, 8-byte aligned); misaligned pointers
 * return EB_ERR_ARG. Its scratch is a fixed 768 KiB array in the library's device
 * memory, held by every GPU that loads the library until exit and shared by all calls:
 * calls that overlap on the GPU race, so order them on one stream. The first call on
 * each device looks up that array's address, which under CUDA's lazy module loading
 * also loads the library's device code (and so reserves device memory): make it at
 * start-up, outside allocator callbacks and before any stream capture. The address
 * belongs to the device's primary context, the one the CUDA runtime uses; callers with
 * their own driver-API contexts, or that reset the device, cannot use this entry point.
 * The work is enqueued on `stream` (a cudaStream_t, NULL = default stream); the result
 * is ready when the stream reaches it. */
#define EB_NOALLOC_MAX_POINTS 16384
int eb_stokes_sum_noalloc(int n, const double* z, const double* dz, const double* h,
                          const double* dens, int sign, double* gradw, void* stream);

/* The Cauchy sum DAPIF2 returns for IFLAG7 = 3 (dapif1.f:458-1077):
 * field_i = sum_{j != i} q_j / (z_i - z_j), on n arbitrary points (own tree). */
int eb_cauchy_sum(eb_ctx* ctx, int n, const double* z, const double* q, double* field,
                  int precision, int mem);

/* GMRES solves with the settings of SOLVEI (stokesbubb.f:294-415) and SOLVE_LAPL
 * (laplace.f:335-425): x0 = rhs, MAXL Krylov vectors, no restart, stop when
 * ||b - A x|| / ||b|| <= gmres_tol (DGMRES ITOL = 0). soln receives the solution.
 * With eb_opts.lap_deflate on, eb_laplace_solve runs the same GMRES on A M^-1 t = b,
 * x = M^-1 t, with M^-1 = I + sum_k (1/mu_k - 1) P_k (P_k: the mean over drop k spread
 * over its nodes, mu_k = -2 h_k mean_k(s')); t0 = M rhs, so x0 = rhs still. */
int eb_stokes_solve(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                    eb_solve_info* info, int mem);
int eb_laplace_solve(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                     eb_solve_info* info, int mem);

/* FDIFFF (dcfft.f:1371-1428) per drop on the installed drop sizes: complex f -> df. */
int eb_fdiff(eb_ctx* ctx, const double* f, double* df, int mem);

/* PVINTEV (pv_integral.f:53-204) on the installed geometry: ucmplx -> phicmplx. */
int eb_pvintev(eb_ctx* ctx, const double* ucmplx, double* phicmplx, int precision, int mem);

/* DIRICH_NEU_MAP (laplace.f:266-331): Laplace density u -> phi, psi, dphi_dn. */
int eb_dirich_neu_map(eb_ctx* ctx, const double* u, double* phi, double* psi,
                      double* dphi_dn, int precision, int mem);

/* INTERFACENEW (electric.f:791-912): Stokes density u (complex, nbk) -> interface normal
 * velocity un and the FLUX diagnostic. zc: per-drop C_k (complex). In wall mode
 * (eb_set_wall) the Stokes sum adds its images and the far field the reflected log
 * sources of REFSING (electric.f:868-872). */
int eb_interface_velocity(eb_ctx* ctx, const double* u, const double* zc, double cap,
                          double* un, double* flux, int precision, int mem);

/* SETVELF (stokesbubb.f:4-135): the right-hand side of the Stokes solve (rhs, 2 nbk
 * doubles, interleaved) from dphi_dn (nbk) on the installed geometry: surface tension,
 * the far field of strain rate cap and the electric stress of strength e0. As in the
 * reference, the electric term's `alpha` is the value left by the previous loop,
 * 2 pi (nd_k - 1) / nd_k of the last drop (stokesbubb.f:125). eb_setvelf is zbond = 0.
 * eb_setvelf_bond takes the Bond number zbond[2] (complex; NULL: 0) and, for zbond != 0,
 * the per-drop C_k zc (complex, k, in rhs's memory): the gravity term and the C_k sums
 * (:38-56, :73-102), and in wall mode minus the reflected log sources of REFSING
 * (:53-60). The wall branch of the reference subtracts a `zstr` it never assigns (:67);
 * here it is the capillary term of the free-space branch, the term INTERFACENEW keeps on
 * a wall (both readings agree for cap = 0). */
int eb_setvelf(eb_ctx* ctx, const double* dphi_dn, double cap, double e0, double* rhs,
               int mem);
int eb_setvelf_bond(eb_ctx* ctx, const double* dphi_dn, double cap, double e0, const double* zbond,
                    const double* zc, double* rhs, int mem);

/* F (electric.f:968-1109): the RK right-hand side of the interface positions. rku
 * (interleaved x, y of all nodes, 2 nbk doubles) -> rkup (the node velocities, same
 * layout): EXTRACTDAT, Laplace solve, DIRICH_NEU_MAP, SETVELF, Stokes solve,
 * INTERFACENEW, EQUIT and the filtered node velocity, all on the GPU. Installs the
 * geometry of rku in the context; model->zbond != 0 runs the wall-bounded branch. */
int eb_rk_f(eb_ctx* ctx, int k, const int* nd, const double* rku, double* rkup,
            const eb_model* model, eb_stage_info* info, int mem);

/* RK2 (electric.f:762-786): one modified-Euler step of size dt on ybar (2 nbk
 * doubles, updated in place). Both stages run on the GPU; with mem = EB_DEVICE the
 * state never leaves device memory. */
int eb_rk2_step(eb_ctx* ctx, int k, const int* nd, double dt, double* ybar,
                const eb_model* model, eb_stage_info* info, int mem);

/* The point-doubling policy of the time loop (electric.f:181-219) on the GPU.
 * eb_getfourier is GETFOURIER (electric.f:531-570) for every drop of the RK state rku
 * (interleaved x, y; drop sizes nd, powers of two): the Fourier coefficients c of z/nd, and
 * idoub[b] = 1 (host array of k) when one of the ten modes below drop b's Nyquist mode
 * has |c_i| + |c_{nd-i}| > 1e-11. fmode (optional, nbk doubles in rku's memory) receives
 * per drop at its node offset |c_0| and |c_i| + |c_{nd-i}|, i < nd/2.
 * eb_double is DOUBLE (electric.f:721-757): the drops with idoub[b] = 1 resampled to
 * 2 nd[b] nodes by FINTERC's spectral interpolation (pv_integral.f:276-328), the others
 * copied, into rku2 laid out with the new sizes. */
int eb_getfourier(eb_ctx* ctx, int k, const int* nd, const double* rku, int* idoub, double* fmode,
                  int mem);
int eb_double(eb_ctx* ctx, int k, const int* nd, const double* rku, const int* idoub, double* rku2,
              int mem);

/* Many independent simulations in one context; no counterpart in the reference, which
 * advances one simulation per process (electric.f:134-251). After eb_batch_define, the
 * drops of every geometry the context installs (eb_set_geometry, eb_extractdat, eb_rk_f,
 * eb_rk2_step) form nsim simulations, simulation s holding the next sim_k[s] drops, and
 *  - no layer sum mixes simulations (the FMM tree is a forest with one cell per
 *    simulation);
 *  - eb_stokes_solve and eb_laplace_solve run GMRES per simulation (its own Krylov space
 *    and stopping test; the simulations iterate in lockstep in the same launches); the
 *    info holds the largest iteration count, residual and IERR over the simulations;
 *  - FASMVP's far-field pressure is that of each simulation's first drop, and SETVELF
 *    takes E0 per simulation (e0[s]; NULL: the eb_model's e0 for all) and the alpha of
 *    each simulation's last drop (stokesbubb.f:125).
 * nsim = 0 returns the context to one simulation. A context in wall mode takes no
 * batch (EB_ERR_ARG). */
int eb_batch_define(eb_ctx* ctx, int nsim, const int* sim_k, const double* e0);

/* Transposed operators and adjoint solves, for reverse-mode gradients of what a solve
 * produces with respect to its right-hand side (and so to the parameters that enter it
 * linearly, such as E0 and cap through SETVELF): for J(x) with A x = b(theta),
 * dJ/dtheta = lambda^T db/dtheta where A^T lambda = dJ/dx. No counterpart in the
 * reference, which has no adjoint; these are the exact transposes, for the real inner
 * product of the solver's unknowns, of FASMVP (stokesbubb.f:496-614, as MATVEC applies
 * it) and of FASMVP_LAP's n x n operator (laplace.f:159-262, without the k constraint
 * sums past YY(N)), formed from the same FMM (a Cauchy sum and a Stokes sum with the
 * charges -v, conj(v) for the Stokes transpose; one Cauchy sum for the Laplace one).
 * The solves are the same GMRES (DGMRES semantics, x0 = rhs; both modes; per simulation
 * in a batch). Not available in wall mode (EB_ERR_ARG): the transposes hold no images. */
int eb_stokes_matvec_adjoint(eb_ctx* ctx, int n, const double* x, double* y, int precision, int mem);
int eb_laplace_matvec_adjoint(eb_ctx* ctx, int n, const double* x, double* y, int precision, int mem);
int eb_stokes_solve_adjoint(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                            eb_solve_info* info, int mem);
int eb_laplace_solve_adjoint(eb_ctx* ctx, int n, const double* rhs, double* soln, int mode,
                             eb_solve_info* info, int mem);

/* Reverse mode through the time stepper: the adjoint of F and of the RK2 step with
 * respect to the node positions, E0 and cap (no counterpart in the reference). Free
 * space and one simulation only (model->zbond = 0, no batch; EB_ERR_ARG otherwise).
 *
 * eb_rk_f_vjp: rku_bar = v^T dF/drku (2 nbk doubles), and param_bar[0] += v^T dF/dE0,
 * param_bar[1] += v^T dF/dcap (param_bar may be NULL). F is differentiated as the map
 * with exact solves: the call reruns the stage at rku (its solves with model->mode and
 * the context's gmres_tol), then solves with the transposed Stokes and Laplace operators
 * (eb_stokes_solve_adjoint, eb_laplace_solve_adjoint) and adds the derivatives of every
 * layer sum with respect to its targets, sources and weights (direct O(nbk^2) sums in
 * FP64), of the spectral derivatives, interpolations and Fourier integrals (their
 * transposes), and of the pointwise geometry. FILTER's zeroing of coefficient parts
 * below 1e-13 is differentiated as the identity (it moves F by at most 1e-13 per
 * coefficient; differences of F at steps above about 1e-7 see those parts move).
 *
 * eb_rk2_step_vjp: the transpose of one eb_rk2_step from the state ybar: rbar (in: dJ/dy
 * after the step, out: dJ/dy before it), param_bar accumulated. The stage states are
 * recomputed from ybar (checkpointed by the caller, one state per step).
 *
 * eb_deformation: value = sum over drops of (L - B)/(L + B), L and B the largest and
 * smallest distance of a drop's nodes from its centroid (the mean of its nodes), the
 * Taylor deformation; rku_bar (optional) = its gradient with respect to rku. */
typedef struct eb_adjoint_info {
  int lap_iters;        /* Krylov iterations of the forward Laplace solves           */
  int stokes_iters;     /* Krylov iterations of the forward Stokes solves            */
  int lap_adj_iters;    /* Krylov iterations of the transposed Laplace solves        */
  int stokes_adj_iters; /* Krylov iterations of the transposed Stokes solves         */
  int ierr;             /* 0 when all four solves converged, else the first nonzero IERR */
} eb_adjoint_info;

int eb_rk_f_vjp(eb_ctx* ctx, int k, const int* nd, const double* rku, const double* v,
                const eb_model* model, double* rku_bar, double* param_bar, eb_adjoint_info* info,
                int mem);
int eb_rk2_step_vjp(eb_ctx* ctx, int k, const int* nd, double dt, const double* ybar, double* rbar,
                    const eb_model* model, double* param_bar, eb_adjoint_info* info, int mem);
int eb_deformation(eb_ctx* ctx, int k, const int* nd, const double* rku, double* value, double* rku_bar,
                   int mem);

/* The whole reverse pass: value = the deformation after nsteps RK2 steps of size dt from
 * y0; y0_bar = its gradient with respect to y0, param_bar[0] += dJ/dE0, param_bar[1] +=
 * dJ/dcap (param_bar may be NULL). The state before each step and its two stages' Laplace
 * and Stokes solutions are kept on the device (8 nbk doubles per step, plus 8 nbk), and the
 * reverse pass replays each step's stages with those solutions. */
int eb_rk2_gradient(eb_ctx* ctx, int k, const int* nd, double dt, int nsteps, const double* y0,
                    const eb_model* model, double* value, double* y0_bar, double* param_bar,
                    eb_adjoint_info* info, int mem);

/* Wall-bounded flow, the IFLAG2 = 1 branch of CADAPDR / CADAPMOD (COMMON /wallinfo/,
 * electric.f:55; cadapdrop.f:142-145, cadapdrop2.f:159-197 and 690-721, cadap2.f:1468-1586):
 * with iwall = 1 every Stokes sum of the installed geometry (eb_stokes_matvec,
 * eb_stokes_sum, eb_interface_velocity, the solves) adds the sum over the images of the
 * sources across the wall y = 0; the nodes must lie on or above it (EB_ERR_ARG otherwise,
 * at the next install). xleft and slength, the square [xleft, xleft + slength] x
 * [0, slength] of the reference's wall-bounded FMM, are EXTRACTDAT's (electric.f:710-711:
 * the smallest x and max(x range, largest y) of the nodes) and are recomputed at every
 * install; eb_get_wall reads them. The mode persists across installs; setting it on an
 * installed geometry rebuilds its tree. Not available for a batch (EB_ERR_ARG).
 * Replaces the reference's IFLAG2 argument of CADAPDR/CADAPMOD (cadapdrop.f:3, cadapmod.f:3)
 * and its XLEFT/SLENGTH arguments. */
int eb_set_wall(eb_ctx* ctx, int iwall);
int eb_get_wall(eb_ctx* ctx, int* iwall, double* xleft, double* slength);

/* Input deck and checkpoint files of the reference (host only, no context).
 * eb_bubbin_read: the first deck of a `bubbin` file as READINI reads it
 * (electric.f:275-337): k drops (k <= kmax), nd[k], params[7] = {dt, tfinal, nplot, cap,
 * bondx, bondy, E0}, drops[6k] = per drop {ai, bi, thetax, cx, cy, ncyc}.
 * eb_geoinit: the initial curves of GEOINIT / INITPARAM (electric.f:340-496) at theta_i =
 * 2 pi i / nd: z (interleaved x, y), and optionally dsdth, kappa (nbk each) and the
 * initial areas area0 (k).
 * eb_dumpdata / eb_readdata: `geometry.data` as DUMPDATA writes and READDATA reads it
 * (electric.f:1360-1421); z holds the nbk nodes interleaved, nmax bounds nbk on read. */
int eb_bubbin_read(const char* path, int kmax, int* k, int* nd, double* params, double* drops);
int eb_geoinit(int k, const int* nd, const double* drops, double* z, double* dsdth, double* kappa,
               double* area0);
int eb_dumpdata(const char* path, int k, const int* nd, double dt, double time, const double* area0,
                const double* arcl0, const double* z);
int eb_readdata(const char* path, int kmax, long nmax, int* k, int* nd, double* dt, double* time,
                double* area0, double* arcl0, double* z);

/* gfortran-callable shims with the exact DGMRES MATVEC signature
 * (dpigmr.f:316-318, stokesbubb.f:419, laplace.f:429). They use the context set with
 * eb_set_default_ctx and host memory, and abort the process on error, as the
 * reference's STOP would. */
int eb_set_default_ctx(eb_ctx* ctx);
void matvec_(const int* n, const double* xx, double* yy, const int* nelt, const int* ia,
             const int* ja, const double* a, const int* isym);
void matvec_lapl_(const int* n, const double* xx, double* yy, const int* nelt,
                  const int* ia, const int* ja, const double* a, const int* isym);

#ifdef __cplusplus
}
#endif
#endif
