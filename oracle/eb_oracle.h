/*
 * CPU oracle for the ElectricBubbles boundary-integral hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: the GPU product never
 * links, loads or calls it. Only tests, the smoke check and the benchmark's CPU
 * baseline leg may use it.
 *
 * Every routine restates a routine of the reference Fortran (mcetal/ElectricBubbles)
 * and cites the file:line it follows. Complex numbers are C99 `double _Complex`,
 * which has the same memory layout as Fortran COMPLEX*16 and as interleaved
 * (re, im) doubles.
 *
 * Pinning: the reference ships no tests and no golden outputs, and the Fortran
 * cannot be compiled where this project is built (no Fortran compiler), so
 * end-to-end parity against the Fortran binary is unpinned. The restatement is
 * pinned instead against the analytic known answers that the reference itself
 * carries: the commented PVINTEV driver (pv_integral.f:1-49, circle with densities
 * 1/(z-z0) and z z'), the CHECK exterior potential (laplace.f:30-73), and the
 * exactness of the direct sums that CADAPDR/DAPIF2 approximate.
 */
#ifndef EB_ORACLE_H
#define EB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double _Complex eb_or_cplx;

/* Geometry of k drops with nd[i] nodes each (nbk total), as filled by EXTRACTDAT
 * (electric.f:636-716) into COMMON /inteqn/ and /problem/. */
typedef struct {
  int k;
  const int* nd;
  int nbk;
  const eb_or_cplx* z;     /* node positions */
  const eb_or_cplx* dz;    /* dz = -z'(alpha) */
  const double* dsda;      /* |dz| */
  const double* kappa;     /* curvature */
  const eb_or_cplx* zk;    /* drop centroids */
  int iwall;               /* 1: wall-bounded (the wall is y = 0) */
  double xleft, slength;   /* wall data of EXTRACTDAT (electric.f:710-711) */
} eb_or_geom;

/* ---- spectral (dcfft.f, electric.f, pv_integral.f) ---- */
void eb_or_fft(int n, eb_or_cplx* c, int dir);
void eb_or_fdifff(int n, const eb_or_cplx* f, eb_or_cplx* df);
void eb_or_fourint(int n, const eb_or_cplx* zf, eb_or_cplx* zfi);
void eb_or_filter(int n, eb_or_cplx* cn);
void eb_or_finterc(int nd, const eb_or_cplx* f, eb_or_cplx* f2);
void eb_or_finter(int nd, const double* f, double* f2);

/* ---- geometry (electric.f:636-716) ---- */
void eb_or_extractdat(int k, const int* nd, const double* rku, eb_or_cplx* z,
                      eb_or_cplx* zk, eb_or_cplx* dz, double* tha, double* dsda,
                      double* kappa, eb_or_cplx* ckern, double* area);

/* ---- layer-potential sums ---- */
void eb_or_stokes_direct(int n, const eb_or_cplx* z, const eb_or_cplx* dz,
                         const double* hpt, const eb_or_cplx* dens, int sign,
                         eb_or_cplx* gradw, int nthreads);
void eb_or_stokes_direct_at(int n, const eb_or_cplx* z, const eb_or_cplx* dz,
                            const double* hpt, const eb_or_cplx* dens, int sign, int nt,
                            const int* tidx, eb_or_cplx* out, int nthreads);
int eb_or_cadap_fmm(int n, const eb_or_cplx* z, const eb_or_cplx* dz,
                    const double* hpt, const eb_or_cplx* dens, int sign, int levmax,
                    double tol, eb_or_cplx* gradw, int nthreads);
/* CADAPDR / CADAPMOD with IFLAG2 = iwall (images across the wall y = 0) */
int eb_or_cadap_fmm_w(int n, const eb_or_cplx* z, const eb_or_cplx* dz,
                      const double* hpt, const eb_or_cplx* dens, int sign, int levmax,
                      double tol, int iwall, double xleft, double slength,
                      eb_or_cplx* gradw, int nthreads);
/* the exact reflected part of the wall-bounded sum (all images, own image included) */
void eb_or_stokes_image_direct(int n, const eb_or_cplx* z, const eb_or_cplx* dz,
                               const double* hpt, const eb_or_cplx* dens, int sign,
                               eb_or_cplx* gimg, int nthreads);
void eb_or_refsing(eb_or_cplx zt, int k, const eb_or_cplx* zk, const eb_or_cplx* zc,
                   const eb_or_cplx* zb, eb_or_cplx* phi, eb_or_cplx* phip, eb_or_cplx* psi);
void eb_or_wallinfo(int nbk, const eb_or_cplx* z, double* xleft, double* slength);
void eb_or_cauchy_direct(int nt, const eb_or_cplx* zt, int ns, const eb_or_cplx* zsrc,
                         const eb_or_cplx* q, int self, eb_or_cplx* field, int nthreads);

/* ---- operators ---- */
enum { EB_OR_DIRECT = 0, EB_OR_CADAP = 1 };
void eb_or_fasmvp(const eb_or_geom* g, const double* u, double* w, int mode,
                  int nthreads);
void eb_or_fasmvp_lap(const eb_or_geom* g, const double* u, double* w, int nthreads);
/* mode EB_OR_CADAP: the Cauchy sum by the restated DAPIF2 (TOL 1e-11, NAPB 30) */
void eb_or_fasmvp_lap2(const eb_or_geom* g, const double* u, double* w, int mode, int nthreads);
/* DAPIF2 (IFLAG7 = 3): field_i = sum_{j != i} q_j / (z_i - z_j), adaptive FMM */
void eb_or_dapif2(int n, const eb_or_cplx* z, const eb_or_cplx* q, double tol, int napb,
                  eb_or_cplx* field, int nthreads);
void eb_or_pvintev(int k, const int* nd, const eb_or_cplx* z, const eb_or_cplx* ucmplx,
                   eb_or_cplx* phicmplx, int nthreads);
void eb_or_dirich_neu_map(const eb_or_geom* g, const double* u, double* phi,
                          double* psi, double* dphi_dn, int nthreads);
void eb_or_interfacenew(const eb_or_geom* g, const eb_or_cplx* ckern,
                        const eb_or_cplx* zc, double cap, const eb_or_cplx* u,
                        double* un, double* flux, int mode, int nthreads);
void eb_or_setvelf(const eb_or_geom* g, const eb_or_cplx* zc, eb_or_cplx zbond,
                   double cap, double e0, const double* dphi_dn, double* rhs);
void eb_or_equit(int nd, const double* tha, const double* un, double* t);

/* ---- GMRES (SLATEC DGMRES with the settings of SOLVEI/SOLVE_LAPL) ---- */
typedef void (*eb_or_matvec_fn)(int n, const double* x, double* y, void* ud);
int eb_or_gmres(int n, const double* b, double* x, eb_or_matvec_fn mv, void* ud,
                int maxl, double tol, int* iter, double* err);

/* ---- one RK2 (Heun) step of the whole model (electric.f:762-786, 968-1109) ---- */
typedef struct {
  double cap, e0;
  eb_or_cplx zbond;
  int mode;       /* EB_OR_DIRECT: direct sums; EB_OR_CADAP: the reference's FMMs
                     (restated CADAPDR for the Stokes sums, DAPIF2 for the Laplace
                     and PV sums) */
  int nthreads;
  int maxl;
  double gmres_tol;
  /* diagnostics of the last F evaluation */
  int lap_iter, stokes_iter;
  double lap_err, stokes_err, flux;
} eb_or_model;
void eb_or_f(eb_or_model* m, int k, const int* nd, const double* rku, double* rkup);
void eb_or_rk2(eb_or_model* m, int k, const int* nd, double dt, double* ybar);

int eb_or_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
