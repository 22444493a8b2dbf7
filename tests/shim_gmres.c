/*
 * A caller of the DGMRES drop-in shims written the way the reference's Fortran calls its
 * operator: the GMRES loop below never sees a context, a device pointer or a precision
 * flag; each operator apply is a call of matvec_ or matvec_lapl_ with every argument
 * passed by reference, exactly as DPIGMR calls MATVEC(N, X, Y, NELT, IA, JA, A, ISYM)
 * (dpigmr.f:316-318). The geometry is installed beforehand, as EXTRACTDAT fills COMMON
 * /inteqn/ before SOLVEI / SOLVE_LAPL run (electric.f:1041, stokesbubb.f:294-415).
 *
 * The GMRES is the unrestarted, unpreconditioned DGMRES of SOLVEI: x0 = b, modified
 * Gram-Schmidt, Givens rotations, stop when the residual estimate over ||b|| is at most
 * TOL (dgmres.f:413-553, dpigmr.f:242-439, dheqr.f, dhels.f).
 *
 *   shim_gmres <in.bin> <out.bin> <0: Stokes matvec_ | 1: Laplace matvec_lapl_> <tol>
 *   in.bin : int32 k, int32 nd[k], float64 rku[2 nbk], int32 n, float64 rhs[n]
 *   out.bin: int32 iters, float64 err, float64 x[n]
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "eb_gb300.h"

#define MAXL 100

static void die(const char* what, int st) {
  fprintf(stderr, "%s failed: %d (%s)\n", what, st, eb_last_error());
  exit(2);
}

static double dot(int n, const double* a, const double* b) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: shim_gmres in.bin out.bin which tol\n");
    return 1;
  }
  const int which = atoi(argv[3]);
  const double tol = atof(argv[4]);
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 1;
  int k = 0, n = 0;
  if (fread(&k, 4, 1, f) != 1 || k <= 0) return 1;
  int* nd = (int*)malloc(sizeof(int) * k);
  if (fread(nd, 4, k, f) != (size_t)k) return 1;
  int nbk = 0;
  for (int b = 0; b < k; ++b) nbk += nd[b];
  double* rku = (double*)malloc(sizeof(double) * 2 * nbk);
  if (fread(rku, 8, 2 * nbk, f) != (size_t)(2 * nbk)) return 1;
  if (fread(&n, 4, 1, f) != 1 || n <= 0) return 1;
  double* b = (double*)malloc(sizeof(double) * n);
  if (fread(b, 8, n, f) != (size_t)n) return 1;
  fclose(f);

  eb_ctx* ctx = NULL;
  int st = eb_ctx_create(&ctx, NULL);
  if (st) die("eb_ctx_create", st);
  st = eb_extractdat(ctx, k, nd, rku, NULL, NULL, NULL, NULL, NULL, NULL, NULL, EB_HOST);
  if (st) die("eb_extractdat", st);
  st = eb_set_default_ctx(ctx);
  if (st) die("eb_set_default_ctx", st);

  /* the arguments DPIGMR passes and the operator ignores */
  int nelt = 1, isym = 0, ia[1] = {0}, ja[1] = {0};
  double a[1] = {0.0};

  double* x = (double*)malloc(sizeof(double) * n);
  double* v = (double*)malloc(sizeof(double) * (size_t)n * (MAXL + 1));
  double* w = (double*)malloc(sizeof(double) * n);
  double h[MAXL + 1][MAXL];
  double cs[MAXL], sn[MAXL], g[MAXL + 1], y[MAXL];
  memcpy(x, b, sizeof(double) * n); /* x0 = b (stokesbubb.f:346-349) */
  const double bnrm = sqrt(dot(n, b, b));
  if (which == 0) matvec_(&n, x, w, &nelt, ia, ja, a, &isym);
  else matvec_lapl_(&n, x, w, &nelt, ia, ja, a, &isym);
  for (int i = 0; i < n; ++i) v[i] = b[i] - w[i];
  double beta = sqrt(dot(n, v, v));
  int iters = 0;
  double err = beta / bnrm;
  if (err > tol) {
    for (int i = 0; i < n; ++i) v[i] /= beta;
    memset(g, 0, sizeof(g));
    g[0] = beta;
    int j;
    for (j = 0; j < MAXL; ++j) {
      double* vj = v + (size_t)j * n;
      double* vn = v + (size_t)(j + 1) * n;
      if (which == 0) matvec_(&n, vj, vn, &nelt, ia, ja, a, &isym);
      else matvec_lapl_(&n, vj, vn, &nelt, ia, ja, a, &isym);
      for (int i = 0; i <= j; ++i) { /* modified Gram-Schmidt */
        double hij = dot(n, v + (size_t)i * n, vn);
        h[i][j] = hij;
        for (int r = 0; r < n; ++r) vn[r] -= hij * v[(size_t)i * n + r];
      }
      double hn = sqrt(dot(n, vn, vn));
      h[j + 1][j] = hn;
      if (hn > 0) for (int r = 0; r < n; ++r) vn[r] /= hn;
      for (int i = 0; i < j; ++i) { /* earlier Givens rotations */
        double t = cs[i] * h[i][j] - sn[i] * h[i + 1][j];
        h[i + 1][j] = sn[i] * h[i][j] + cs[i] * h[i + 1][j];
        h[i][j] = t;
      }
      double d = hypot(h[j][j], h[j + 1][j]);
      cs[j] = h[j][j] / d;
      sn[j] = -h[j + 1][j] / d;
      h[j][j] = d;
      h[j + 1][j] = 0.0;
      g[j + 1] = sn[j] * g[j];
      g[j] = cs[j] * g[j];
      iters = j + 1;
      err = fabs(g[j + 1]) / bnrm;
      if (err <= tol) break;
    }
    int m = iters;
    for (int i = m - 1; i >= 0; --i) { /* back substitution (DHELS) */
      double s = g[i];
      for (int c = i + 1; c < m; ++c) s -= h[i][c] * y[c];
      y[i] = s / h[i][i];
    }
    for (int i = 0; i < m; ++i)
      for (int r = 0; r < n; ++r) x[r] += y[i] * v[(size_t)i * n + r];
  }
  eb_ctx_destroy(ctx);
  f = fopen(argv[2], "wb");
  if (!f) return 1;
  fwrite(&iters, 4, 1, f);
  fwrite(&err, 8, 1, f);
  fwrite(x, 8, n, f);
  fclose(f);
  return 0;
}
