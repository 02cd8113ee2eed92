/*
 * CPU oracle of the geometric-multigrid pressure solvers -- TEST
 * INFRASTRUCTURE ONLY.
 *
 * The reference's multigrid (src/solver-mg.c) never applies its coarse-grid
 * correction (prolongate() writes r[level], correct() adds the never-written
 * e[0]) and, sequentially, never coarsens. The library's "mg" and "mg-mixed"
 * solvers are therefore a corrected algorithm with no reference
 * implementation; this file restates that algorithm on the CPU as the checker
 * of the GPU kernels ("parity unpinned" against the reference: there is
 * nothing in the reference to pin it to; tests pin it instead against the
 * converged red-black solution of the same right-hand side).
 *
 * Algorithm (identical in the GPU library):
 *  - levels: level 0 is the grid; an axis is halved while its size is even
 *    and >= 16; coarsening stops when no axis halves or at the level cap.
 *  - operator: the 7-point Laplacian with homogeneous Neumann walls applied
 *    without ghost cells (a neighbour outside the domain is replaced by the
 *    cell itself).
 *  - smoother: red-black Gauss-Seidel, odd cells (i+j+k odd) first,
 *    x -= r / (2 sum 1/h^2) with r = b - Ax.
 *  - restriction: average of the 2, 4 or 8 children of the residual.
 *  - prolongation: trilinear (weights 3/4, 1/4 per coarsened axis; a
 *    neighbour outside the domain is replaced by the parent), added to x.
 *  - V(pre, post) cycle; coarsest level: a fixed number of sweeps from zero.
 *  - the right-hand side is made mean-free (Neumann null space); convergence
 *    is ||b - Ap||_2 <= rtol ||b||_2 with b the mean-free right-hand side.
 *  - "mg": everything FP64 on p itself, residual checked after pre-smoothing.
 *  - "mg-mixed": FP64 residual of p, FP32 V-cycle for the correction e from
 *    zero, p += e in FP64 (iterative refinement).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "nusif_oracle.h"

#define MG_MAX_LEVELS 16

typedef struct {
  int n[3];       /* cells per axis */
  int r[3];       /* coarsening ratio from the finer level (1 or 2) */
  double ih2[3];  /* 1/h^2 per axis */
} MgLev;

static int mg_build(const OrGrid *g, int cap, MgLev *lv)
{
  int nl = 0;
  lv[0].n[0] = g->imax;
  lv[0].n[1] = g->jmax;
  lv[0].n[2] = g->kmax;
  double h[3] = { g->dx, g->dy, g->dz };
  for (int a = 0; a < 3; a++) {
    lv[0].r[a] = 1;
    lv[0].ih2[a] = 1.0 / (h[a] * h[a]);
  }
  nl = 1;
  while (nl < MG_MAX_LEVELS && (cap <= 0 || nl < cap)) {
    MgLev *f = &lv[nl - 1], *c = &lv[nl];
    int any = 0;
    for (int a = 0; a < 3; a++) {
      if (f->n[a] % 2 == 0 && f->n[a] >= 16) {
        c->n[a] = f->n[a] / 2;
        c->r[a] = 2;
        h[a] *= 2.0;
        any = 1;
      } else {
        c->n[a] = f->n[a];
        c->r[a] = 1;
      }
      c->ih2[a] = 1.0 / (h[a] * h[a]);
    }
    if (!any) break;
    nl++;
  }
  return nl;
}

int or_mg_levels(const OrGrid *g, int cap, int *dims_out)
{
  MgLev lv[MG_MAX_LEVELS];
  int nl = mg_build(g, cap, lv);
  if (dims_out)
    for (int l = 0; l < nl; l++)
      for (int a = 0; a < 3; a++) dims_out[3 * l + a] = lv[l].n[a];
  return nl;
}

/* interior-only arrays of a level: index (k*ny + j)*nx + i with 0-based i,j,k */
#define LIX(L, i, j, k) (((size_t)(k) * (L)->n[1] + (size_t)(j)) * (L)->n[0] + (size_t)(i))

/* ---- level kernels, instantiated for double and float ---- */
#define REAL double
#define SFX d
#include "nusif_oracle_mg.inc"
#undef REAL
#undef SFX
#define REAL float
#define SFX f
#include "nusif_oracle_mg.inc"
#undef REAL
#undef SFX

/* FP64 residual of the fine level, stored as FP32; returns its sum of squares */
static double mg_residual_to_f(const MgLev *L, const double *x, const double *b, float *r32)
{
  double s = 0.0;
  for (int k = 0; k < L->n[2]; k++)
    for (int j = 0; j < L->n[1]; j++)
      for (int i = 0; i < L->n[0]; i++) {
        const size_t c = LIX(L, i, j, k);
        const double r = b[c] - mg_lap_d(L, x, i, j, k);
        r32[c] = (float)r;
        s += r * r;
      }
  return s;
}

/* interior of a padded reference-layout array <-> compact array */
static size_t pad_ix(const OrGrid *g, int i, int j, int k) /* 0-based interior */
{
  return (size_t)(k + 1) * (size_t)(g->imax + 2) * (size_t)(g->jmax + 2) +
         (size_t)(j + 1) * (size_t)(g->imax + 2) + (size_t)(i + 1);
}

/* mean-free right-hand side (compact) and its squared norm */
static double mean_free_rhs(const OrGrid *g, const double *rhs, double *b, double *nb2)
{
  size_t n = (size_t)g->imax * g->jmax * g->kmax, q = 0;
  double s = 0.0;
  for (int k = 0; k < g->kmax; k++)
    for (int j = 0; j < g->jmax; j++)
      for (int i = 0; i < g->imax; i++) s += rhs[pad_ix(g, i, j, k)];
  double mean = s / (double)n;
  double s2 = 0.0;
  for (int k = 0; k < g->kmax; k++)
    for (int j = 0; j < g->jmax; j++)
      for (int i = 0; i < g->imax; i++, q++) {
        b[q] = rhs[pad_ix(g, i, j, k)] - mean;
        s2 += b[q] * b[q];
      }
  *nb2 = s2;
  return mean;
}

/*
 * Inverse of the coarsest operator deflated by its null space:
 * M = A - (s/n) 1 1^T with s = 2 sum 1/h^2; -M is SPD, factorised by Cholesky
 * and inverted column by column (row-major result). For a mean-free b,
 * x = M^-1 b solves A x = b with mean(x) = 0. Returns NULL on failure.
 */
static double *coarse_inverse(const MgLev *L)
{
  const int nx = L->n[0], ny = L->n[1], nz = L->n[2], n = nx * ny * nz;
  const double s = 2.0 * (L->ih2[0] + L->ih2[1] + L->ih2[2]);
  double *a = (double *)malloc(sizeof(double) * (size_t)n * n);
  double *minv = (double *)malloc(sizeof(double) * (size_t)n * n);
  double *y = (double *)malloc(sizeof(double) * (size_t)n);
  for (size_t q = 0; q < (size_t)n * n; q++) a[q] = s / n;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const int q = i + nx * (j + ny * k);
        const int idx[3] = { i, j, k }, n3[3] = { nx, ny, nz }, st[3] = { 1, nx, nx * ny };
        for (int ax = 0; ax < 3; ax++)
          for (int sg = -1; sg <= 1; sg += 2) {
            const int c = idx[ax] + sg;
            if (c < 0 || c >= n3[ax]) continue;
            a[(size_t)q * n + q] += L->ih2[ax];
            a[(size_t)q * n + q + sg * st[ax]] -= L->ih2[ax];
          }
      }
  for (int c = 0; c < n; c++) {
    double d = a[(size_t)c * n + c];
    for (int q = 0; q < c; q++) d -= a[(size_t)c * n + q] * a[(size_t)c * n + q];
    if (!(d > 0.0)) {
      free(a);
      free(minv);
      free(y);
      return NULL;
    }
    d = sqrt(d);
    a[(size_t)c * n + c] = d;
    for (int r = c + 1; r < n; r++) {
      double v = a[(size_t)r * n + c];
      for (int q = 0; q < c; q++) v -= a[(size_t)r * n + q] * a[(size_t)c * n + q];
      a[(size_t)r * n + c] = v / d;
    }
  }
  for (int col = 0; col < n; col++) {
    for (int r = 0; r < n; r++) {
      double v = (r == col) ? 1.0 : 0.0;
      for (int q = 0; q < r; q++) v -= a[(size_t)r * n + q] * y[q];
      y[r] = v / a[(size_t)r * n + r];
    }
    for (int r = n - 1; r >= 0; r--) {
      double v = y[r];
      for (int q = r + 1; q < n; q++) v -= a[(size_t)q * n + r] * y[q];
      y[r] = v / a[(size_t)r * n + r];
    }
    for (int r = 0; r < n; r++) minv[(size_t)r * n + col] = -y[r];
  }
  free(a);
  free(y);
  return minv;
}

#define MG_MAX_DIRECT 1024

/*
 * Solve A p = rhs - mean(rhs) on the padded array p (warm start = its
 * interior). mode 0: "mg" (FP64), mode 1: "mg-mixed". coarse_sweeps 0 selects
 * the exact coarsest solve when that level has at most 1024 cells (else, and
 * for a single-level FP64 solve, 64 sweeps). mode 1 runs up to `inner` FP32
 * V-cycles per FP64 residual and ends them once ||r - A e||^2 <= (rtol/2)^2
 * ||b||^2. Returns the number of V-cycles; *relres = ||b - Ap|| / ||b|| of the
 * returned p. The ghost layer of p is refreshed (Neumann copy) on return.
 */
int or_mg_solve(const OrGrid *g, int mode, int level_cap, int pre, int post, int coarse_sweeps,
    int inner, int maxcycles, double rtol, double *p, const double *rhs, double *relres)
{
  MgLev lv[MG_MAX_LEVELS];
  int nl = mg_build(g, level_cap, lv);
  size_t n0 = (size_t)g->imax * g->jmax * g->kmax;
  const MgLev *Lc = &lv[nl - 1];
  const int nc = Lc->n[0] * Lc->n[1] * Lc->n[2];
  if (coarse_sweeps == 0 && (nc > MG_MAX_DIRECT || (mode == 0 && nl == 1))) coarse_sweeps = 64;
  double *minv = coarse_sweeps == 0 ? coarse_inverse(Lc) : NULL;
  float *minv32 = NULL;
  if (minv && mode == 1) {
    minv32 = (float *)malloc(sizeof(float) * (size_t)nc * nc);
    for (size_t q = 0; q < (size_t)nc * nc; q++) minv32[q] = (float)minv[q];
  }
  if (inner < 1) inner = 1;
  double *b0 = (double *)malloc(n0 * sizeof(double));
  double *x0 = (double *)malloc(n0 * sizeof(double));
  double nb2 = 0.0;
  mean_free_rhs(g, rhs, b0, &nb2);
  {
    size_t q = 0;
    for (int k = 0; k < g->kmax; k++)
      for (int j = 0; j < g->jmax; j++)
        for (int i = 0; i < g->imax; i++, q++) x0[q] = p[pad_ix(g, i, j, k)];
  }
  const double tol2 = rtol * rtol * nb2;
  int cycles = 0;
  double res2 = 0.0;
  if (nb2 == 0.0) {
    res2 = 0.0;
  } else if (mode == 0) {
    /* FP64 levels 1..nl-1 */
    double *xs[MG_MAX_LEVELS] = { 0 }, *bs[MG_MAX_LEVELS] = { 0 };
    xs[0] = x0;
    bs[0] = b0;
    for (int l = 1; l < nl; l++) {
      size_t nn = (size_t)lv[l].n[0] * lv[l].n[1] * lv[l].n[2];
      xs[l] = (double *)calloc(nn, sizeof(double));
      bs[l] = (double *)calloc(nn, sizeof(double));
    }
    for (int m = 1;; m++) {
      if (nl == 1) {
        for (int s = 0; s < coarse_sweeps; s++) mg_sweep_d(&lv[0], xs[0], bs[0], 0);
        res2 = mg_residual_norm2_d(&lv[0], xs[0], bs[0]);
      } else {
        for (int s = 0; s < pre; s++) mg_sweep_d(&lv[0], xs[0], bs[0], 0);
        res2 = mg_restrict_d(&lv[0], &lv[1], xs[0], bs[0], bs[1]);
      }
      cycles = m;
      if (res2 <= tol2 || m >= maxcycles) break;
      if (nl > 1) {
        mg_vcycle_d(lv, nl, 1, xs, bs, pre, post, coarse_sweeps, minv);
        mg_prolong_add_d(&lv[0], &lv[1], xs[0], xs[1]);
        for (int s = 0; s < post; s++) mg_sweep_d(&lv[0], xs[0], bs[0], 0);
      }
    }
    for (int l = 1; l < nl; l++) {
      free(xs[l]);
      free(bs[l]);
    }
  } else {
    /* FP32 V-cycle on the correction, FP64 residual and update */
    float *xs[MG_MAX_LEVELS] = { 0 }, *bs[MG_MAX_LEVELS] = { 0 };
    for (int l = 0; l < nl; l++) {
      size_t nn = (size_t)lv[l].n[0] * lv[l].n[1] * lv[l].n[2];
      xs[l] = (float *)calloc(nn, sizeof(float));
      bs[l] = (float *)calloc(nn, sizeof(float));
    }
    const double tol_inner = 0.25 * rtol * rtol * nb2;
    for (int m = 0;; m++) {
      res2 = mg_residual_to_f(&lv[0], x0, b0, bs[0]);
      if (res2 <= tol2 || m >= maxcycles) break;
      if (nl == 1) {
        mg_coarsest_f(&lv[0], xs[0], bs[0], coarse_sweeps, minv32);
        cycles++;
      } else {
        for (int q = 0; q < inner; q++) {
          for (int s = 0; s < pre; s++) mg_sweep_f(&lv[0], xs[0], bs[0], q == 0 && s == 0);
          if (pre == 0 && q == 0) memset(xs[0], 0, sizeof(float) * n0);
          const double rin = mg_restrict_f(&lv[0], &lv[1], xs[0], bs[0], bs[1]);
          cycles++;
          if (rin <= tol_inner) break;
          mg_vcycle_f(lv, nl, 1, xs, bs, pre, post, coarse_sweeps, minv32);
          mg_prolong_add_f(&lv[0], &lv[1], xs[0], xs[1]);
          for (int s = 0; s < post; s++) mg_sweep_f(&lv[0], xs[0], bs[0], 0);
        }
      }
      for (size_t q = 0; q < n0; q++) x0[q] += (double)xs[0][q];
    }
    for (int l = 0; l < nl; l++) {
      free(xs[l]);
      free(bs[l]);
    }
  }
  {
    size_t q = 0;
    for (int k = 0; k < g->kmax; k++)
      for (int j = 0; j < g->jmax; j++)
        for (int i = 0; i < g->imax; i++, q++) p[pad_ix(g, i, j, k)] = x0[q];
  }
  or_pressure_ghosts(g, p);
  free(b0);
  free(x0);
  free(minv);
  free(minv32);
  if (relres) *relres = nb2 > 0.0 ? sqrt(res2 / nb2) : 0.0;
  return cycles;
}
