/*
 * CPU oracle for the NuSiF per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * algorithms (HPC-Dwarfs/CFD-Bench, "NuSiF", src/discretization.c,
 * src/solver-rb.c, src/solver-mg.c) used as the checker for the GPU library.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it. The product library never links or calls it.
 *
 * Parity pin: every function here is checked against the reference's own
 * sources compiled from source (oracle/build_ref.sh -> oracle/_ref) on random
 * fields and on whole runs, and against the golden vectors in tests/golden/
 * that the reference itself produced (tests/golden/make_golden.py).
 *
 * Layout (reference src/util.h:19-34): every field is one FP64 array of
 * (imax+2)(jmax+2)(kmax+2) cells, i fastest, one ghost layer;
 * idx = k*(imax+2)*(jmax+2) + j*(imax+2) + i.
 */
#ifndef NUSIF_ORACLE_H
#define NUSIF_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int imax, jmax, kmax;
  double dx, dy, dz;
} OrGrid;

/* boundary flags, reference src/discretization.h:12 */
enum { OR_NOSLIP = 1, OR_SLIP = 2, OR_OUTFLOW = 3, OR_PERIODIC = 4 };
/* face order used for bc[6]: left, right, bottom, top, front, back */
enum { OR_LEFT = 0, OR_RIGHT, OR_BOTTOM, OR_TOP, OR_FRONT, OR_BACK };
/* special boundary problems, reference src/discretization.c:364-389 */
enum { OR_PROBLEM_NONE = 0, OR_PROBLEM_DCAVITY = 1, OR_PROBLEM_CANAL = 2 };

size_t or_padded_size(const OrGrid *g);

double or_max_abs(const double *a, size_t n);
double or_timestep(double dtBound, double dx, double dy, double dz, double umax,
    double vmax, double wmax, double tau);
void or_set_bc(const OrGrid *g, const int bc[6], double *u, double *v, double *w);
void or_special_bc(const OrGrid *g, int problem, double lid, double inflow, double *u);
void or_compute_fgh(const OrGrid *g, double re, double gamma, double gx, double gy,
    double gz, double dt, const double *u, const double *v, const double *w, double *f,
    double *gf, double *h);
void or_compute_rhs(
    const OrGrid *g, double dt, const double *f, const double *gf, const double *h, double *rhs);
double or_normalize_pressure(const OrGrid *g, double *p);
void or_adapt_uv(const OrGrid *g, double dt, const double *f, const double *gf,
    const double *h, const double *p, double *u, double *v, double *w);

/* red-black SOR, reference src/solver-rb.c:27-172; returns iterations, *res_out = res */
int or_solve_rb(const OrGrid *g, double eps, double omega, int itermax, double *p,
    const double *rhs, double *res_out);
/* one red-black SOR sweep without residual (reference src/solver-mg.c:177-224) */
void or_sor_sweep(const OrGrid *g, double omega, double *p, const double *rhs);
/* pressure Neumann ghost copy, six faces (reference src/solver-rb.c:129-148) */
void or_pressure_ghosts(const OrGrid *g, double *p);
/* reference multigrid as it behaves (src/solver-mg.c:299-402, sequential build) */
double or_solve_mg_ref(const OrGrid *g, double omega, int levels, int presmooth,
    int postsmooth, double *p, const double *rhs);

/* geometric multigrid of the library (nusif_oracle_mg.c): level count and
 * dims (3 ints per level), and the solve; mode 0 = FP64, 1 = FP32 in FP64
 * iterative refinement. Returns V-cycles; *relres = ||b-Ap||/||b||. */
int or_mg_levels(const OrGrid *g, int cap, int *dims_out);
int or_mg_solve(const OrGrid *g, int mode, int level_cap, int pre, int post, int coarse_sweeps,
    int inner, int maxcycles, double rtol, double *p, const double *rhs, double *relres);

/* whole-run driver mirroring reference src/main.c:53-88 */
typedef struct {
  int imax, jmax, kmax;
  double xlength, ylength, zlength;
  double re, gamma, tau, te, dt0;
  double gx, gy, gz;
  double u_init, v_init, w_init, p_init;
  int bc[6];
  int problem;
  double lid, inflow;
  double eps, omega;
  int itermax;
  int solver; /* 0 = rb, 1 = mg-ref, 2 = mg, 3 = mg-mixed */
  int levels, presmooth, postsmooth;
  double rtol;
  int mg_levels, mg_pre, mg_post, mg_coarse, mg_cycles, mg_inner;
} OrCase;

typedef struct {
  OrGrid g;
  OrCase c;
  double *u, *v, *w, *p, *rhs, *f, *gf, *h;
  double dt, t, dtBound;
  int nt;
} OrState;

int or_state_init(OrState *s, const OrCase *c);
void or_state_free(OrState *s);
/* one timestep (reference src/main.c:60-80); returns solver iterations (0 for mg-ref) */
int or_state_step(OrState *s, double *res_out);

#ifdef __cplusplus
}
#endif
#endif
