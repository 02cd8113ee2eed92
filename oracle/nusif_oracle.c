/*
 * CPU oracle for the NuSiF per-timestep hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithms, written for checking the
 * GPU library, never linked into it. Each function names the reference
 * file:line range it restates (paths inside HPC-Dwarfs/CFD-Bench).
 *
 * The arithmetic inside each cell update keeps the reference's expression
 * trees (operand order and parenthesisation), because the oracle is pinned
 * bit-for-bit against the reference compiled from source with the same
 * compiler flags. Loop structure, helpers and naming are this project's own.
 *
 * Parity pin: tests/test_oracle_pin.py compares every function with the
 * reference built by oracle/build_ref.sh, and tests/golden/ holds vectors
 * the reference produced (tests/golden/make_golden.py).
 */
#include "nusif_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* padded index, reference src/util.h:19-34 (i fastest, one ghost layer) */
#define IX(g, i, j, k) \
  ((size_t)(k) * (size_t)((g)->imax + 2) * (size_t)((g)->jmax + 2) + \
   (size_t)(j) * (size_t)((g)->imax + 2) + (size_t)(i))

size_t or_padded_size(const OrGrid *g)
{
  return (size_t)(g->imax + 2) * (size_t)(g->jmax + 2) * (size_t)(g->kmax + 2);
}

/* maxElement, reference src/discretization.c:391-401: running max of |a| over
 * the whole padded array (ghosts included), seeded with DBL_MIN. */
double or_max_abs(const double *a, size_t n)
{
  double m = DBL_MIN;
  for (size_t q = 0; q < n; q++) {
    double x = fabs(a[q]);
    if (!(m > x)) m = x;
  }
  return m;
}

/* computeTimestep, reference src/discretization.c:431-453 */
double or_timestep(double dtBound, double dx, double dy, double dz, double umax,
    double vmax, double wmax, double tau)
{
  double dt = dtBound;
  if (umax > 0 && dt > dx / umax) dt = dx / umax;
  if (vmax > 0 && dt > dy / vmax) dt = dy / vmax;
  if (wmax > 0 && dt > dz / wmax) dt = dz / wmax;
  return dt * tau;
}

/*
 * setBoundaryConditions, reference src/discretization.c:119-332.
 *
 * Every face is the same rule seen along its own normal axis: the velocity
 * component normal to the face lives on the wall face (index 0 on the low
 * side, n on the high side), the two tangential components have a ghost cell
 * (index 0 or n+1) mirrored from the first interior cell. Faces are applied
 * in the reference order top, bottom, left, right, front, back, because later
 * faces read values that earlier faces wrote.
 */
typedef struct {
  int axis; /* 0 = x, 1 = y, 2 = z */
  int high; /* 0 = low side, 1 = high side */
  int flag_slot;
} FaceDesc;

static void face_apply(const OrGrid *g, const FaceDesc *fd, int bc, double *vel[3])
{
  if (bc != OR_NOSLIP && bc != OR_SLIP && bc != OR_OUTFLOW) return; /* periodic: no-op */
  int n[3] = { g->imax, g->jmax, g->kmax };
  int ax = fd->axis;
  int a1 = (ax == 0) ? 1 : 0; /* first tangential axis (outer loop is the other) */
  int a2 = (ax == 2) ? 1 : 2;
  int wall = fd->high ? n[ax] : 0;            /* normal component on the wall face */
  int wall_in = fd->high ? n[ax] - 1 : 1;     /* its interior neighbour (outflow) */
  int ghost = fd->high ? n[ax] + 1 : 0;       /* tangential ghost */
  int inner = fd->high ? n[ax] : 1;           /* tangential first interior */
  for (int b = 1; b <= n[a2]; b++) {
    for (int a = 1; a <= n[a1]; a++) {
      int c[3];
      c[a1] = a;
      c[a2] = b;
      for (int comp = 0; comp < 3; comp++) {
        double *q = vel[comp];
        if (comp == ax) {
          c[ax] = wall;
          size_t dst = IX(g, c[0], c[1], c[2]);
          if (bc == OR_OUTFLOW) {
            c[ax] = wall_in;
            q[dst] = q[IX(g, c[0], c[1], c[2])];
          } else {
            q[dst] = 0.0;
          }
        } else {
          c[ax] = inner;
          double in = q[IX(g, c[0], c[1], c[2])];
          c[ax] = ghost;
          q[IX(g, c[0], c[1], c[2])] = (bc == OR_NOSLIP) ? -in : in;
        }
      }
    }
  }
}

void or_set_bc(const OrGrid *g, const int bc[6], double *u, double *v, double *w)
{
  static const FaceDesc order[6] = {
    { 1, 1, OR_TOP }, { 1, 0, OR_BOTTOM }, { 0, 0, OR_LEFT },
    { 0, 1, OR_RIGHT }, { 2, 0, OR_FRONT }, { 2, 1, OR_BACK },
  };
  double *vel[3] = { u, v, w };
  for (int f = 0; f < 6; f++) face_apply(g, &order[f], bc[order[f].flag_slot], vel);
}

/* setSpecialBoundaryCondition, reference src/discretization.c:364-389.
 * dcavity: lid ghost U(i,jmax+1,k) = 2*lid - U(i,jmax,k) for i<imax, k<kmax
 * (the reference hard-codes lid = 1, i.e. "2.0 - U").
 * canal: inflow face U(0,j,k) = inflow (the reference hard-codes 2.0). */
void or_special_bc(const OrGrid *g, int problem, double lid, double inflow, double *u)
{
  if (problem == OR_PROBLEM_DCAVITY) {
    double twice = 2.0 * lid;
    for (int k = 1; k < g->kmax; k++)
      for (int i = 1; i < g->imax; i++)
        u[IX(g, i, g->jmax + 1, k)] = twice - u[IX(g, i, g->jmax, k)];
  } else if (problem == OR_PROBLEM_CANAL) {
    for (int k = 1; k <= g->kmax; k++)
      for (int j = 1; j <= g->jmax; j++) u[IX(g, 0, j, k)] = inflow;
  }
}

/* Donor-cell convective difference d(c q)/ds (reference discretization.c:491-594).
 * cp / cm: doubled transport velocity on the + / - side; q, qp, qm: transported
 * quantity at the centre, + and - neighbours. */
static inline double donor(
    double inv, double gamma, double cp, double cm, double q, double qp, double qm)
{
  return inv * 0.25 * (cp * (q + qp) - cm * (q + qm)) +
         gamma * inv * 0.25 * (fabs(cp) * (q - qp) + fabs(cm) * (q - qm));
}

/* second difference (reference discretization.c:517-522 and siblings) */
static inline double second(double inv, double qp, double q, double qm)
{
  return inv * inv * (qp - 2.0 * q + qm);
}

/* computeFG, reference src/discretization.c:455-652 */
void or_compute_fgh(const OrGrid *g, double re, double gamma, double gx, double gy,
    double gz, double dt, const double *u, const double *v, const double *w, double *f,
    double *gf, double *h)
{
  const double iRe = 1.0 / re;
  const double ix = 1.0 / g->dx, iy = 1.0 / g->dy, iz = 1.0 / g->dz;
  const size_t sj = (size_t)(g->imax + 2);
  const size_t sk = sj * (size_t)(g->jmax + 2);

  for (int k = 1; k <= g->kmax; k++) {
    for (int j = 1; j <= g->jmax; j++) {
      for (int i = 1; i <= g->imax; i++) {
        const size_t c = IX(g, i, j, k);
        /* F: x-momentum at the +x face */
        {
          double uc = u[c];
          double cx = donor(ix, gamma, uc + u[c + 1], uc + u[c - 1], uc, u[c + 1], u[c - 1]);
          double cy = donor(iy, gamma, v[c] + v[c + 1], v[c - sj] + v[c + 1 - sj], uc,
              u[c + sj], u[c - sj]);
          double cz = donor(iz, gamma, w[c] + w[c + 1], w[c - sk] + w[c + 1 - sk], uc,
              u[c + sk], u[c - sk]);
          double lap = second(ix, u[c + 1], uc, u[c - 1]) +
                       second(iy, u[c + sj], uc, u[c - sj]) +
                       second(iz, u[c + sk], uc, u[c - sk]);
          f[c] = uc + dt * (iRe * lap - cx - cy - cz + gx);
        }
        /* G: y-momentum at the +y face */
        {
          double vc = v[c];
          double cx = donor(ix, gamma, u[c] + u[c + sj], u[c - 1] + u[c - 1 + sj], vc,
              v[c + 1], v[c - 1]);
          double cy = donor(iy, gamma, vc + v[c + sj], vc + v[c - sj], vc, v[c + sj], v[c - sj]);
          /* the reference's "minus" half uses V(i,j,k+1) where the textbook
           * stencil has V(i,j,k-1) (discretization.c:543-550); kept for parity */
          double cz = donor(iz, gamma, w[c] + w[c + sj], w[c - sk] + w[c + sj - sk], vc,
              v[c + sk], v[c + sk]);
          double lap = second(ix, v[c + 1], vc, v[c - 1]) +
                       second(iy, v[c + sj], vc, v[c - sj]) +
                       second(iz, v[c + sk], vc, v[c - sk]);
          gf[c] = vc + dt * (iRe * lap - cx - cy - cz + gy);
        }
        /* H: z-momentum at the +z face */
        {
          double wc = w[c];
          double cx = donor(ix, gamma, u[c] + u[c + sk], u[c - 1] + u[c - 1 + sk], wc,
              w[c + 1], w[c - 1]);
          double cy = donor(iy, gamma, v[c] + v[c + sk], v[c - sj + sk] + v[c - sj], wc,
              w[c + sj], w[c - sj]);
          double cz = donor(iz, gamma, wc + w[c + sk], wc + w[c - sk], wc, w[c + sk], w[c - sk]);
          double lap = second(ix, w[c + 1], wc, w[c - 1]) +
                       second(iy, w[c + sj], wc, w[c - sj]) +
                       second(iz, w[c + sk], wc, w[c - sk]);
          h[c] = wc + dt * (iRe * lap - cx - cy - cz + gz);
        }
      }
    }
  }
  /* wall faces carry the velocity itself (discretization.c:599-651) */
  for (int k = 1; k <= g->kmax; k++)
    for (int j = 1; j <= g->jmax; j++) {
      f[IX(g, 0, j, k)] = u[IX(g, 0, j, k)];
      f[IX(g, g->imax, j, k)] = u[IX(g, g->imax, j, k)];
    }
  for (int k = 1; k <= g->kmax; k++)
    for (int i = 1; i <= g->imax; i++) {
      gf[IX(g, i, 0, k)] = v[IX(g, i, 0, k)];
      gf[IX(g, i, g->jmax, k)] = v[IX(g, i, g->jmax, k)];
    }
  for (int j = 1; j <= g->jmax; j++)
    for (int i = 1; i <= g->imax; i++) {
      h[IX(g, i, j, 0)] = w[IX(g, i, j, 0)];
      h[IX(g, i, j, g->kmax)] = w[IX(g, i, j, g->kmax)];
    }
}

/* computeRHS, reference src/discretization.c:334-362 */
void or_compute_rhs(
    const OrGrid *g, double dt, const double *f, const double *gf, const double *h, double *rhs)
{
  const double ix = 1.0 / g->dx, iy = 1.0 / g->dy, iz = 1.0 / g->dz, it = 1.0 / dt;
  const size_t sj = (size_t)(g->imax + 2);
  const size_t sk = sj * (size_t)(g->jmax + 2);
  for (int k = 1; k <= g->kmax; k++)
    for (int j = 1; j <= g->jmax; j++)
      for (int i = 1; i <= g->imax; i++) {
        size_t c = IX(g, i, j, k);
        rhs[c] = ((f[c] - f[c - 1]) * ix + (gf[c] - gf[c - sj]) * iy + (h[c] - h[c - sk]) * iz) * it;
      }
}

/* normalizePressure, reference src/discretization.c:403-429; returns the mean */
double or_normalize_pressure(const OrGrid *g, double *p)
{
  double sum = 0.0;
  for (int k = 1; k <= g->kmax; k++)
    for (int j = 1; j <= g->jmax; j++)
      for (int i = 1; i <= g->imax; i++) sum += p[IX(g, i, j, k)];
  sum /= (g->imax * g->jmax * g->kmax);
  for (int k = 1; k <= g->kmax; k++)
    for (int j = 1; j <= g->jmax; j++)
      for (int i = 1; i <= g->imax; i++) p[IX(g, i, j, k)] = p[IX(g, i, j, k)] - sum;
  return sum;
}

/* adaptUV, reference src/discretization.c:654-681 */
void or_adapt_uv(const OrGrid *g, double dt, const double *f, const double *gf,
    const double *h, const double *p, double *u, double *v, double *w)
{
  const double fx = dt / g->dx, fy = dt / g->dy, fz = dt / g->dz;
  const size_t sj = (size_t)(g->imax + 2);
  const size_t sk = sj * (size_t)(g->jmax + 2);
  for (int k = 1; k <= g->kmax; k++)
    for (int j = 1; j <= g->jmax; j++)
      for (int i = 1; i <= g->imax; i++) {
        size_t c = IX(g, i, j, k);
        u[c] = f[c] - (p[c + 1] - p[c]) * fx;
        v[c] = gf[c] - (p[c + sj] - p[c]) * fy;
        w[c] = h[c] - (p[c + sk] - p[c]) * fz;
      }
}

/* SOR relaxation factor, reference src/solver-rb.c:46-47 */
static double sor_factor(const OrGrid *g, double omega)
{
  double dx2 = g->dx * g->dx, dy2 = g->dy * g->dy, dz2 = g->dz * g->dz;
  return omega * 0.5 * (dx2 * dy2 * dz2) / (dy2 * dz2 + dx2 * dz2 + dx2 * dy2);
}

/* residual of the 7-point Laplacian at padded index c (solver-rb.c:66-69) */
static inline double cell_residual(const double *p, const double *rhs, size_t c, size_t sj,
    size_t sk, double idx2, double idy2, double idz2)
{
  return rhs[c] - ((p[c + 1] - 2.0 * p[c] + p[c - 1]) * idx2 +
                      (p[c + sj] - 2.0 * p[c] + p[c - sj]) * idy2 +
                      (p[c + sk] - 2.0 * p[c] + p[c - sk]) * idz2);
}

/*
 * One colour pass. Colour 1 ("odd", the reference's pass 0) updates cells with
 * odd i+j+k, colour 0 the even ones (solver-rb.c:55-79). Cells of one colour
 * only read the other colour, so the update order inside a pass is free; the
 * residual sum keeps the reference's k, j, i order.
 * relax != 0: p -= factor*r; accumulate r^2 into *acc when acc != NULL;
 * store r into r_out (when non-NULL) instead of relaxing when relax == 0.
 */
static void colour_pass(const OrGrid *g, int odd, double factor, int relax, double *p,
    const double *rhs, double *acc, double *r_out)
{
  const double idx2 = 1.0 / (g->dx * g->dx), idy2 = 1.0 / (g->dy * g->dy),
               idz2 = 1.0 / (g->dz * g->dz);
  const size_t sj = (size_t)(g->imax + 2);
  const size_t sk = sj * (size_t)(g->jmax + 2);
  double s = acc ? *acc : 0.0;
  for (int k = 1; k <= g->kmax; k++)
    for (int j = 1; j <= g->jmax; j++) {
      int i0 = 1 + ((1 + j + k + odd) & 1); /* first i with (i+j+k)%2 == odd */
      for (int i = i0; i <= g->imax; i += 2) {
        size_t c = IX(g, i, j, k);
        double r = cell_residual(p, rhs, c, sj, sk, idx2, idy2, idz2);
        if (relax) p[c] -= (factor * r);
        if (r_out) r_out[c] = r;
        if (acc) s += (r * r);
      }
    }
  if (acc) *acc = s;
}

/* Neumann ghost copy on the six faces, no edges or corners
 * (reference src/solver-rb.c:129-148, src/solver-mg.c:153-174) */
void or_pressure_ghosts(const OrGrid *g, double *p)
{
  for (int j = 1; j <= g->jmax; j++)
    for (int i = 1; i <= g->imax; i++) {
      p[IX(g, i, j, 0)] = p[IX(g, i, j, 1)];
      p[IX(g, i, j, g->kmax + 1)] = p[IX(g, i, j, g->kmax)];
    }
  for (int k = 1; k <= g->kmax; k++)
    for (int i = 1; i <= g->imax; i++) {
      p[IX(g, i, 0, k)] = p[IX(g, i, 1, k)];
      p[IX(g, i, g->jmax + 1, k)] = p[IX(g, i, g->jmax, k)];
    }
  for (int k = 1; k <= g->kmax; k++)
    for (int j = 1; j <= g->jmax; j++) {
      p[IX(g, 0, j, k)] = p[IX(g, 1, j, k)];
      p[IX(g, g->imax + 1, j, k)] = p[IX(g, g->imax, j, k)];
    }
}

/*
 * solve (red-black SOR), reference src/solver-rb.c:27-172.
 * The mean-square residual is carried between iterations without a reset:
 * res starts at 1 and each iteration sets res = (res + sum r^2) / N.
 */
int or_solve_rb(const OrGrid *g, double eps, double omega, int itermax, double *p,
    const double *rhs, double *res_out)
{
  const double factor = sor_factor(g, omega);
  const double epssq = eps * eps;
  const double ncell = (double)(g->imax * g->jmax * g->kmax);
  double res = 1.0;
  int it = 0;
  while ((res >= epssq) && (it < itermax)) {
    colour_pass(g, 1, factor, 1, p, rhs, &res, NULL);
    colour_pass(g, 0, factor, 1, p, rhs, &res, NULL);
    or_pressure_ghosts(g, p);
    res = res / ncell;
    it++;
  }
  if (res_out) *res_out = res;
  return it;
}

/* smooth, reference src/solver-mg.c:177-224: one SOR sweep, no residual */
void or_sor_sweep(const OrGrid *g, double omega, double *p, const double *rhs)
{
  const double factor = sor_factor(g, omega);
  colour_pass(g, 1, factor, 1, p, rhs, NULL, NULL);
  colour_pass(g, 0, factor, 1, p, rhs, NULL, NULL);
}

/* calculateResidual at the finest level, reference src/solver-mg.c:226-289 */
static double mg_ref_residual(const OrGrid *g, const double *p, const double *rhs)
{
  double res = 1.0;
  colour_pass(g, 1, 0.0, 0, (double *)p, rhs, &res, NULL);
  colour_pass(g, 0, 0.0, 0, (double *)p, rhs, &res, NULL);
  return res / (double)(g->imax * g->jmax * g->kmax);
}

/*
 * The reference multigrid solve as it behaves in the sequential build
 * (src/solver-mg.c:299-402). Its coarse-grid correction never reaches the
 * fine pressure: prolongate() writes into r[level] while correct() adds
 * e[0], which nothing writes and stays zero. What remains observable is
 * presmooth x (sweep + ghost copy), the mean-square residual (returned),
 * a ghost copy, then postsmooth x (sweep + ghost copy). With levels == 1, or a
 * grid thinner than two cells, the finest level is the coarsest: presmooth
 * sweeps without ghost copies, then the residual.
 */
double or_solve_mg_ref(const OrGrid *g, double omega, int levels, int presmooth,
    int postsmooth, double *p, const double *rhs)
{
  if (levels - 1 == 0 || g->imax < 2 || g->jmax < 2 || g->kmax < 2) {
    for (int s = 0; s < presmooth; s++) or_sor_sweep(g, omega, p, rhs);
    return mg_ref_residual(g, p, rhs);
  }
  for (int s = 0; s < presmooth; s++) {
    or_sor_sweep(g, omega, p, rhs);
    or_pressure_ghosts(g, p);
  }
  double res = mg_ref_residual(g, p, rhs);
  or_pressure_ghosts(g, p);
  for (int s = 0; s < postsmooth; s++) {
    or_sor_sweep(g, omega, p, rhs);
    or_pressure_ghosts(g, p);
  }
  return res;
}

/* ---- whole-run driver (reference src/main.c:53-88) ---- */

int or_state_init(OrState *s, const OrCase *c)
{
  memset(s, 0, sizeof(*s));
  s->c = *c;
  s->g.imax = c->imax;
  s->g.jmax = c->jmax;
  s->g.kmax = c->kmax;
  /* initDiscretization, reference src/discretization.c:49-117 */
  s->g.dx = c->xlength / c->imax;
  s->g.dy = c->ylength / c->jmax;
  s->g.dz = c->zlength / c->kmax;
  size_t n = or_padded_size(&s->g);
  double **fields[8] = { &s->u, &s->v, &s->w, &s->p, &s->rhs, &s->f, &s->gf, &s->h };
  for (int q = 0; q < 8; q++) {
    *fields[q] = (double *)malloc(n * sizeof(double));
    if (!*fields[q]) return -1;
  }
  for (size_t q = 0; q < n; q++) {
    s->u[q] = c->u_init;
    s->v[q] = c->v_init;
    s->w[q] = c->w_init;
    s->p[q] = c->p_init;
    s->rhs[q] = s->f[q] = s->gf[q] = s->h[q] = 0.0;
  }
  double dx = s->g.dx, dy = s->g.dy, dz = s->g.dz;
  double invSqrSum = 1.0 / (dx * dx) + 1.0 / (dy * dy) + 1.0 / (dz * dz);
  s->dtBound = 0.5 * c->re * 1.0 / invSqrSum;
  s->dt = c->dt0;
  s->t = 0.0;
  s->nt = 0;
  return 0;
}

void or_state_free(OrState *s)
{
  double *fields[8] = { s->u, s->v, s->w, s->p, s->rhs, s->f, s->gf, s->h };
  for (int q = 0; q < 8; q++) free(fields[q]);
  memset(s, 0, sizeof(*s));
}

int or_state_step(OrState *s, double *res_out)
{
  const OrGrid *g = &s->g;
  const OrCase *c = &s->c;
  size_t n = or_padded_size(g);
  if (c->tau > 0.0) {
    s->dt = or_timestep(s->dtBound, g->dx, g->dy, g->dz, or_max_abs(s->u, n),
        or_max_abs(s->v, n), or_max_abs(s->w, n), c->tau);
  }
  or_set_bc(g, c->bc, s->u, s->v, s->w);
  or_special_bc(g, c->problem, c->lid, c->inflow, s->u);
  or_compute_fgh(g, c->re, c->gamma, c->gx, c->gy, c->gz, s->dt, s->u, s->v, s->w, s->f,
      s->gf, s->h);
  or_compute_rhs(g, s->dt, s->f, s->gf, s->h, s->rhs);
  if (s->nt % 100 == 0) or_normalize_pressure(g, s->p);
  double res = 0.0;
  int it = 0;
  if (c->solver == 0)
    it = or_solve_rb(g, c->eps, c->omega, c->itermax, s->p, s->rhs, &res);
  else if (c->solver == 1)
    res = or_solve_mg_ref(g, c->omega, c->levels, c->presmooth, c->postsmooth, s->p, s->rhs);
  else
    it = or_mg_solve(g, c->solver - 2, c->mg_levels, c->mg_pre, c->mg_post, c->mg_coarse,
        c->mg_inner, c->mg_cycles, c->rtol, s->p, s->rhs, &res);
  or_adapt_uv(g, s->dt, s->f, s->gf, s->h, s->p, s->u, s->v, s->w);
  s->t += s->dt;
  s->nt++;
  if (res_out) *res_out = res;
  return it;
}
