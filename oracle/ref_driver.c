/*
 * Driver around the reference NuSiF sources, compiled from source by
 * oracle/build_ref.sh into oracle/_ref/ -- TEST INFRASTRUCTURE ONLY.
 *
 * It mirrors the reference time loop (src/main.c:53-88) one step per call and
 * exposes the reference's field arrays, so tests can pin the CPU oracle
 * (oracle/nusif_oracle.c) and generate golden vectors. The reference objects
 * are compiled with -fvisibility=hidden; only the refdrv_* symbols below are
 * exported. The reference prints the red-black iteration count only under
 * VERBOSE ("Solver took %d iterations", src/solver-rb.c:165); the recipe
 * renames printf in the reference objects to refdrv_printf, which records it.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "comm.h"
#include "discretization.h"
#include "parameter.h"
#include "solver.h"

#define EXPORT __attribute__((visibility("default")))

static Parameter g_param;
static Discretization g_d;
static Solver g_s;
static int g_ready = 0;
static int g_last_it = -1;
static int g_echo = 0;
static double g_t = 0.0;
static int g_nt = 0;

/* printf replacement for the reference objects: records the RB iteration count */
EXPORT int refdrv_printf(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  if (strncmp(fmt, "Solver took %d", 14) == 0) {
    va_list aq;
    va_copy(aq, ap);
    g_last_it = va_arg(aq, int);
    va_end(aq);
  }
  int n = 0;
  if (g_echo) n = vprintf(fmt, ap);
  va_end(ap);
  return n;
}

EXPORT void refdrv_set_echo(int on) { g_echo = on; }

/* parse a .par file with the reference parser (src/parameter.c:13-98) */
EXPORT int refdrv_read_parameter(const char *path, Parameter *out)
{
  initParameter(out);
  readParameter(out, path);
  return 0;
}

EXPORT int refdrv_sizeof_parameter(void) { return (int)sizeof(Parameter); }

EXPORT int refdrv_init(const char *parfile)
{
  memset(&g_param, 0, sizeof(g_param));
  memset(&g_d, 0, sizeof(g_d));
  memset(&g_s, 0, sizeof(g_s));
  commInit(&g_d.comm, 0, NULL);
  initParameter(&g_param);
  readParameter(&g_param, parfile);
  commPartition(&g_d.comm, g_param.kmax, g_param.jmax, g_param.imax);
  initDiscretization(&g_d, &g_param);
  initSolver(&g_s, &g_d, &g_param);
  g_t = 0.0;
  g_nt = 0;
  g_ready = 1;
  return 0;
}

/* one pass of the reference time-loop body (src/main.c:61-79) */
EXPORT int refdrv_step(double *res_out, int *it_out, double *dt_out, double *t_out)
{
  if (!g_ready) return -1;
  g_last_it = -1;
  if (g_d.tau > 0.0) computeTimestep(&g_d);
  setBoundaryConditions(&g_d);
  setSpecialBoundaryCondition(&g_d);
  computeFG(&g_d);
  computeRHS(&g_d);
  if (g_nt % 100 == 0) normalizePressure(&g_d);
  double res = solve(&g_s, g_d.p, g_d.rhs);
  adaptUV(&g_d);
  g_t += g_d.dt;
  g_nt++;
  if (res_out) *res_out = res;
  if (it_out) *it_out = g_last_it;
  if (dt_out) *dt_out = g_d.dt;
  if (t_out) *t_out = g_t;
  return 0;
}

EXPORT double refdrv_time(void) { return g_t; }
EXPORT double refdrv_te(void) { return g_d.te; }
EXPORT double refdrv_dt(void) { return g_d.dt; }
EXPORT void refdrv_set_dt(double dt) { g_d.dt = dt; }
EXPORT double refdrv_dtbound(void) { return g_d.dtBound; }
EXPORT void refdrv_dims(int *dims)
{
  dims[0] = g_d.grid.imax;
  dims[1] = g_d.grid.jmax;
  dims[2] = g_d.grid.kmax;
}

/* field by index: 0 u, 1 v, 2 w, 3 p, 4 rhs, 5 f, 6 g, 7 h */
EXPORT double *refdrv_field(int which)
{
  double *f[8] = { g_d.u, g_d.v, g_d.w, g_d.p, g_d.rhs, g_d.f, g_d.g, g_d.h };
  return (which >= 0 && which < 8) ? f[which] : NULL;
}

/* single reference operators on the current state (per-kernel pin tests) */
EXPORT void refdrv_compute_timestep(void) { computeTimestep(&g_d); }
EXPORT void refdrv_set_bc(void) { setBoundaryConditions(&g_d); }
EXPORT void refdrv_special_bc(void) { setSpecialBoundaryCondition(&g_d); }
EXPORT void refdrv_compute_fg(void) { computeFG(&g_d); }
EXPORT void refdrv_compute_rhs(void) { computeRHS(&g_d); }
EXPORT void refdrv_normalize(void) { normalizePressure(&g_d); }
EXPORT void refdrv_adapt_uv(void) { adaptUV(&g_d); }
EXPORT double refdrv_solve(int *it_out)
{
  g_last_it = -1;
  double res = solve(&g_s, g_d.p, g_d.rhs);
  if (it_out) *it_out = g_last_it;
  return res;
}
