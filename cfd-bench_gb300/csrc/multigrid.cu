// Geometric multigrid V-cycle solvers (kinds mg and mg-mixed).
#include "solver_internal.h"

namespace nusif {

struct MgHierarchy {
  int levels = 0;
};

bool mg_setup(Solver *s, Discretization *d, SolverState *ss)
{
  (void)s;
  (void)d;
  (void)ss;
  fail(NUSIF_ERR_ARG, "solver kinds mg and mg-mixed are not available in this build");
  return false;
}

double mg_solve(Solver *s, SolverState *ss, double *p, const double *rhs)
{
  (void)s;
  (void)ss;
  (void)p;
  (void)rhs;
  fail(NUSIF_ERR_STATE, "mg solve without a hierarchy");
  return 0.0;
}

void mg_free(Solver *s, SolverState *ss)
{
  (void)s;
  delete ss->mg;
  ss->mg = nullptr;
}

}  // namespace nusif
