// Solver-side internal declarations (not part of the C ABI).
#pragma once

#include "df32.cuh"
#include "nusif_internal.h"

namespace nusif {

// Convergence state of one solve, kept in device memory and mirrored in
// pinned host memory.
struct SolveState {
  double res;     // carried mean-square residual (rb) / residual (mg-ref)
  double epssq;   // eps^2
  double ncell;   // imax*jmax*kmax
  int it;         // iterations done
  int itermax;
  int done;       // set by the device when the loop condition fails
  int pad;
};

struct SorArgs {
  Dims g;
  double idx2, idy2, idz2, diag, factor;
  // the same constants as pairs of FP32 numbers (df32.cuh), formed on the
  // host: GB300 runs double <-> float conversions on its FP64 pipe
  df::f2 pidx2, pidy2, pidz2, pmdiag, pmfactor;
  int kb;  // k planes per block
};

SorArgs make_sor_args(const Dims &g, double dx, double dy, double dz, double omega);
dim3 sor_grid(const SorArgs &A);
int sor_blocks(const SorArgs &A);
// df: the SOR residual in double-float arithmetic (key arith df32)
bool launch_rb_iteration(const SorArgs &A, double *p, const double *rhs, SolveState *st,
    ReduceScratch &red, bool df = false);
bool launch_sor_sweep(const SorArgs &A, double *p, const double *rhs, bool ghosts);
bool launch_residual_ref(const SorArgs &A, const double *p, const double *rhs, SolveState *st,
    ReduceScratch &red);
bool launch_pressure_ghosts(const Dims &g, double *p);

struct MgHierarchy;  // multigrid.cu

struct SolverState {
  int kind = SOLVER_RB;
  Extras ext;
  SolveState *d_state = nullptr;
  SolveState *h_state = nullptr;  // pinned
  ReduceScratch red;
  int last_iterations = 0;
  MgHierarchy *mg = nullptr;
  struct GuessState *guess = nullptr;  // learned warm start (guess.cu)
};

SolverState *solver_state(const Solver *s);

bool mg_setup(Solver *s, Discretization *d, SolverState *ss);
double mg_solve(Solver *s, SolverState *ss, double *p, const double *rhs);
void mg_free(Solver *s, SolverState *ss);
bool mg_time_kernel(SolverState *ss, const double *p, const double *rhs, int which, int reps,
    double *ms_out);
bool mg_enqueue(SolverState *ss, double *p, const double *rhs, int queue, int *unconverged,
    int *last_cycles);
bool mg_enqueue_loop(SolverState *ss, double *p, const double *rhs, cudaStream_t body,
    int *unconverged, int *last_cycles);
bool mg_capture_ok(const SolverState *ss);

}  // namespace nusif
