// Internal declarations of the GB300 NuSiF library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "nusif_gb300.h"

namespace nusif {

// ---- error handling (runtime.cpp) ----
void fail(int code, const char *fmt, ...);  // records or exits per error mode
bool cuda_ok(cudaError_t e, const char *what);  // false after recording a failure
bool has_error();                              // an error is pending (record mode)
cudaStream_t stream();
// asynchronous field copies (runtime.cpp): make the launch stream wait for the
// queued copies of these device arrays (before work that writes them) / for
// their queued uploads only (before work that only reads them) / of every
// array / of d's eight fields
bool await_copies(const void *const *ptrs, int n);
bool await_uploads(const void *const *ptrs, int n);
bool await_all_copies();
bool await_fields(const Discretization *d);
// after every kernel launch: counts it and checks the launch error
bool launched(const char *what);
unsigned long long launch_count();
void set_launch_count(unsigned long long n);

// ---- problem kinds and solver kinds ----
enum Problem { PROBLEM_NONE = 0, PROBLEM_DCAVITY = 1, PROBLEM_CANAL = 2 };
enum SolverKind { SOLVER_RB = 0, SOLVER_MG_REF = 1, SOLVER_MG = 2, SOLVER_MG_MIXED = 3 };

// Extension settings carried beside a Parameter (keys this library adds).
struct Extras {
  int solver = -1;          // -1: not set (environment, then rb)
  double lid = 1.0;         // dcavity lid speed (reference hard-codes 1)
  double inflow = 2.0;      // canal inflow speed (reference hard-codes 2.0)
  double rtol = 1e-6;       // relative residual target of the V-cycle solvers
  int mg_levels = 0;        // 0: halve an axis while it is even and >= 16
  int mg_pre = 2, mg_post = 2;
  int mg_coarse_sweeps = 0;  // 0: exact coarsest solve (<= 1024 cells), else sweeps
  int mg_inner = 4;          // mg-mixed: most FP32 V-cycles per FP64 residual
  double mg_theta = 0.9;     // mg-mixed: FP32 correction target, a fraction of rtol
  double mg_omega = 1.0;     // relaxation of the multigrid red-black smoother (1: Gauss-Seidel)
  int mg_guess = 0;          // initial guess: 0 previous p, 1 linear, 2 quadratic, 3 cubic
                             // extrapolation in time
  int mg_graph = 1;          // 1: each solve is one CUDA graph launch (while-loops on the device)
  int mg_tail = 0;           // levels of at most this many cells run as one kernel (0: off)
  int mg_chunk = 0;          // planes per block of the FP32 one-kernel sweep (0: autotuned)
  int host_fields = 0;       // 1: fields in managed memory (host-readable pointers)
  int mg_guess_probe = 1;    // key mg_probe: learned guess every P-th step after 2 rejections
  int mg_maxcycles = 100;
  int fg_fp64 = 0;           // key fg_arith: computeFG in FP64 instructions (fp64) or FP32 pairs (df32)
  int arith_fp64 = 0;        // key arith: every FP64-bound stencil in FP64 instructions (fp64)
                             // or FP32 pairs (df32); also sets fg_arith
  int fuse_dt = 0;           // key fuse_dt: adaptUV keeps the maxima of the velocities it writes
                             // and the next computeTimestep reads only the ghost shell
};
Extras *extras_for(const Parameter *p, bool create);

// Grid geometry shared by all kernels.
struct Dims {
  int imax, jmax, kmax;
  int sj, sk;      // strides of j and k in the padded layout
  int64_t padded;  // (imax+2)(jmax+2)(kmax+2)
};
inline Dims make_dims(int imax, int jmax, int kmax)
{
  Dims d;
  d.imax = imax;
  d.jmax = jmax;
  d.kmax = kmax;
  d.sj = imax + 2;
  d.sk = (imax + 2) * (jmax + 2);
  d.padded = (int64_t)(imax + 2) * (jmax + 2) * (kmax + 2);
  return d;
}

// Reduction scratch: per-block partials plus a ticket counter, so that the
// last block to finish folds the partials in a fixed order (deterministic,
// no spin-waits).
struct ReduceScratch {
  double *partials = nullptr;   // device
  unsigned *ticket = nullptr;   // device, returns to 0 after every use
  int capacity = 0;
};
bool reduce_scratch_alloc(ReduceScratch &r, int capacity);
void reduce_scratch_free(ReduceScratch &r);

// Scalars of one time step kept in device memory, so that a step can run
// without a host round trip (graph-captured batched steps). Same expressions
// as the host path: dt (computeTimestep), 1/dt (computeRHS), dt/h (adaptUV).
struct StepScalars {
  double dt, idt, fx, fy, fz;
  double rx, ry, rz;  // (1/dx)(1/dt), (1/dy)(1/dt), (1/dz)(1/dt): computeRHS factors
  double t;  // simulated time after the last completed step
  int nt;    // completed steps
  int pad;
};

// Device state of one Discretization (kept beside the reference struct).
// fuse_dt: per-slot maxima of |u|, |v|, |w| (bit patterns of non-negative
// doubles) that adaptUV accumulates, and what they hold
constexpr int kAmaxSlots = 1024;
enum AmaxState { kAmaxReset = 0, kAmaxValid = 1, kAmaxDirty = 2 };

struct DiscState {
  Dims dims;
  int problem = PROBLEM_NONE;
  Extras ext;
  ReduceScratch red;
  double *d_scalars = nullptr;  // device: [0..2] max |u|,|v|,|w|, [3] sum p
  double *h_scalars = nullptr;  // pinned host mirror
  // fuse_dt: kAmaxReset, the slots are zero; kAmaxValid, they hold the
  // interior maxima of exactly the last adaptUV and nothing wrote u, v, w
  // since; kAmaxDirty, anything else
  unsigned long long *d_amax = nullptr;  // [kAmaxSlots][3]
  int amax = kAmaxReset;
  long long dt_shell = 0, dt_full = 0;  // computeTimestep calls by path
};
// u, v or w changed other than by adaptUV: the kept maxima no longer hold
inline void velocity_written(DiscState *st)
{
  if (st && st->amax == kAmaxValid) st->amax = kAmaxDirty;
}
DiscState *disc_state(const Discretization *d);

// ---- kernels launched by the discretization entry points (discretization.cu) ----
bool launch_max3(const Dims &g, const double *u, const double *v, const double *w,
    ReduceScratch &red, double *d_out3);
bool launch_bc(const Dims &g, const int bc[6], int problem, double lid, double inflow,
    double *u, double *v, double *w);
bool launch_fgh(const Dims &g, double re, double gamma, double gx, double gy, double gz,
    double dt, double dx, double dy, double dz, const double *u, const double *v,
    const double *w, double *f, double *gg, double *h, const StepScalars *sp = nullptr,
    int kb_fixed = 0, bool fp64 = false);
bool launch_rhs(const Dims &g, double dt, double dx, double dy, double dz, const double *f,
    const double *gg, const double *h, double *rhs, const StepScalars *sp = nullptr);
bool launch_interior_sum(const Dims &g, const double *p, ReduceScratch &red, double *d_out);
bool launch_subtract_mean(const Dims &g, double *p, const double *d_mean);
bool launch_adapt_uv(const Dims &g, double dt, double dx, double dy, double dz,
    const double *f, const double *gg, const double *h, const double *p, double *u, double *v,
    double *w, const StepScalars *sp = nullptr, unsigned long long *amax_slots = nullptr);
bool launch_shell_max3(const Dims &g, const double *u, const double *v, const double *w,
    unsigned long long *amax_slots, ReduceScratch &red, double *d_out3);
bool launch_special(const Dims &g, int problem, double lid, double inflow, double *u);
int problem_code(const char *name);

}  // namespace nusif
