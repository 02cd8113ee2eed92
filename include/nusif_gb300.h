/*
 * nusif_gb300.h -- C ABI of the GB300 (sm_103a) NuSiF hot-path library.
 *
 * The library replaces the reference objects parameter.o, discretization.o
 * and solver-{rb,mg}.o of HPC-Dwarfs/CFD-Bench ("NuSiF", src/). The entry
 * points below have the reference names, signatures, argument meaning and
 * error behaviour; the structs have the reference member order and types, so
 * an unchanged src/main.c links against the library: link main.o and the
 * reference's remaining objects (comm.o, allocate.o, timing.o, progress.o,
 * profiler.o, vtkWriter-seq.o) with -L<lib dir> -lnusif_gb300 -lcudart -lstdc++
 * in place of parameter.o, discretization.o and solver-*.o.
 *
 * Differences a caller must know:
 *  - The field pointers in Discretization (p, rhs, f, g, h, u, v, w) are
 *    DEVICE pointers to FP64 arrays in the reference layout
 *    ((imax+2)(jmax+2)(kmax+2) doubles, i fastest, one ghost layer;
 *    src/util.h:19-34). Read them on the host with nusifDownloadField().
 *  - All scalar time-step logic (dt, dtBound, t) stays on the host in the
 *    reference's own expressions.
 *  - Errors: by default a failing call prints to stderr and exits with
 *    EXIT_FAILURE, as the reference does (src/allocate.c:18-31,
 *    src/parameter.c:38-41). nusifSetErrorMode(NUSIF_ERRORS_RECORD) makes
 *    calls return instead and report through nusifGetLastError().
 *  - Single host thread, no reentrancy (as the reference).
 */
#ifndef NUSIF_GB300_H
#define NUSIF_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define NUSIF_API __attribute__((visibility("default")))
#else
#define NUSIF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference types (layouts identical to the sequential reference build) ---- */

/* src/grid.h:8-12 */
typedef struct {
  double dx, dy, dz;
  int imax, jmax, kmax;
  double xlength, ylength, zlength;
} Grid;

/* src/comm.h:33-44, sequential build (no MPI members) */
typedef struct {
  int rank;
  int size;
  int neighbours[6];
  int coords[3], dims[3];
  int imaxLocal, jmaxLocal, kmaxLocal;
} CommType;

/* src/parameter.h:8-19 */
typedef struct {
  int imax, jmax, kmax;
  double xlength, ylength, zlength;
  int itermax;
  double eps, omg;
  double re, tau, gamma;
  double te, dt;
  double gx, gy, gz;
  char *name;
  int bcLeft, bcRight, bcBottom, bcTop, bcFront, bcBack;
  double u_init, v_init, w_init, p_init;
  int levels, presmooth, postsmooth;
} Parameter;

/* src/discretization.h:12 */
enum BC { NOSLIP = 1, SLIP, OUTFLOW, PERIODIC };

/* src/discretization.h:14-32; field pointers are device pointers */
typedef struct {
  Grid grid;
  double *p, *rhs;
  double *f, *g, *h;
  double *u, *v, *w;
  double eps, omega;
  double re, tau, gamma;
  double gx, gy, gz;
  int itermax;
  double dt, te;
  double dtBound;
  char *problem;
  int bcLeft, bcRight, bcBottom, bcTop, bcFront, bcBack;
  CommType comm;
} Discretization;

/* src/solver.h:12-33 */
typedef struct {
  Grid *grid;
  double *p, *rhs;
  double *f, *g, *h;
  double *u, *v, *w;
  double eps, omega;
  double re, tau, gamma;
  double gx, gy, gz;
  int itermax;
  double dt, te;
  double dtBound;
  char *problem;
  int bcLeft, bcRight, bcBottom, bcTop, bcFront, bcBack;
  double **r, **e;
  int levels, presmooth, postsmooth;
  CommType *comm;
} Solver;

/* ---- reference entry points ---- */

/* src/parameter.h:22-24 (parameter.c:13-30, 32-98, 100-131). Same parsing
 * rules: text after '#' dropped, split on spaces only, keys matched by prefix
 * of the key's length, atoi/atof/strdup. Extra keys of this library (solver,
 * lid, inflow, rtol, mg_*) are stored beside the struct, keyed by its address. */
NUSIF_API void initParameter(Parameter *param);
NUSIF_API void readParameter(Parameter *param, const char *filename);
NUSIF_API void printParameter(Parameter *param);

/* src/discretization.h:34-41 */
NUSIF_API void initDiscretization(Discretization *d, Parameter *params); /* discretization.c:49-117 */
NUSIF_API void computeTimestep(Discretization *d);                       /* discretization.c:431-453 */
NUSIF_API void setBoundaryConditions(Discretization *d);                 /* discretization.c:119-332 */
NUSIF_API void setSpecialBoundaryCondition(Discretization *d);           /* discretization.c:364-389 */
NUSIF_API void computeFG(Discretization *d);                             /* discretization.c:455-652 */
NUSIF_API void computeRHS(Discretization *d);                            /* discretization.c:334-362 */
NUSIF_API void normalizePressure(Discretization *d);                     /* discretization.c:403-429 */
NUSIF_API void adaptUV(Discretization *d);                               /* discretization.c:654-681 */

/* src/solver.h:35-36. The solver kind is chosen at run time (the reference
 * picks solver-rb.o or solver-mg.o at link time, Makefile:19-21): the .par key
 * "solver" (rb | mg-ref | mg | mg-mixed), else the environment variable
 * NUSIF_SOLVER, else rb.
 *   rb       red-black SOR, solver-rb.c:27-172 (residual recurrence kept)
 *   mg-ref   the reference multigrid as it behaves, solver-mg.c:299-402
 *   mg       FP64 geometric V-cycles (full weighting, trilinear prolongation,
 *            red-black Gauss-Seidel) to a relative residual (key rtol)
 *   mg-mixed FP32 V-cycles inside FP64 iterative refinement, same stopping rule
 * solve() returns what the reference returns: the mean-square residual
 * (rb, mg-ref) or, for mg and mg-mixed, the final relative residual. */
NUSIF_API void initSolver(Solver *s, Discretization *d, Parameter *p); /* solver-rb.c:17-25, solver-mg.c:356-389 */
NUSIF_API double solve(Solver *s, double *p, const double *rhs);     /* solver-rb.c:27-172, solver-mg.c:391-402 */

/* ---- extensions (no reference counterpart) ---- */

enum { NUSIF_ERRORS_EXIT = 0, NUSIF_ERRORS_RECORD = 1 };
enum { NUSIF_OK = 0, NUSIF_ERR_CUDA = 1, NUSIF_ERR_ARG = 2, NUSIF_ERR_IO = 3,
       NUSIF_ERR_STATE = 4, NUSIF_ERR_DEVICE = 5 };
/* field selectors for upload/download */
enum { NUSIF_U = 0, NUSIF_V, NUSIF_W, NUSIF_P, NUSIF_RHS, NUSIF_F, NUSIF_G, NUSIF_H };

NUSIF_API void nusifSetErrorMode(int mode);
/* last error code (0 = none) and message; clears it */
NUSIF_API int nusifGetLastError(char *msg, int len);
/* CUDA stream (cudaStream_t) every later call launches on; NULL = legacy default stream */
NUSIF_API void nusifSetStream(void *stream);
NUSIF_API void *nusifGetStream(void);
/* copies between a host array of (imax+2)(jmax+2)(kmax+2) doubles and a field */
NUSIF_API int nusifDownloadField(const Discretization *d, int which, double *host);
NUSIF_API int nusifUploadField(Discretization *d, int which, const double *host);
/* The same copies queued asynchronously (no counterpart in the reference,
 * whose fields live in host memory): each runs on a copy stream of the
 * library after the work already queued on the launch stream, and the first
 * later call that uses the field (or solve() with it as p or rhs) waits for it
 * on the device, not on the host -- a call that writes the field for every
 * queued copy of it, a call that only reads it for its queued uploads only --
 * so an upload of p overlaps computeTimestep .. computeRHS, which do not read
 * p, and a download of p queued after solve() overlaps adaptUV, which only
 * reads it. The host array
 * must stay untouched, and a downloaded one unread, until nusifWaitCopies()
 * returns; pinned host memory makes the copies asynchronous. Entry points
 * that take bare device pointers and the batch API do not wait per field:
 * call nusifWaitCopies() before them (nusifBatchStep does). */
NUSIF_API int nusifUploadFieldAsync(Discretization *d, int which, const double *host);
NUSIF_API int nusifDownloadFieldAsync(const Discretization *d, int which, double *host);
/* blocks until every queued asynchronous field copy has finished */
NUSIF_API int nusifWaitCopies(void);
/* iteration count of the last solve() (the reference prints it under VERBOSE,
 * solver-rb.c:163-166); V-cycles for mg and mg-mixed */
NUSIF_API int nusifSolverIterations(const Solver *s);
/* set an extension key on a Parameter, as a .par line "key value" would */
NUSIF_API int nusifParameterSet(Parameter *param, const char *key, const char *value);
/* release device memory of a discretization / solver (the reference never frees) */
NUSIF_API void nusifFreeDiscretization(Discretization *d);
NUSIF_API void nusifFreeSolver(Solver *s);
/* Red-black SOR solve that allocates no memory. No counterpart in the
 * reference. Same result as solve() with the rb solver and the key arith fp64
 * (the residual in FP64 instructions, as here) on the same p, rhs (device
 * arrays in the padded layout) and parameters, for callers that cannot
 * call cudaMalloc (hosts that hand out only pre-sized device buffers, runtimes
 * that reserve all device memory at start-up). Its scratch is a fixed
 * 256.5 KiB __device__ array of the library: grids needing more than 32768
 * per-block partial sums (larger than about 512^3 cells) are rejected with
 * NUSIF_ERR_ARG. The first call on a device looks up that array's address and
 * should come before any stream capture; do not reset the device between
 * calls. Like solve(), it synchronises the library's stream after every chunk
 * of iterations. Calls share the array: calls that overlap on the GPU race.
 * Returns a NUSIF_* code; *res_out and *it_out get solve()'s residual and
 * iterations. */
NUSIF_API int nusifSolveRBStatic(double *p, const double *rhs, int imax, int jmax, int kmax,
    double dx, double dy, double dz, double omega, double eps, int itermax, double *res_out,
    int *it_out);
/* Result collection, replaces commCollectResult (reference src/comm.c:327-477,
 * sequential path): cell-centred u, v, w (face averages) and interior p as
 * host arrays of imax*jmax*kmax doubles, i fastest. */
NUSIF_API int nusifCollectResult(const Discretization *d, double *ug, double *vg, double *wg,
    double *pg);
/* The reference's VTK output (src/vtkWriter-seq.c:12-146, called from
 * src/main.c:135-141): STRUCTURED_POINTS with "pressure" and "velocity";
 * binary = 0 writes ASCII "%f" (the reference's default), 1 big-endian doubles. */
NUSIF_API int nusifWriteVTK(const Discretization *d, const char *path, int binary);
/* Batched instances (no reference counterpart: the reference runs one case per
 * process). Each parameter file is one independent case (uneven grids welcome)
 * with the mg or mg-mixed solver (even mg_pre / mg_post). One time step of
 * every instance is captured as one CUDA graph (device-side dt; the multigrid
 * solve a graph while-loop that stops at rtol like the host-driven solve, or
 * with queue > 0 a fixed `queue` device-gated units per step); tune != 0
 * times the F/G/H tile depth per instance first. Returns NULL on error. */
typedef struct NusifBatch NusifBatch;
NUSIF_API NusifBatch *nusifBatchCreate(int n, const char *const *parfiles, int queue, int tune);
/* advance every instance by `steps` time steps (one graph launch each) */
NUSIF_API int nusifBatchStep(NusifBatch *b, int steps);
NUSIF_API int nusifBatchSize(const NusifBatch *b);
/* the instance's Discretization / Solver, for nusifDownloadField and friends */
NUSIF_API int nusifBatchInstance(NusifBatch *b, int idx, Discretization **d, Solver **s);
/* per instance: time, last dt, steps, V-cycles of the last step, steps that
 * ended above rtol (fixed queue too short, or mg_cycles reached), autotuned
 * F/G/H planes per block */
NUSIF_API int nusifBatchStats(NusifBatch *b, int idx, double *t, double *dt, int *nt, int *cycles,
    int *unconverged, int *fg_planes);
NUSIF_API void nusifBatchFree(NusifBatch *b);
/* kernels this library launched since it was loaded (observability) */
NUSIF_API unsigned long long nusifLaunchCount(void);
/* computeTimestep calls on d that read only the ghost shell (key fuse_dt 1:
 * the interior maxima came with the preceding adaptUV) and that read the
 * whole arrays (observability) */
NUSIF_API int nusifTimestepCounts(const Discretization *d, long long *shell, long long *full);
/* Measurement hook (mg and mg-mixed solvers): average duration in ms of `reps`
 * launches of one fine-level kernel, timed with CUDA events on the library
 * stream; which = 0 the fine smoother (mg-mixed: one whole FP32 red-black
 * sweep; mg: one colour pass of the FP64 smoother), 1 the FP64 residual of
 * mg-mixed, 2 + l one FP32 V-cycle of mg-mixed from level l (0 = finest)
 * down, from zero on that level's right-hand side of the last solve, replayed
 * as a captured CUDA graph.
 * Works on scratch copies: p and rhs are only read. */
NUSIF_API int nusifTimeKernel(Solver *s, const double *p, const double *rhs, int which, int reps,
    double *ms_out);
/* library version string */
NUSIF_API const char *nusifVersion(void);
/* `sweeps` exact red-black Gauss-Seidel sweeps of the mixed-precision
 * multigrid's FP32 smoother (one kernel per sweep) on compact device arrays
 * x, b [nz][ny][nx] (nx a multiple of 4) -> xout: ghost-free Neumann
 * operator with spacings hx, hy, hz; first colour (i + j + k) even, 0-based.
 * x may be NULL: the sweeps start from x = 0 (as the first pre-sweep of every
 * V-cycle level does).
 * No reference counterpart (the smoother of the corrected multigrid). */
NUSIF_API int nusifSmoothRBF32(const float *x, const float *b, float *xout, int nx, int ny, int nz,
    double hx, double hy, double hz, int sweeps);
/* The FP64 <-> FP32 conversions of the mixed-precision kernels (computed on
 * the integer pipe: round to nearest even, and exact widening), element-wise
 * on n device values. Results are those of the hardware conversions. No
 * reference counterpart. */
NUSIF_API int nusifConvertF64ToF32(const double *x, float *y, long long n);
NUSIF_API int nusifConvertF32ToF64(const float *x, double *y, long long n);

/* Learned pressure warm start (no reference counterpart). A 3-level 3D U-Net
 * (16/32/64 channels, 243,473 parameters; BF16 weights and activations, FP32
 * accumulation and master weights) trained and run by this library's kernels.
 * Volumes are device arrays, channels-last [B][Z][Y][X][C], every edge a
 * multiple of 4; the input has 2 channels, the output 1. Parameters form one
 * flat FP32 vector: per layer (e0a e0b e1a e1b e2a d1a d1b d0a d0b out)
 * W[27][cout][cin] then b[cout]. */
typedef struct NusifUNet NusifUNet;
/* He-normal initial weights from `seed`, zero biases, Adam state zero */
NUSIF_API NusifUNet *nusifUNetCreate(unsigned long long seed);
NUSIF_API void nusifUNetFree(NusifUNet *net);
NUSIF_API long long nusifUNetParamCount(const NusifUNet *net);
NUSIF_API int nusifUNetGetParams(const NusifUNet *net, float *host, long long count);
/* replaces the weights and clears the Adam state */
NUSIF_API int nusifUNetSetParams(NusifUNet *net, const float *host, long long count);
/* gradients of the last nusifUNetTrainStep (host copy) */
NUSIF_API int nusifUNetGetGrads(const NusifUNet *net, float *host, long long count);
/* out (device, [B][Z][Y][X]) = net(x) */
NUSIF_API int nusifUNetForward(NusifUNet *net, const float *x, int B, int Z, int Y, int X,
    float *out);
/* Convolution kernels: 1 (default) the tcgen05 tensor-core kernels wherever the
 * volume's x-rows tile into 128-cell blocks (x a divisor of 128 or a multiple
 * of it), else and with 0 the mma.sync kernels. Results agree to BF16
 * rounding of the activations. */
NUSIF_API int nusifUNetSetTensorCore(NusifUNet *net, int mode);
/* forward, mean-squared-error loss against `target` (device), backward; with
 * update != 0 one Adam step (lr, beta 0.9 / 0.999, eps 1e-8). loss_host may be
 * NULL (no synchronisation). */
NUSIF_API int nusifUNetTrainStep(NusifUNet *net, const float *x, const float *target, int B, int Z,
    int Y, int X, float lr, int update, float *loss_host);
/* Warm start of an mg / mg-mixed solver (grid edges multiples of 8). Each
 * solve then computes, on the half-resolution grid, the features of its warm
 * start p0 (restricted residual and restricted mean-free rhs, each over its
 * RMS), runs the network, forms p1 = p0 + trilinear(net * sigma / kappa),
 * kappa = pi^2 (1/Lx^2 + 1/Ly^2 + 1/Lz^2) for the domain lengths L,
 * and keeps p1 only if its restricted residual ||R(b - A p1)|| (R the 8-cell
 * mean, so the smooth error the V-cycles pay for) is below p0's; the V-cycles then run to
 * the same rtol. net = NULL detaches (the network is borrowed, not owned). */
NUSIF_API int nusifSolverSetGuessNet(Solver *s, NusifUNet *net);
/* The next solve of s also writes its training pair to device buffers:
 * x [kmax/2][jmax/2][imax/2][2] features of its warm start and, after it
 * converged, t [kmax/2][jmax/2][imax/2] = restricted (p* - p0) * kappa / sigma. */
NUSIF_API int nusifSolverRecordPair(Solver *s, float *x, float *t);
/* last solve with a network: whether its guess was taken, and the relative
 * restricted residuals ||R(b - A p)|| / ||R b|| (b mean-free) of the plain
 * warm start and of the guess (the decision criterion) */
NUSIF_API int nusifSolverGuessStats(Solver *s, int *used, double *rel_warm, double *rel_guess);
/* Network evaluations and taken guesses since the last nusifSolverSetGuessNet.
 * With the .par key mg_probe P > 1 the network runs, after two rejections in a
 * row, only every P-th step until a guess is taken again (in between the
 * plain warm start is used, as after a rejection; nusifSolverGuessStats keeps
 * the last evaluated step's figures). */
NUSIF_API int nusifSolverGuessCounts(Solver *s, long long *evaluated, long long *taken);

#ifdef __cplusplus
}
#endif
#endif /* NUSIF_GB300_H */
