// Internal interface of the learned warm start (unet.cu, guess.cu) for the
// solver (not part of the C ABI).
#pragma once

#include <stdint.h>

#include "nusif_gb300.h"

namespace nusif {

// forward pass of `net` on a device volume x [Z][Y][X][2] (batch 1); *out
// points at the network's own FP32 output [Z][Y][X], valid until its next call
bool unet_infer(NusifUNet *net, const float *x, int Z, int Y, int X, const float **out);

// per-solver state of the warm start (guess.cu)
struct GuessState;
// before the V-cycles: features of the warm start p; with a network, its
// guess replaces p when it has the smaller residual; with a recording request,
// the features go to the caller's buffer and p is kept for the target
bool guess_before_solve(GuessState *g, const Grid *grid, double *p, const double *rhs);
// after the V-cycles: the recorded target from the converged p
bool guess_after_solve(GuessState *g, const Grid *grid, const double *p);
void guess_free(GuessState *g);

}  // namespace nusif
