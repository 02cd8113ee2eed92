// Internal interface of the learned warm start (unet.cu) for the solver.
#pragma once

#include <stdint.h>

namespace nusif {

struct UNetState;

}  // namespace nusif
