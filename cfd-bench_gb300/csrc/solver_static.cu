// Red-black SOR solve that allocates no memory.
//
// Some callers cannot call cudaMalloc: solver hosts that hand out only
// pre-sized device buffers and forbid growth after start-up, embedded or
// plug-in runtimes that reserve all device memory when they initialise, and
// services that must not fail a request on an out-of-memory error. They still
// pass their own pressure and right-hand-side arrays; the per-block partial
// sums, the ticket counter and the convergence state that solve() keeps in
// cudaMalloc'd scratch live here instead in one file-scope __device__ array of
// fixed size. Every GPU that loads the library holds that array until the
// process exits.
//
// The array's name in host code is only a host-side stand-in, not a device
// address, so it is never passed to a kernel. The first call on each device
// (with that device current) looks up the real address with
// cudaGetSymbolAddress and keeps it; make that first call before any stream
// capture, because the lookup is not a stream operation. The kept address is
// only valid for the device context it was looked up in: do not call
// cudaDeviceReset on a device between calls of this function.
//
// Like solve(), the function reads the convergence state back to the host
// and synchronises the library's stream after every chunk of iterations.
//
// All calls share the one array and it keeps the last call's contents: each
// call first resets the counter and the convergence state it reads. Calls
// that overlap on the GPU (two streams, two host threads) race on the array.
#include <atomic>
#include <cmath>
#include <cstdio>

#include "nusif_internal.h"
#include "solver_internal.h"

namespace nusif {
namespace {

// Layout of the static scratch: [state | ticket | partial sums]
constexpr size_t kStateBytes = 256;
constexpr size_t kTicketBytes = 256;
constexpr int kStaticPartials = 32768;  // two per block of the red-black passes
constexpr size_t kStaticBytes = kStateBytes + kTicketBytes + kStaticPartials * sizeof(double);
static_assert(sizeof(SolveState) <= kStateBytes, "solve state does not fit its slot");

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
// device address per device ordinal; atomic because host threads may call
// concurrently on different devices (the address is the same for every thread)
static std::atomic<unsigned char *> g_scratch_addr[kMaxDevices];

__global__ void k_static_init(SolveState *st, unsigned *ticket, double epssq, int itermax,
    double ncell)
{
  st->res = 1.0;
  st->epssq = epssq;
  st->ncell = ncell;
  st->it = 0;
  st->itermax = itermax;
  st->done = !((1.0 >= epssq) && (0 < itermax));
  st->pad = 0;
  for (int q = 0; q < (int)(kTicketBytes / sizeof(unsigned)); q++) ticket[q] = 0u;
}

// device address of the static scratch on the current device (looked up once)
unsigned char *static_scratch()
{
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
  if (dev < 0 || dev >= kMaxDevices) {
    fail(NUSIF_ERR_ARG, "nusifSolveRBStatic: device ordinal %d beyond %d", dev, kMaxDevices);
    return nullptr;
  }
  unsigned char *addr = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (addr == nullptr) {
    void *ptr = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(&ptr, g_static_scratch), "cudaGetSymbolAddress(scratch)"))
      return nullptr;
    addr = static_cast<unsigned char *>(ptr);
    g_scratch_addr[dev].store(addr, std::memory_order_release);
  }
  return addr;
}

}  // namespace
}  // namespace nusif

using namespace nusif;

extern "C" {

int nusifSolveRBStatic(double *p, const double *rhs, int imax, int jmax, int kmax, double dx,
    double dy, double dz, double omega, double eps, int itermax, double *res_out, int *it_out)
{
  if (!p || !rhs || imax < 1 || jmax < 1 || kmax < 1 || itermax < 0 || !(dx > 0) ||
      !(dy > 0) || !(dz > 0)) {
    fail(NUSIF_ERR_ARG, "nusifSolveRBStatic: invalid arguments");
    return NUSIF_ERR_ARG;
  }
  const int64_t padded = (int64_t)(imax + 2) * (jmax + 2) * (kmax + 2);
  if (padded >= ((int64_t)1 << 31)) {
    fail(NUSIF_ERR_ARG, "nusifSolveRBStatic: %lld padded cells exceed the 2^31 index range",
        (long long)padded);
    return NUSIF_ERR_ARG;
  }
  const Dims g = make_dims(imax, jmax, kmax);
  const SorArgs A = make_sor_args(g, dx, dy, dz, omega);
  const int nb = sor_blocks(A);
  if (2 * nb > kStaticPartials) {
    fail(NUSIF_ERR_ARG,
        "nusifSolveRBStatic: a %d x %d x %d grid needs %d partial-sum slots, the static "
        "scratch holds %d; use solve() for grids this large",
        imax, jmax, kmax, 2 * nb, kStaticPartials);
    return NUSIF_ERR_ARG;
  }
  unsigned char *base = static_scratch();
  if (!base) return NUSIF_ERR_CUDA;
  SolveState *st = reinterpret_cast<SolveState *>(base);
  ReduceScratch red;
  red.ticket = reinterpret_cast<unsigned *>(base + kStateBytes);
  red.partials = reinterpret_cast<double *>(base + kStateBytes + kTicketBytes);
  red.capacity = kStaticPartials;

  const double epssq = eps * eps;
  const double ncell = (double)((int64_t)imax * jmax * kmax);
  k_static_init<<<1, 1, 0, stream()>>>(st, red.ticket, epssq, itermax, ncell);
  if (!launched("k_static_init")) return NUSIF_ERR_CUDA;

  SolveState h;
  int chunk = 16;
  for (;;) {
    if (!cuda_ok(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, stream()),
            "static solve state read") ||
        !cuda_ok(cudaStreamSynchronize(stream()), "static solve sync"))
      return NUSIF_ERR_CUDA;
    if (h.done) break;
    for (int q = 0; q < chunk; q++)
      if (!launch_rb_iteration(A, p, rhs, st, red)) return NUSIF_ERR_CUDA;
    if (chunk < 512) chunk *= 2;
  }
  if (res_out) *res_out = h.res;
  if (it_out) *it_out = h.it;
  return NUSIF_OK;
}

}  // extern "C"
