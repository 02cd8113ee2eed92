// Runtime of the GB300 NuSiF library: error reporting, the launch stream,
// field upload/download and the side tables that hold device state beside the
// reference structs (whose layouts have no room for it).
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "nusif_internal.h"

namespace nusif {

static int g_error_mode = NUSIF_ERRORS_EXIT;
static int g_error_code = 0;
static std::string g_error_msg;
static cudaStream_t g_stream = nullptr;

void fail(int code, const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (g_error_mode == NUSIF_ERRORS_EXIT) {
    fprintf(stderr, "Error: %s\n", buf);
    exit(EXIT_FAILURE);
  }
  if (g_error_code == 0) {  // keep the first failure of a call chain
    g_error_code = code;
    g_error_msg = buf;
  }
}

bool cuda_ok(cudaError_t e, const char *what)
{
  if (e == cudaSuccess) return true;
  fail(NUSIF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return false;
}

bool has_error() { return g_error_code != 0; }

cudaStream_t stream() { return g_stream; }

static unsigned long long g_launches = 0;

unsigned long long launch_count() { return g_launches; }
// kernels captured into a graph are not launched at capture time; a graph's
// executed kernels are added when it has run
void set_launch_count(unsigned long long n) { g_launches = n; }

bool launched(const char *what)
{
  g_launches++;
  return cuda_ok(cudaGetLastError(), what);
}

bool reduce_scratch_alloc(ReduceScratch &r, int capacity)
{
  if (r.capacity >= capacity) return true;
  reduce_scratch_free(r);
  if (!cuda_ok(cudaMalloc(&r.partials, sizeof(double) * (size_t)capacity), "cudaMalloc(partials)"))
    return false;
  if (!cuda_ok(cudaMalloc(&r.ticket, sizeof(unsigned) * 4), "cudaMalloc(ticket)")) return false;
  if (!cuda_ok(cudaMemset(r.ticket, 0, sizeof(unsigned) * 4), "cudaMemset(ticket)")) return false;
  r.capacity = capacity;
  return true;
}

void reduce_scratch_free(ReduceScratch &r)
{
  if (r.partials) cudaFree(r.partials);
  if (r.ticket) cudaFree(r.ticket);
  r = ReduceScratch();
}

// ---- side tables ----
static std::unordered_map<const void *, DiscState *> &disc_table()
{
  static std::unordered_map<const void *, DiscState *> t;
  return t;
}

DiscState *disc_state(const Discretization *d)
{
  auto &t = disc_table();
  auto it = t.find(d);
  return it == t.end() ? nullptr : it->second;
}

DiscState *disc_state_create(const Discretization *d)
{
  auto &t = disc_table();
  auto it = t.find(d);
  if (it != t.end()) return it->second;
  DiscState *s = new DiscState();
  t[d] = s;
  return s;
}

void disc_state_erase(const Discretization *d)
{
  auto &t = disc_table();
  auto it = t.find(d);
  if (it == t.end()) return;
  delete it->second;
  t.erase(it);
}

// ---- asynchronous field copies ----
// nusifUploadFieldAsync / nusifDownloadFieldAsync queue a copy on a copy
// stream of the library (one per device), after the work already queued on
// the launch stream; the copy's completion event is kept per device pointer.
// The first later entry point that touches that pointer makes the launch
// stream wait for the event (on the device: the host does not wait), so an
// upload can overlap the kernels that do not read its field, and a queued
// download is never overwritten by a later kernel. A kernel that only reads
// the field waits for a pending upload but not for a pending download (both
// only read the device array), so a download of p can overlap adaptUV.
namespace {
// the copies of one device array still in flight: `done` completes with the
// last of them (the copy stream runs them in order); `upload`: one of them
// writes the array
struct Pending {
  cudaEvent_t done = nullptr;
  bool upload = false;
};
std::mutex g_copy_mu;
std::unordered_map<int, cudaStream_t> g_copy_streams;  // device -> copy stream
std::unordered_map<const void *, Pending> g_pending;   // device pointer -> its copies in flight
std::vector<cudaEvent_t> g_spare_events;

cudaEvent_t take_event()
{
  if (!g_spare_events.empty()) {
    cudaEvent_t e = g_spare_events.back();
    g_spare_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (!cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy event")) return nullptr;
  return e;
}

cudaStream_t copy_stream()
{
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), "copy stream device")) return nullptr;
  auto it = g_copy_streams.find(dev);
  if (it != g_copy_streams.end()) return it->second;
  cudaStream_t s = nullptr;
  if (!cuda_ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "copy stream")) return nullptr;
  g_copy_streams[dev] = s;
  return s;
}

// queue one copy of `bytes` touching the device array `field`
bool queue_copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, const void *field)
{
  std::lock_guard<std::mutex> lock(g_copy_mu);
  cudaStream_t cs = copy_stream();
  if (!cs) return false;
  cudaEvent_t after = take_event();
  if (!after) return false;
  // after the launch stream's work so far (which may read or write the field)
  bool ok = cuda_ok(cudaEventRecord(after, g_stream), "copy order record") &&
            cuda_ok(cudaStreamWaitEvent(cs, after, 0), "copy order wait") &&
            cuda_ok(cudaMemcpyAsync(dst, src, bytes, kind, cs), "field copy");
  g_spare_events.push_back(after);  // the wait is queued: the event may be recorded again
  if (!ok) return false;
  Pending &pd = g_pending[field];
  if (!pd.done) pd.done = take_event();
  if (!pd.done) return false;
  // re-recording the event makes it the completion of this copy, which in
  // stream order implies the earlier ones
  if (kind == cudaMemcpyHostToDevice) pd.upload = true;
  return cuda_ok(cudaEventRecord(pd.done, cs), "copy done record");
}

}  // namespace

bool await_copies(const void *const *ptrs, int n)
{
  std::lock_guard<std::mutex> lock(g_copy_mu);
  if (g_pending.empty()) return true;
  bool ok = true;
  for (int q = 0; q < n; q++) {
    auto it = g_pending.find(ptrs[q]);
    if (it == g_pending.end()) continue;
    ok = cuda_ok(cudaStreamWaitEvent(g_stream, it->second.done, 0), "wait for field copy") && ok;
    g_spare_events.push_back(it->second.done);
    g_pending.erase(it);
  }
  return ok;
}

bool await_uploads(const void *const *ptrs, int n)
{
  std::lock_guard<std::mutex> lock(g_copy_mu);
  if (g_pending.empty()) return true;
  bool ok = true;
  for (int q = 0; q < n; q++) {
    auto it = g_pending.find(ptrs[q]);
    if (it == g_pending.end() || !it->second.upload) continue;  // downloads only: reads go on
    ok = cuda_ok(cudaStreamWaitEvent(g_stream, it->second.done, 0), "wait for field upload") && ok;
    g_spare_events.push_back(it->second.done);
    g_pending.erase(it);
  }
  return ok;
}

bool await_all_copies()
{
  std::lock_guard<std::mutex> lock(g_copy_mu);
  bool ok = true;
  for (auto &kv : g_pending) {
    ok = cuda_ok(cudaStreamWaitEvent(g_stream, kv.second.done, 0), "wait for field copy") && ok;
    g_spare_events.push_back(kv.second.done);
  }
  g_pending.clear();
  return ok;
}

bool await_fields(const Discretization *d)
{
  const void *f[8] = { d->u, d->v, d->w, d->p, d->rhs, d->f, d->g, d->h };
  return await_copies(f, 8);
}

static double *field_ptr(const Discretization *d, int which)
{
  switch (which) {
  case NUSIF_U: return d->u;
  case NUSIF_V: return d->v;
  case NUSIF_W: return d->w;
  case NUSIF_P: return d->p;
  case NUSIF_RHS: return d->rhs;
  case NUSIF_F: return d->f;
  case NUSIF_G: return d->g;
  case NUSIF_H: return d->h;
  default: return nullptr;
  }
}

}  // namespace nusif

using namespace nusif;

extern "C" {

void nusifSetErrorMode(int mode) { g_error_mode = mode; }

int nusifGetLastError(char *msg, int len)
{
  int code = g_error_code;
  if (msg && len > 0) {
    strncpy(msg, g_error_msg.c_str(), (size_t)len - 1);
    msg[len - 1] = '\0';
  }
  g_error_code = 0;
  g_error_msg.clear();
  return code;
}

void nusifSetStream(void *s) { g_stream = (cudaStream_t)s; }
void *nusifGetStream(void) { return (void *)g_stream; }

int nusifDownloadField(const Discretization *d, int which, double *host)
{
  DiscState *st = disc_state(d);
  double *src = field_ptr(d, which);
  if (!st || !src || !host) {
    fail(NUSIF_ERR_ARG, "nusifDownloadField: unknown discretization or field %d", which);
    return NUSIF_ERR_ARG;
  }
  size_t bytes = sizeof(double) * (size_t)st->dims.padded;
  const void *fp = src;
  if (!await_uploads(&fp, 1)) return NUSIF_ERR_CUDA;
  if (!cuda_ok(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, g_stream),
          "download field"))
    return NUSIF_ERR_CUDA;
  if (!cuda_ok(cudaStreamSynchronize(g_stream), "download field sync")) return NUSIF_ERR_CUDA;
  return NUSIF_OK;
}

int nusifUploadField(Discretization *d, int which, const double *host)
{
  DiscState *st = disc_state(d);
  double *dst = field_ptr(d, which);
  if (!st || !dst || !host) {
    fail(NUSIF_ERR_ARG, "nusifUploadField: unknown discretization or field %d", which);
    return NUSIF_ERR_ARG;
  }
  velocity_written(st);
  size_t bytes = sizeof(double) * (size_t)st->dims.padded;
  const void *fp = dst;
  if (!await_copies(&fp, 1)) return NUSIF_ERR_CUDA;
  if (!cuda_ok(cudaMemcpyAsync(dst, host, bytes, cudaMemcpyHostToDevice, g_stream),
          "upload field"))
    return NUSIF_ERR_CUDA;
  if (!cuda_ok(cudaStreamSynchronize(g_stream), "upload field sync")) return NUSIF_ERR_CUDA;
  return NUSIF_OK;
}

int nusifUploadFieldAsync(Discretization *d, int which, const double *host)
{
  DiscState *st = disc_state(d);
  double *dst = field_ptr(d, which);
  if (!st || !dst || !host) {
    fail(NUSIF_ERR_ARG, "nusifUploadFieldAsync: unknown discretization or field %d", which);
    return NUSIF_ERR_ARG;
  }
  velocity_written(st);
  const size_t bytes = sizeof(double) * (size_t)st->dims.padded;
  return queue_copy(dst, host, bytes, cudaMemcpyHostToDevice, dst) ? NUSIF_OK : NUSIF_ERR_CUDA;
}

int nusifDownloadFieldAsync(const Discretization *d, int which, double *host)
{
  DiscState *st = disc_state(d);
  double *src = field_ptr(d, which);
  if (!st || !src || !host) {
    fail(NUSIF_ERR_ARG, "nusifDownloadFieldAsync: unknown discretization or field %d", which);
    return NUSIF_ERR_ARG;
  }
  const size_t bytes = sizeof(double) * (size_t)st->dims.padded;
  return queue_copy(host, src, bytes, cudaMemcpyDeviceToHost, src) ? NUSIF_OK : NUSIF_ERR_CUDA;
}

int nusifWaitCopies(void)
{
  std::vector<std::pair<int, cudaStream_t>> streams;
  {
    std::lock_guard<std::mutex> lock(g_copy_mu);
    for (auto &kv : g_copy_streams) streams.push_back(kv);
  }
  int dev = 0;
  cudaGetDevice(&dev);
  bool ok = true;
  for (auto &kv : streams) {
    // a copy stream's work belongs to its device
    if (!cuda_ok(cudaSetDevice(kv.first), "copy device") ||
        !cuda_ok(cudaStreamSynchronize(kv.second), "field copies sync"))
      ok = false;
  }
  cudaSetDevice(dev);
  if (!ok) return NUSIF_ERR_CUDA;
  // every queued copy has ended: nothing is pending any more
  std::lock_guard<std::mutex> lock(g_copy_mu);
  for (auto &kv : g_pending) g_spare_events.push_back(kv.second.done);
  g_pending.clear();
  return NUSIF_OK;
}

unsigned long long nusifLaunchCount(void) { return g_launches; }

const char *nusifVersion(void) { return "nusif-gb300 1.0 (sm_103a)"; }

}  // extern "C"
