// Result output: cell-centred fields and the legacy VTK file of the reference.
//
// commCollectResult (reference src/comm.c:327-477, sequential path) averages
// the staggered velocities to cell centres and copies the interior pressure;
// here one kernel does that on the device and the host receives compact
// imax*jmax*kmax arrays. nusifWriteVTK writes the reference's
// STRUCTURED_POINTS file (src/vtkWriter-seq.c:12-146): ASCII "%f" values (the
// reference's default, its VtkOptions.fmt is zero-initialised) or big-endian
// binary doubles.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "nusif_internal.h"

namespace nusif {
namespace {

__global__ void k_collect(Dims g, const double *__restrict__ u, const double *__restrict__ v,
    const double *__restrict__ w, const double *__restrict__ p, double *__restrict__ out)
{
  const int64_t n = (int64_t)g.imax * g.jmax * g.kmax;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % g.imax) + 1;
    const int64_t r = q / g.imax;
    const int j = (int)(r % g.jmax) + 1;
    const int k = (int)(r / g.jmax) + 1;
    const int64_t c = (int64_t)k * g.sk + (int64_t)j * g.sj + i;
    out[q] = (u[c] + u[c - 1]) / 2.0;
    out[n + q] = (v[c] + v[c - g.sj]) / 2.0;
    out[2 * n + q] = (w[c] + w[c - g.sk]) / 2.0;
    out[3 * n + q] = p[c];
  }
}

double swap_bytes(double f)
{
  unsigned char b[8], s[8];
  memcpy(b, &f, 8);
  for (int q = 0; q < 8; q++) s[q] = b[7 - q];
  double out;
  memcpy(&out, s, 8);
  return out;
}

bool host_is_little_endian()
{
  const unsigned one = 1;
  unsigned char c;
  memcpy(&c, &one, 1);
  return c == 1;
}

}  // namespace

}  // namespace nusif

using namespace nusif;

extern "C" {

int nusifCollectResult(const Discretization *d, double *ug, double *vg, double *wg, double *pg)
{
  DiscState *st = disc_state(d);
  if (!st || !ug || !vg || !wg || !pg) {
    fail(NUSIF_ERR_ARG, "nusifCollectResult: unknown discretization or null output");
    return NUSIF_ERR_ARG;
  }
  if (!await_fields(d)) return NUSIF_ERR_CUDA;
  const Dims &g = st->dims;
  const int64_t n = (int64_t)g.imax * g.jmax * g.kmax;
  double *dev = nullptr;
  if (!cuda_ok(cudaMalloc(&dev, 4 * n * sizeof(double)), "cudaMalloc(collect)"))
    return NUSIF_ERR_CUDA;
  k_collect<<<1024, 256, 0, stream()>>>(g, d->u, d->v, d->w, d->p, dev);
  int rc = NUSIF_OK;
  double *outs[4] = { ug, vg, wg, pg };
  if (!launched("k_collect")) rc = NUSIF_ERR_CUDA;
  for (int q = 0; q < 4 && rc == NUSIF_OK; q++)
    if (!cuda_ok(cudaMemcpyAsync(outs[q], dev + q * n, n * sizeof(double),
                     cudaMemcpyDeviceToHost, stream()),
            "collect copy"))
      rc = NUSIF_ERR_CUDA;
  if (rc == NUSIF_OK && !cuda_ok(cudaStreamSynchronize(stream()), "collect sync"))
    rc = NUSIF_ERR_CUDA;
  cudaFree(dev);
  return rc;
}

int nusifWriteVTK(const Discretization *d, const char *path, int binary)
{
  DiscState *st = disc_state(d);
  if (!st || !path) {
    fail(NUSIF_ERR_ARG, "nusifWriteVTK: unknown discretization or null path");
    return NUSIF_ERR_ARG;
  }
  const Dims &g = st->dims;
  const size_t n = (size_t)g.imax * g.jmax * g.kmax;
  std::vector<double> u(n), v(n), w(n), p(n);
  int rc = nusifCollectResult(d, u.data(), v.data(), w.data(), p.data());
  if (rc != NUSIF_OK) return rc;
  FILE *fh = fopen(path, "w");
  if (!fh) {
    fail(NUSIF_ERR_IO, "nusifWriteVTK: cannot open %s", path);
    return NUSIF_ERR_IO;
  }
  const Grid &gr = d->grid;
  fprintf(fh, "# vtk DataFile Version 3.0\n");
  fprintf(fh, "PAMPI cfd solver output\n");
  fprintf(fh, binary ? "BINARY\n" : "ASCII\n");
  fprintf(fh, "DATASET STRUCTURED_POINTS\n");
  fprintf(fh, "DIMENSIONS %d %d %d\n", gr.imax, gr.jmax, gr.kmax);
  fprintf(fh, "ORIGIN %f %f %f\n", gr.dx * 0.5, gr.dy * 0.5, gr.dz * 0.5);
  fprintf(fh, "SPACING %f %f %f\n", gr.dx, gr.dy, gr.dz);
  fprintf(fh, "POINT_DATA %d\n", gr.imax * gr.jmax * gr.kmax);
  const bool swap = host_is_little_endian();
  auto be = [swap](double x) { return swap ? swap_bytes(x) : x; };
  fprintf(fh, "SCALARS %s double 1\n", "pressure");
  fprintf(fh, "LOOKUP_TABLE default\n");
  for (size_t q = 0; q < n; q++) {
    if (binary) {
      const double x = be(p[q]);
      fwrite(&x, sizeof(double), 1, fh);
    } else {
      fprintf(fh, "%f\n", p[q]);
    }
  }
  if (binary) fprintf(fh, "\n");
  fprintf(fh, "VECTORS %s double\n", "velocity");
  for (size_t q = 0; q < n; q++) {
    if (binary) {
      const double x[3] = { be(u[q]), be(v[q]), be(w[q]) };
      fwrite(x, sizeof(double), 3, fh);
    } else {
      fprintf(fh, "%f %f %f\n", u[q], v[q], w[q]);
    }
  }
  if (binary) fprintf(fh, "\n");
  if (fclose(fh) != 0) {
    fail(NUSIF_ERR_IO, "nusifWriteVTK: write error on %s", path);
    return NUSIF_ERR_IO;
  }
  return NUSIF_OK;
}

}  // extern "C"
