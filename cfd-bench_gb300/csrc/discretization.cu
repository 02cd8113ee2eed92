// FP64 discretization kernels of the NuSiF time step and the reference
// entry points that launch them (src/discretization.h:34-41).
//
// Layout in HBM: each field is one cudaMalloc'd FP64 array (managed memory kept
// in HBM with the key host_fields) in the reference
// layout ((imax+2)(jmax+2)(kmax+2) doubles, i fastest, one ghost layer,
// src/util.h:19-34). Threads map x -> i so every warp touches consecutive
// doubles. All arithmetic is FP64 (the reference computes in double).
#include <algorithm>
#include <cfloat>
#include <initializer_list>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "nusif_internal.h"
#include "fgh_df.cuh"
#include "fp_bits.cuh"
#include "reduce.cuh"

namespace nusif {

DiscState *disc_state_create(const Discretization *d);
void disc_state_erase(const Discretization *d);

namespace {

constexpr int kBlock = 256;

inline int sm_count()
{
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

// ---- fill (initDiscretization, discretization.c:96-105) ----
__global__ void k_fill(double *a, int64_t n, double value)
{
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    a[q] = value;
}

// ---- max |u|, |v|, |w| over the padded arrays (discretization.c:391-401) ----
// Seeded with DBL_MIN like the reference. Threads compare |x| as bit patterns
// on the integer pipe (abs_max_key: non-negative doubles order like their
// bits, NaN skipped as the reference's `>` test skips it), so the FP64 pipe
// stays free; block maxima go to partials as doubles and the last block
// folds them.
__global__ void __launch_bounds__(kBlock) k_max3(const double *__restrict__ u,
    const double *__restrict__ v, const double *__restrict__ w, int64_t n,
    double *__restrict__ partials, unsigned *ticket, double *__restrict__ out3)
{
  // running maxima as bit-pattern pairs (high, low), seeded with DBL_MIN
  unsigned uh = 0x00100000u, ul = 0u, vh = 0x00100000u, vl = 0u, wh = 0x00100000u, wl = 0u;
  const int64_t stride = (int64_t)gridDim.x * kBlock;
  // pairs of doubles (cudaMalloc bases are 256-byte aligned)
  const int64_t npair = n / 2;
  const double2 *u2 = reinterpret_cast<const double2 *>(u);
  const double2 *v2 = reinterpret_cast<const double2 *>(v);
  const double2 *w2 = reinterpret_cast<const double2 *>(w);
  for (int64_t q = blockIdx.x * (int64_t)kBlock + threadIdx.x; q < npair; q += stride) {
    double2 a = __ldg(u2 + q), b = __ldg(v2 + q), c = __ldg(w2 + q);
    abs_max_key(uh, ul, a.x);
    abs_max_key(uh, ul, a.y);
    abs_max_key(vh, vl, b.x);
    abs_max_key(vh, vl, b.y);
    abs_max_key(wh, wl, c.x);
    abs_max_key(wh, wl, c.y);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    abs_max_key(uh, ul, u[n - 1]);
    abs_max_key(vh, vl, v[n - 1]);
    abs_max_key(wh, wl, w[n - 1]);
  }
  double mu = __hiloint2double((int)uh, (int)ul), mv = __hiloint2double((int)vh, (int)vl),
         mw = __hiloint2double((int)wh, (int)wl);
  __shared__ double sm[3][kBlock / 32];
  mu = block_reduce_max<kBlock>(mu, sm[0]);
  mv = block_reduce_max<kBlock>(mv, sm[1]);
  mw = block_reduce_max<kBlock>(mw, sm[2]);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x + 0] = mu;
    partials[3 * blockIdx.x + 1] = mv;
    partials[3 * blockIdx.x + 2] = mw;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  double a = DBL_MIN, b = DBL_MIN, c = DBL_MIN;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += kBlock) {
    a = fmax(a, ld_cg(partials + 3 * q + 0));
    b = fmax(b, ld_cg(partials + 3 * q + 1));
    c = fmax(c, ld_cg(partials + 3 * q + 2));
  }
  a = block_reduce_max<kBlock>(a, sm[0]);
  b = block_reduce_max<kBlock>(b, sm[1]);
  c = block_reduce_max<kBlock>(c, sm[2]);
  if (threadIdx.x == 0) {
    out3[0] = a;
    out3[1] = b;
    out3[2] = c;
    *ticket = 0;
  }
}

// ---- velocity boundary conditions, one face per launch (discretization.c:119-332) ----
// The normal component lives on the wall face (index 0 or n), the tangential
// components have a ghost cell (0 or n+1) mirrored from the first interior
// cell. Faces run in the reference order (top, bottom, left, right, front,
// back) as separate launches: later faces read edge values earlier ones wrote.
struct FaceArgs {
  Dims g;
  int axis, high, bc;
};

__global__ void k_face(FaceArgs fa, double *__restrict__ u, double *__restrict__ v,
    double *__restrict__ w)
{
  const Dims &g = fa.g;
  const int ax = fa.axis;
  const int a1 = (ax == 0) ? 1 : 0;
  const int a2 = (ax == 2) ? 1 : 2;
  const int n[3] = { g.imax, g.jmax, g.kmax };
  const int a = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int b = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (a > n[a1] || b > n[a2]) return;
  const int s[3] = { 1, g.sj, g.sk };
  const int64_t base = (int64_t)a * s[a1] + (int64_t)b * s[a2];
  const int na = n[ax];
  const int wall = fa.high ? na : 0, wall_in = fa.high ? na - 1 : 1;
  const int ghost = fa.high ? na + 1 : 0, inner = fa.high ? na : 1;
  double *vel[3] = { u, v, w };
  for (int comp = 0; comp < 3; comp++) {
    double *q = vel[comp];
    if (comp == ax) {
      q[base + (int64_t)wall * s[ax]] =
          (fa.bc == OUTFLOW) ? q[base + (int64_t)wall_in * s[ax]] : 0.0;
    } else {
      const double in = q[base + (int64_t)inner * s[ax]];
      q[base + (int64_t)ghost * s[ax]] = (fa.bc == NOSLIP) ? -in : in;
    }
  }
}

// ---- special boundary conditions (discretization.c:364-389) ----
__global__ void k_lid(Dims g, double twice_lid, double *__restrict__ u)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (i >= g.imax || k >= g.kmax) return;
  const int64_t c = (int64_t)k * g.sk + (int64_t)g.jmax * g.sj + i;
  u[c + g.sj] = twice_lid - u[c];
}

__global__ void k_inflow(Dims g, double inflow, double *__restrict__ u)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y * blockDim.y + threadIdx.y + 1;
  if (j > g.jmax || k > g.kmax) return;
  u[(int64_t)k * g.sk + (int64_t)j * g.sj] = inflow;
}

// ---- F, G, H (discretization.c:455-652) in flux form ----
// The donor-cell scheme is conservative: the reference's convective
// difference du2dx (discretization.c:491-497) is Tx(i) - Tx(i-1) with
// Tx(i) = c1*cp*(u_i + u_i+1) + c2*|cp|*(u_i - u_i+1), cp the doubled transport
// velocity on face i+1/2, and the same holds for every term except the
// z-convection of G, whose "minus" half uses V(i,j,k+1) (discretization.c:
// 543-550, kept). The viscous term joins the face flux (nu*(q_a - q_b) with
// nu = (1/Re)/h^2), so a cell needs three face fluxes per component instead of
// six convective halves plus three second differences.
// A face flux c1*cp*(q_a + q_b) + (c2*|cp| + nu)*(q_a - q_b) is evaluated as
// A*q_a + B*q_b with A = cp*(c1 +- c2) + nu, B = cp*(c1 -+ c2) - nu, the signs
// picked by the sign bit of cp on the integer pipe: five FP64 instructions per
// face (the add making cp included) instead of seven, about 73 per cell in
// all. GB300 issues two FP64 lanes per SM and clock, so the FP64 instruction
// count, not HBM, bounds this kernel. A block owns a 32 x 8 tile of (i, j)
// columns and marches in k: x-face fluxes reach the right neighbour and
// y-face fluxes the next row through shared memory, z-face fluxes stay in
// registers.
struct FaceCoef {
  double P, M, nu;  // (1 + gamma)*0.25/h, (1 - gamma)*0.25/h, (1/Re)/h^2
};

struct FluxArgs {
  Dims g;
  FaceCoef ax, ay, az;
  double dt, gx, gy, gz;
  const StepScalars *sp;  // when set, dt comes from device memory (captured steps)
  int kb;                 // k planes per block
};

// total (convective + viscous) flux of q across the face between q_a (minus
// side) and q_b (plus side), transported by the doubled velocity cp
__device__ __forceinline__ double face_flux(const FaceCoef &a, double cp, double qa, double qb)
{
  const bool neg = __double2hiint(cp) < 0;  // sign bit (an integer test, not DSETP)
  const double A = fma(cp, neg ? a.M : a.P, a.nu);
  const double B = fma(cp, neg ? a.P : a.M, -a.nu);
  return fma(A, qa, B * qb);
}

struct XFace { double f, g, h; };
struct ZFace { double f, h, gv, gc; };  // gv: viscous flux of G, gc: G's transport velocity

__device__ __forceinline__ XFace x_face(const double *__restrict__ u, const double *__restrict__ v,
    const double *__restrict__ w, int64_t c, int sj, int sk, const FaceCoef &a)
{
  const double uc = __ldg(u + c);
  XFace r;
  r.f = face_flux(a, uc + __ldg(u + c + 1), uc, __ldg(u + c + 1));
  r.g = face_flux(a, uc + __ldg(u + c + sj), __ldg(v + c), __ldg(v + c + 1));
  r.h = face_flux(a, uc + __ldg(u + c + sk), __ldg(w + c), __ldg(w + c + 1));
  return r;
}

__device__ __forceinline__ XFace y_face(const double *__restrict__ u, const double *__restrict__ v,
    const double *__restrict__ w, int64_t c, int sj, int sk, const FaceCoef &a)
{
  const double vc = __ldg(v + c);
  XFace r;
  r.f = face_flux(a, vc + __ldg(v + c + 1), __ldg(u + c), __ldg(u + c + sj));
  r.g = face_flux(a, vc + __ldg(v + c + sj), vc, __ldg(v + c + sj));
  r.h = face_flux(a, vc + __ldg(v + c + sk), __ldg(w + c), __ldg(w + c + sj));
  return r;
}

__device__ __forceinline__ ZFace z_face(const double *__restrict__ u, const double *__restrict__ v,
    const double *__restrict__ w, int64_t c, int sj, int sk, const FaceCoef &a)
{
  const double wc = __ldg(w + c);
  ZFace r;
  r.f = face_flux(a, wc + __ldg(w + c + 1), __ldg(u + c), __ldg(u + c + sk));
  r.h = face_flux(a, wc + __ldg(w + c + sk), wc, __ldg(w + c + sk));
  r.gv = a.nu * (__ldg(v + c) - __ldg(v + c + sk));
  r.gc = wc + __ldg(w + c + sj);
  return r;
}

constexpr int kFX = 32, kFY = 8;

// GRAVITY false: gx = gy = gz = 0, where fma(dt, 0 - s, q) is exactly
// fma(-dt, s, q): one FP64 instruction less per component, same bits.
template <bool GRAVITY>
__global__ void __launch_bounds__(kFX *kFY) k_fgh_flux(FluxArgs A, const double *__restrict__ u,
    const double *__restrict__ v, const double *__restrict__ w, double *__restrict__ f,
    double *__restrict__ gg, double *__restrict__ h)
{
  __shared__ XFace ys[2][kFY][kFX];
  __shared__ XFace xs[2][kFY][kFX + 1];  // [row][1 + tx]: plus face of cell tx; [row][0]: the row's left halo face
  const Dims &g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i_raw = blockIdx.x * kFX + tx + 1;
  const int j_raw = blockIdx.y * kFY + ty + 1;
  const bool active = i_raw <= g.imax && j_raw <= g.jmax;
  const int i = min(i_raw, g.imax), j = min(j_raw, g.jmax);  // loads stay in bounds
  const int k0 = blockIdx.z * A.kb + 1;
  const int k1 = min(k0 + A.kb - 1, g.kmax);
  const int sj = g.sj, sk = g.sk;
  const int64_t col = (int64_t)j * sj + i;
  // the left halo face of row `tx` (lanes 0..kFY-1 of the first warp): the
  // minus face of the row's first cell, computed once per row and plane
  const bool halo = ty == 0 && tx < kFY;
  const int64_t halo_col =
      (int64_t)min((int)(blockIdx.y * kFY) + tx + 1, g.jmax) * sj +
      min((int)(blockIdx.x * kFX) + 1, g.imax) - 1;
  const double dt = A.sp ? A.sp->dt : A.dt;
  ZFace zm = z_face(u, v, w, (int64_t)(k0 - 1) * sk + col, sj, sk, A.az);
  int buf = 0;
  for (int k = k0; k <= k1; k++, buf ^= 1) {
    const int64_t c = (int64_t)k * sk + col;
    const XFace xp = x_face(u, v, w, c, sj, sk, A.ax);
    xs[buf][ty][tx + 1] = xp;
    if (halo) xs[buf][tx][0] = x_face(u, v, w, (int64_t)k * sk + halo_col, sj, sk, A.ax);
    const XFace yp = y_face(u, v, w, c, sj, sk, A.ay);
    ys[buf][ty][tx] = yp;
    __syncthreads();
    const XFace xm = xs[buf][ty][tx];
    const XFace ym = ty > 0 ? ys[buf][ty - 1][tx] : y_face(u, v, w, c - sj, sj, sk, A.ay);
    const ZFace zp = z_face(u, v, w, c, sj, sk, A.az);
    if (active) {
      const double uc = __ldg(u + c), vc = __ldg(v + c), wc = __ldg(w + c);
      // F(imax), G(jmax), H(kmax) are wall faces carrying the velocity (discretization.c:609-651)
      const double sf = (xp.f - xm.f) + (yp.f - ym.f) + (zp.f - zm.f);
      f[c] = (i == g.imax) ? uc : GRAVITY ? fma(dt, A.gx - sf, uc) : fma(-dt, sf, uc);
      // c1*(vc + vt)*(gp - gm) + c2*(vc - vt)*(|gp| + |gm|) as gp*Xp - gm*Xm,
      // Xp and Xm weighted sums of vc and vt chosen by the signs of gp and gm
      const double vt = __ldg(v + c + sk);
      const bool np = __double2hiint(zp.gc) < 0, nm = __double2hiint(zm.gc) < 0;
      const double xpz = fma(np ? A.az.M : A.az.P, vc, (np ? A.az.P : A.az.M) * vt);
      const double xmz = fma(nm ? A.az.P : A.az.M, vc, (nm ? A.az.M : A.az.P) * vt);
      const double zconv = fma(zp.gc, xpz, -(zm.gc * xmz));
      const double sg = (xp.g - xm.g) + (yp.g - ym.g) + (zp.gv - zm.gv) + zconv;
      gg[c] = (j == g.jmax) ? vc : GRAVITY ? fma(dt, A.gy - sg, vc) : fma(-dt, sg, vc);
      const double sh = (xp.h - xm.h) + (yp.h - ym.h) + (zp.h - zm.h);
      h[c] = (k == g.kmax) ? wc : GRAVITY ? fma(dt, A.gz - sh, wc) : fma(-dt, sh, wc);
      // low wall faces F(0), G(0), H(0) carry the velocity (discretization.c:601-643)
      if (i == 1) f[c - 1] = __ldg(u + c - 1);
      if (j == 1) gg[c - sj] = __ldg(v + c - sj);
      if (k == 1) h[c - sk] = __ldg(w + c - sk);
    }
    zm = zp;
  }
}

// ---- F, G, H in double-float arithmetic (fgh_df.cuh) ----
// The same flux form, tile (32 x 8 columns marching in k) and flux sharing
// as k_fgh_flux, with the face fluxes carried in pairs of FP32 numbers on the
// FP32 pipe (about 2^-47 of the operands, measured within 2e-14 of the FP64
// oracle on random fields at 64^3..256^3) instead of ~70 FP64 instructions
// per cell. u, v, w are split into pairs once per block: a ring of three
// planes in shared memory holds the pairs of the (34 x 10) region around the
// tile (one halo column and row on each side); plane k+2 is loaded into
// registers while plane k's fluxes are computed and split into the ring
// slot plane k-1 used, so one barrier per plane suffices. The result
// q + dt (g - s) is formed in FP64 (two FP64 adds per component) from the
// exact velocity q and the pair dt (g - s).
constexpr int kDX = 32, kDY = 8;
constexpr int kRW = kDX + 2, kRH = kDY + 2;  // region columns i0-1 .. i0+32, rows j0-1 .. j0+8
constexpr int kRC = kRW * kRH;               // cells per field and plane
constexpr int kRItems = 3 * kRC;             // u, v, w
constexpr int kRPer = (kRItems + kDX * kDY - 1) / (kDX * kDY);
constexpr size_t kDfRingBytes = 3 * (size_t)kRItems * sizeof(df::f2);
constexpr size_t kDfXsBytes = 2 * (size_t)kDY * (kDX + 1) * sizeof(df::Face);
constexpr size_t kDfYsBytes = 2 * (size_t)kDY * kDX * sizeof(df::Face);
constexpr size_t kDfSmemBytes = kDfRingBytes + kDfXsBytes + kDfYsBytes;

struct FluxArgsDF {
  Dims g;
  df::AxisCoef ax, ay, az;
  df::f2 gx, gy, gz;
  double dt;
  const StepScalars *sp;  // when set, dt comes from device memory (captured steps)
  int kb;                 // k planes per block
};

template <bool GRAVITY>
__global__ void __launch_bounds__(kDX *kDY, 3) k_fgh_df(FluxArgsDF A, const double *__restrict__ u,
    const double *__restrict__ v, const double *__restrict__ w, double *__restrict__ f,
    double *__restrict__ gg, double *__restrict__ h)
{
  using namespace df;
  extern __shared__ __align__(16) unsigned char df_smem[];
  f2 *ring = reinterpret_cast<f2 *>(df_smem);  // [slot][field][row][col]
  Face(*xs)[kDY][kDX + 1] = reinterpret_cast<Face(*)[kDY][kDX + 1]>(df_smem + kDfRingBytes);
  Face(*ys)[kDY][kDX] =
      reinterpret_cast<Face(*)[kDY][kDX]>(df_smem + kDfRingBytes + kDfXsBytes);

  const Dims &g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kDX + tx;
  const int i0 = blockIdx.x * kDX + 1, j0 = blockIdx.y * kDY + 1;
  const bool active = i0 + tx <= g.imax && j0 + ty <= g.jmax;
  const int i = min(i0 + tx, g.imax), j = min(j0 + ty, g.jmax);
  const int k0 = blockIdx.z * A.kb + 1;
  const int k1 = min(k0 + A.kb - 1, g.kmax);
  const int sj = g.sj, sk = g.sk;

  // the region cells this thread loads for every plane: field pointer + column offset
  const double *src[kRPer];
  int soff[kRPer];
#pragma unroll
  for (int r = 0; r < kRPer; r++) {
    const int q = min(tid + r * kDX * kDY, kRItems - 1);  // surplus threads repeat the last item
    const int fld = q / kRC, cell = q - fld * kRC;
    const int row = cell / kRW, col = cell - row * kRW;
    // region row/col -> padded j/i, clamped to the array (clamped cells feed inactive cells only)
    const int jj = min(j0 - 1 + row, g.jmax + 1), ii = min(i0 - 1 + col, g.imax + 1);
    src[r] = (fld == 0 ? u : fld == 1 ? v : w) + (int64_t)jj * sj + ii;
    soff[r] = q;
  }
  auto load_plane = [&](int kk, double (&val)[kRPer]) {
    const int64_t o = (int64_t)min(kk, g.kmax + 1) * sk;
#pragma unroll
    for (int r = 0; r < kRPer; r++) val[r] = __ldg(src[r] + o);
  };
  auto store_plane = [&](int slot, const double (&val)[kRPer]) {
#pragma unroll
    for (int r = 0; r < kRPer; r++) ring[slot * kRItems + soff[r]] = split(val[r]);
  };
  // the quad (cell, +x, +y, +z neighbours) of field fld at region (row, col), planes s0 / s1
  auto quad = [&](int s0, int s1, int fld, int row, int col) {
    const f2 *p0 = ring + s0 * kRItems + fld * kRC + row * kRW + col;
    const f2 *p1 = ring + s1 * kRItems + fld * kRC + row * kRW + col;
    return Quad{ p0[0], p0[1], p0[kRW], p1[0] };
  };

  const double dt = A.sp ? A.sp->dt : A.dt;
  const f2 mdt = split(-dt);

  // planes k0-1, k0, k0+1 into slots 0, 1, 2
  {
    double val[kRPer];
    load_plane(k0 - 1, val);
    store_plane(0, val);
    load_plane(k0, val);
    store_plane(1, val);
    load_plane(k0 + 1, val);
    store_plane(2, val);
  }
  __syncthreads();
  ZFaceG zgm;
  Face zm;
  {
    const Quad U = quad(0, 1, 0, ty + 1, tx + 1), V = quad(0, 1, 1, ty + 1, tx + 1),
               W = quad(0, 1, 2, ty + 1, tx + 1);
    zm = z_face(A.az, U, V, W, zgm);
  }
  __syncthreads();  // slot 0 (plane k0-1) is refilled in the first iteration

  int s0 = 1, s1 = 2, s2 = 0;  // slots of planes k, k+1, k+2
  int buf = 0;
  for (int k = k0; k <= k1; k++) {
    double val[kRPer];
    load_plane(k + 2, val);
    const Quad U = quad(s0, s1, 0, ty + 1, tx + 1), V = quad(s0, s1, 1, ty + 1, tx + 1),
               W = quad(s0, s1, 2, ty + 1, tx + 1);
    const Face xp = x_face(A.ax, U, V, W);
    const Face yp = y_face(A.ay, U, V, W);
    ZFaceG zgp;
    const Face zp = z_face(A.az, U, V, W, zgp);
    xs[buf][ty][tx + 1] = xp;
    ys[buf][ty][tx] = yp;
    if (ty == 1 && tx < kDY) {  // the left halo x-face of row tx (column i0-1)
      const Quad Uh = quad(s0, s1, 0, tx + 1, 0), Vh = quad(s0, s1, 1, tx + 1, 0),
                 Wh = quad(s0, s1, 2, tx + 1, 0);
      xs[buf][tx][0] = x_face(A.ax, Uh, Vh, Wh);
    }
    Face ymh;
    if (ty == 0) {  // the y-face below the tile's first row (row j0-1)
      const Quad Uh = quad(s0, s1, 0, 0, tx + 1), Vh = quad(s0, s1, 1, 0, tx + 1),
                 Wh = quad(s0, s1, 2, 0, tx + 1);
      ymh = y_face(A.ay, Uh, Vh, Wh);
    }
    store_plane(s2, val);
    __syncthreads();
    const Face xm = xs[buf][ty][tx];
    const Face ym = ty > 0 ? ys[buf][ty - 1][tx] : ymh;
    if (active) {
      const int64_t c = (int64_t)k * sk + (int64_t)j * sj + i;
      const double uc = __ldg(u + c), vc = __ldg(v + c), wc = __ldg(w + c);
      // F(imax), G(jmax), H(kmax) are wall faces carrying the velocity (discretization.c:609-651)
      // the flux sums stay unnormalised pairs (df32.cuh add_u): they only feed update()
      const f2 sf = add_u(add_u(sub_u(xp.f, xm.f), sub_u(yp.f, ym.f)), sub_u(zp.f, zm.f));
      f[c] = (i == g.imax) ? uc : update(uc, sf, A.gx, mdt, GRAVITY);
      const f2 zc = g_zconv(A.az, zgp.gc, zgm.gc, V.c, V.z);
      const f2 sg =
          add_u(add_u(add_u(sub_u(xp.g, xm.g), sub_u(yp.g, ym.g)), sub_u(zgp.gv, zgm.gv)), zc);
      gg[c] = (j == g.jmax) ? vc : update(vc, sg, A.gy, mdt, GRAVITY);
      const f2 sh = add_u(add_u(sub_u(xp.h, xm.h), sub_u(yp.h, ym.h)), sub_u(zp.h, zm.h));
      h[c] = (k == g.kmax) ? wc : update(wc, sh, A.gz, mdt, GRAVITY);
      // low wall faces F(0), G(0), H(0) carry the velocity (discretization.c:601-643)
      if (i == 1) f[c - 1] = __ldg(u + c - 1);
      if (j == 1) gg[c - sj] = __ldg(v + c - sj);
      if (k == 1) h[c - sk] = __ldg(w + c - sk);
    }
    zm = zp;
    zgm = zgp;
    buf ^= 1;
    const int t = s0;
    s0 = s1;
    s1 = s2;
    s2 = t;
  }
}

// ---- RHS (discretization.c:334-362) ----
// ((F - F_w)/dx + (G - G_s)/dy + (H - H_b)/dz)/dt with 1/(h dt) folded into
// one factor per axis: six FP64 instructions per cell instead of seven.
__global__ void __launch_bounds__(kBlock) k_rhs(Dims g, double rx_arg, double ry_arg,
    double rz_arg, const StepScalars *sp, const double *__restrict__ f,
    const double *__restrict__ gg, const double *__restrict__ h, double *__restrict__ rhs)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > g.imax || j > g.jmax || k > g.kmax) return;
  const double rx = sp ? sp->rx : rx_arg, ry = sp ? sp->ry : ry_arg, rz = sp ? sp->rz : rz_arg;
  const int64_t c = (int64_t)k * g.sk + (int64_t)j * g.sj + i;
  rhs[c] = (f[c] - f[c - 1]) * rx + (gg[c] - gg[c - g.sj]) * ry + (h[c] - h[c - g.sk]) * rz;
}

// ---- adaptUV (discretization.c:654-681) ----
// With MAX the block also folds the maxima of |u|, |v|, |w| it wrote (bit
// patterns, NaN skipped, as k_max3) and raises one slot of amax_slots per
// field with an integer atomic maximum (non-negative doubles order like their
// bits); blocks spread over kAmaxSlots slots.
template <bool MAX>
__global__ void __launch_bounds__(kBlock) k_adapt(Dims g, double fx_arg, double fy_arg,
    double fz_arg, const StepScalars *sp, const double *__restrict__ f,
    const double *__restrict__ gg, const double *__restrict__ h, const double *__restrict__ p,
    double *__restrict__ u, double *__restrict__ v, double *__restrict__ w,
    unsigned long long *amax_slots)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  const bool in = i <= g.imax && j <= g.jmax && k <= g.kmax;
  unsigned uh = 0u, ul = 0u, vh = 0u, vl = 0u, wh = 0u, wl = 0u;
  if (in) {
    const double fx = sp ? sp->fx : fx_arg, fy = sp ? sp->fy : fy_arg, fz = sp ? sp->fz : fz_arg;
    const int64_t c = (int64_t)k * g.sk + (int64_t)j * g.sj + i;
    const double pc = p[c];
    const double un = f[c] - (p[c + 1] - pc) * fx;
    const double vn = gg[c] - (p[c + g.sj] - pc) * fy;
    const double wn = h[c] - (p[c + g.sk] - pc) * fz;
    u[c] = un;
    v[c] = vn;
    w[c] = wn;
    if (MAX) {
      abs_max_key(uh, ul, un);
      abs_max_key(vh, vl, vn);
      abs_max_key(wh, wl, wn);
    }
  }
  if (!MAX) return;
  // keys stay 32-bit pairs on the integer pipe: an FP64 maximum per thread
  // would cost more than the whole kernel on GB300's FP64 rate
  warp_key_max(uh, ul);
  warp_key_max(vh, vl);
  warp_key_max(wh, wl);
  __shared__ unsigned sk[kBlock / 32][6];
  const int t = flat_tid();
  if ((t & 31) == 0) {
    sk[t >> 5][0] = uh;
    sk[t >> 5][1] = ul;
    sk[t >> 5][2] = vh;
    sk[t >> 5][3] = vl;
    sk[t >> 5][4] = wh;
    sk[t >> 5][5] = wl;
  }
  __syncthreads();
  if (t == 0) {
    for (int q = 1; q < kBlock / 32; q++) {
      key_max(uh, ul, sk[q][0], sk[q][1]);
      key_max(vh, vl, sk[q][2], sk[q][3]);
      key_max(wh, wl, sk[q][4], sk[q][5]);
    }
    const unsigned b = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    unsigned long long *slot = amax_slots + 3 * (b % kAmaxSlots);
    atomicMax(slot + 0, ((unsigned long long)uh << 32) | ul);
    atomicMax(slot + 1, ((unsigned long long)vh << 32) | vl);
    atomicMax(slot + 2, ((unsigned long long)wh << 32) | wl);
  }
}

// ---- computeTimestep's maxima after a fused adaptUV ----
// max |u|, |v|, |w| over the padded cells adaptUV does not write (the ghost
// shell: planes k = 0 and kmax + 1, rows j = 0 and jmax + 1 of the planes
// between, cells i = 0 and imax + 1 of the rows between), folded with the
// slots k_adapt<true> raised and the reference's DBL_MIN seed: the maximum
// over the whole arrays, as k_max3. The last block zeroes the slots.
__global__ void __launch_bounds__(kBlock) k_shell_max3(Dims g, const double *__restrict__ u,
    const double *__restrict__ v, const double *__restrict__ w, unsigned long long *amax_slots,
    double *__restrict__ partials, unsigned *ticket, double *__restrict__ out3)
{
  // 32-bit indices: the padded size is below 2^31 (checked at init)
  const int P = g.imax + 2, PQ = g.sk;
  const int n1 = 2 * PQ, n2 = g.kmax * 2 * P, n3 = g.kmax * g.jmax * 2;
  unsigned uh = 0u, ul = 0u, vh = 0u, vl = 0u, wh = 0u, wl = 0u;
  for (int q = blockIdx.x * kBlock + threadIdx.x; q < n1 + n2 + n3; q += gridDim.x * kBlock) {
    int c;
    if (q < n1) {
      c = q < PQ ? q : (g.kmax + 1) * PQ + (q - PQ);
    } else if (q < n1 + n2) {
      const int r = q - n1;
      const int k = 1 + r / (2 * P), rr = r - (k - 1) * (2 * P);
      c = k * PQ + (rr < P ? rr : (g.jmax + 1) * g.sj + (rr - P));
    } else {
      const int r = q - n1 - n2;
      const int k = 1 + r / (2 * g.jmax), rr = r - (k - 1) * (2 * g.jmax);
      c = k * PQ + (1 + (rr >> 1)) * g.sj + ((rr & 1) ? g.imax + 1 : 0);
    }
    abs_max_key(uh, ul, u[c]);
    abs_max_key(vh, vl, v[c]);
    abs_max_key(wh, wl, w[c]);
  }
  __shared__ double sm[3][kBlock / 32];
  double mu = block_reduce_max<kBlock>(__hiloint2double((int)uh, (int)ul), sm[0]);
  double mv = block_reduce_max<kBlock>(__hiloint2double((int)vh, (int)vl), sm[1]);
  double mw = block_reduce_max<kBlock>(__hiloint2double((int)wh, (int)wl), sm[2]);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x + 0] = mu;
    partials[3 * blockIdx.x + 1] = mv;
    partials[3 * blockIdx.x + 2] = mw;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  double a = DBL_MIN, b = DBL_MIN, c = DBL_MIN;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += kBlock) {
    a = fmax(a, ld_cg(partials + 3 * q + 0));
    b = fmax(b, ld_cg(partials + 3 * q + 1));
    c = fmax(c, ld_cg(partials + 3 * q + 2));
  }
  for (int q = threadIdx.x; q < kAmaxSlots; q += kBlock) {
    a = fmax(a, __longlong_as_double((long long)amax_slots[3 * q + 0]));
    b = fmax(b, __longlong_as_double((long long)amax_slots[3 * q + 1]));
    c = fmax(c, __longlong_as_double((long long)amax_slots[3 * q + 2]));
    amax_slots[3 * q + 0] = 0ull;
    amax_slots[3 * q + 1] = 0ull;
    amax_slots[3 * q + 2] = 0ull;
  }
  a = block_reduce_max<kBlock>(a, sm[0]);
  b = block_reduce_max<kBlock>(b, sm[1]);
  c = block_reduce_max<kBlock>(c, sm[2]);
  if (threadIdx.x == 0) {
    out3[0] = a;
    out3[1] = b;
    out3[2] = c;
    *ticket = 0;
  }
}

// ---- normalizePressure (discretization.c:403-429) ----
// Interior sum (block partials folded by the last block), then the mean is
// subtracted by a second kernel that reads it from device memory.
__global__ void __launch_bounds__(kBlock) k_interior_sum(Dims g, const double *__restrict__ p,
    double *__restrict__ partials, unsigned *ticket, double *__restrict__ out)
{
  const int64_t ncell = (int64_t)g.imax * g.jmax * g.kmax;
  double s = 0.0;
  for (int64_t q = blockIdx.x * (int64_t)kBlock + threadIdx.x; q < ncell;
       q += (int64_t)gridDim.x * kBlock) {
    const int i = (int)(q % g.imax) + 1;
    const int64_t r = q / g.imax;
    const int j = (int)(r % g.jmax) + 1;
    const int k = (int)(r / g.jmax) + 1;
    s += p[(int64_t)k * g.sk + (int64_t)j * g.sj + i];
  }
  __shared__ double sm[kBlock / 32];
  s = block_reduce_sum<kBlock>(s, sm);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s;
    last = ticket_is_last(ticket);
  }
  __syncthreads();
  if (!last) return;
  double t = 0.0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += kBlock) t += ld_cg(partials + q);
  t = block_reduce_sum<kBlock>(t, sm);
  if (threadIdx.x == 0) {
    out[0] = t;
    out[1] = t / (double)ncell;
    *ticket = 0;
  }
}

__global__ void __launch_bounds__(kBlock) k_subtract_mean(Dims g, double *__restrict__ p,
    const double *__restrict__ mean)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > g.imax || j > g.jmax || k > g.kmax) return;
  const int64_t c = (int64_t)k * g.sk + (int64_t)j * g.sj + i;
  p[c] = p[c] - mean[0];
}

dim3 cell_grid(const Dims &g, dim3 blk)
{
  return dim3((g.imax + blk.x - 1) / blk.x, (g.jmax + blk.y - 1) / blk.y,
      (g.kmax + blk.z - 1) / blk.z);
}

const dim3 kCellBlock(64, 2, 2);

}  // namespace

// ---- launchers ----

bool launch_max3(const Dims &g, const double *u, const double *v, const double *w,
    ReduceScratch &red, double *d_out3)
{
  int blocks = 4 * sm_count();
  if (!reduce_scratch_alloc(red, 3 * blocks)) return false;
  k_max3<<<blocks, kBlock, 0, stream()>>>(u, v, w, g.padded, red.partials, red.ticket, d_out3);
  return launched("k_max3");
}

bool launch_bc(const Dims &g, const int bc[6], int problem, double lid, double inflow,
    double *u, double *v, double *w)
{
  // reference order: top, bottom, left, right, front, back (discretization.c:129-331)
  static const int order[6][3] = { // axis, high, slot in bc[] (left,right,bottom,top,front,back)
    { 1, 1, 3 }, { 1, 0, 2 }, { 0, 0, 0 }, { 0, 1, 1 }, { 2, 0, 4 }, { 2, 1, 5 } };
  (void)problem;
  (void)lid;
  (void)inflow;
  const int n[3] = { g.imax, g.jmax, g.kmax };
  for (int f = 0; f < 6; f++) {
    FaceArgs fa{ g, order[f][0], order[f][1], bc[order[f][2]] };
    if (fa.bc != NOSLIP && fa.bc != SLIP && fa.bc != OUTFLOW) continue;  // periodic: no-op
    const int a1 = (fa.axis == 0) ? 1 : 0, a2 = (fa.axis == 2) ? 1 : 2;
    dim3 blk(32, 8);
    dim3 grd((n[a1] + 31) / 32, (n[a2] + 7) / 8);
    k_face<<<grd, blk, 0, stream()>>>(fa, u, v, w);
    if (!launched("k_face")) return false;
  }
  return true;
}

bool launch_special(const Dims &g, int problem, double lid, double inflow, double *u)
{
  dim3 blk(32, 8);
  if (problem == PROBLEM_DCAVITY) {
    if (g.imax < 2 || g.kmax < 2) return true;
    dim3 grd((g.imax - 1 + 31) / 32, (g.kmax - 1 + 7) / 8);
    k_lid<<<grd, blk, 0, stream()>>>(g, 2.0 * lid, u);
    return launched("k_lid");
  }
  if (problem == PROBLEM_CANAL) {
    dim3 grd((g.jmax + 31) / 32, (g.kmax + 7) / 8);
    k_inflow<<<grd, blk, 0, stream()>>>(g, inflow, u);
    return launched("k_inflow");
  }
  return true;
}

bool launch_fgh(const Dims &g, double re, double gamma, double gx, double gy, double gz,
    double dt, double dx, double dy, double dz, const double *u, const double *v,
    const double *w, double *f, double *gg, double *h, const StepScalars *sp, int kb_fixed,
    bool fp64)
{
  FluxArgs A;
  A.g = g;
  const double inv[3] = { 1.0 / dx, 1.0 / dy, 1.0 / dz };
  const double iRe = 1.0 / re;
  FaceCoef *fc[3] = { &A.ax, &A.ay, &A.az };
  for (int a = 0; a < 3; a++) {
    const double c1 = inv[a] * 0.25, c2 = gamma * inv[a] * 0.25;
    fc[a]->P = c1 + c2;
    fc[a]->M = c1 - c2;
    fc[a]->nu = iRe * (inv[a] * inv[a]);
  }
  A.dt = dt;
  A.gx = gx;
  A.gy = gy;
  A.gz = gz;
  A.sp = sp;
  const int gx_blocks = (g.imax + kFX - 1) / kFX, gy_blocks = (g.jmax + kFY - 1) / kFY;
  int kb = 32;
  while (kb > 1 && (int64_t)gx_blocks * gy_blocks * ((g.kmax + kb - 1) / kb) < 8 * sm_count())
    kb >>= 1;
  if (kb_fixed > 0) kb = kb_fixed;
  A.kb = kb;
  dim3 grid(gx_blocks, gy_blocks, (g.kmax + kb - 1) / kb);
  const bool gravity = !(gx == 0.0 && gy == 0.0 && gz == 0.0);
  if (fp64) {
    if (!gravity)
      k_fgh_flux<false><<<grid, dim3(kFX, kFY), 0, stream()>>>(A, u, v, w, f, gg, h);
    else
      k_fgh_flux<true><<<grid, dim3(kFX, kFY), 0, stream()>>>(A, u, v, w, f, gg, h);
    return launched("k_fgh_flux");
  }
  static_assert(kDX == kFX && kDY == kFY, "both computeFG kernels share one tiling");
  FluxArgsDF D;
  D.g = g;
  df::AxisCoef *dc[3] = { &D.ax, &D.ay, &D.az };
  for (int a = 0; a < 3; a++) *dc[a] = df::axis_coef(fc[a]->P, fc[a]->M, fc[a]->nu);
  D.gx = df::from_double_rn(gx);
  D.gy = df::from_double_rn(gy);
  D.gz = df::from_double_rn(gz);
  D.dt = dt;
  D.sp = sp;
  D.kb = kb;
  // the kernel's shared memory (49.4 KB) is above the 48 KB default: opt in once per device
  static bool attr_set[64] = {};
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return false;
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    if (!cuda_ok(cudaFuncSetAttribute(k_fgh_df<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                     (int)kDfSmemBytes),
            "k_fgh_df<false> shared memory") ||
        !cuda_ok(cudaFuncSetAttribute(k_fgh_df<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                     (int)kDfSmemBytes),
            "k_fgh_df<true> shared memory"))
      return false;
    attr_set[dev] = true;
  }
  if (!gravity)
    k_fgh_df<false><<<grid, dim3(kDX, kDY), kDfSmemBytes, stream()>>>(D, u, v, w, f, gg, h);
  else
    k_fgh_df<true><<<grid, dim3(kDX, kDY), kDfSmemBytes, stream()>>>(D, u, v, w, f, gg, h);
  return launched("k_fgh_df");
}

bool launch_rhs(const Dims &g, double dt, double dx, double dy, double dz, const double *f,
    const double *gg, const double *h, double *rhs, const StepScalars *sp)
{
  const double idt = sp ? 0.0 : 1.0 / dt;
  k_rhs<<<cell_grid(g, kCellBlock), kCellBlock, 0, stream()>>>(
      g, (1.0 / dx) * idt, (1.0 / dy) * idt, (1.0 / dz) * idt, sp, f, gg, h, rhs);
  return launched("k_rhs");
}

bool launch_interior_sum(const Dims &g, const double *p, ReduceScratch &red, double *d_out)
{
  int blocks = 4 * sm_count();
  if (!reduce_scratch_alloc(red, 3 * blocks)) return false;
  k_interior_sum<<<blocks, kBlock, 0, stream()>>>(g, p, red.partials, red.ticket, d_out);
  return launched("k_interior_sum");
}

bool launch_subtract_mean(const Dims &g, double *p, const double *d_mean)
{
  k_subtract_mean<<<cell_grid(g, kCellBlock), kCellBlock, 0, stream()>>>(g, p, d_mean);
  return launched("k_subtract_mean");
}

bool launch_adapt_uv(const Dims &g, double dt, double dx, double dy, double dz,
    const double *f, const double *gg, const double *h, const double *p, double *u, double *v,
    double *w, const StepScalars *sp, unsigned long long *amax_slots)
{
  if (amax_slots)
    k_adapt<true><<<cell_grid(g, kCellBlock), kCellBlock, 0, stream()>>>(
        g, dt / dx, dt / dy, dt / dz, sp, f, gg, h, p, u, v, w, amax_slots);
  else
    k_adapt<false><<<cell_grid(g, kCellBlock), kCellBlock, 0, stream()>>>(
        g, dt / dx, dt / dy, dt / dz, sp, f, gg, h, p, u, v, w, nullptr);
  return launched("k_adapt");
}

bool launch_shell_max3(const Dims &g, const double *u, const double *v, const double *w,
    unsigned long long *amax_slots, ReduceScratch &red, double *d_out3)
{
  const int64_t shell = 2 * (int64_t)g.sk + (int64_t)g.kmax * 2 * (g.imax + 2) +
                        (int64_t)g.kmax * g.jmax * 2;
  int blocks = (int)std::min<int64_t>(4 * sm_count(), (shell + kBlock - 1) / kBlock);
  if (blocks < 1) blocks = 1;
  if (!reduce_scratch_alloc(red, 3 * blocks)) return false;
  k_shell_max3<<<blocks, kBlock, 0, stream()>>>(g, u, v, w, amax_slots, red.partials, red.ticket,
      d_out3);
  return launched("k_shell_max3");
}

bool launch_fill(double *a, int64_t n, double value)
{
  k_fill<<<4 * sm_count(), kBlock, 0, stream()>>>(a, n, value);
  return launched("k_fill");
}

int problem_code(const char *name)
{
  if (name == nullptr) return PROBLEM_NONE;
  if (strcmp(name, "dcavity") == 0) return PROBLEM_DCAVITY;
  if (strcmp(name, "canal") == 0) return PROBLEM_CANAL;
  return PROBLEM_NONE;
}

}  // namespace nusif

using namespace nusif;

namespace {

// the launch stream waits for queued asynchronous copies of the fields an
// entry point reads (their uploads) and writes (every copy)
bool await_arrays(std::initializer_list<const double *> reads,
    std::initializer_list<const double *> writes)
{
  const void *r[8], *w[8];
  int nr = 0, nw = 0;
  for (const double *x : reads) r[nr++] = x;
  for (const double *x : writes) w[nw++] = x;
  return await_uploads(r, nr) && await_copies(w, nw);
}

DiscState *need_state(const Discretization *d, const char *what)
{
  DiscState *st = disc_state(d);
  if (!st) fail(NUSIF_ERR_STATE, "%s: discretization not initialised by initDiscretization", what);
  return st;
}

bool verbose()
{
  const char *v = getenv("NUSIF_VERBOSE");
  return v && v[0] && v[0] != '0';
}

// printConfig, reference src/discretization.c:16-47 (printed when NUSIF_VERBOSE is set)
void print_config(const Discretization *s)
{
  printf("Parameters for #%s#\n", s->problem);
  printf("BC Left:%d Right:%d Bottom:%d Top:%d Front:%d Back:%d\n", s->bcLeft, s->bcRight,
      s->bcBottom, s->bcTop, s->bcFront, s->bcBack);
  printf("\tReynolds number: %.2f\n", s->re);
  printf("\tGx Gy: %.2f %.2f %.2f\n", s->gx, s->gy, s->gz);
  printf("Geometry data:\n");
  printf("\tDomain box size (x, y, z): %.2f, %.2f, %.2f\n", s->grid.xlength, s->grid.ylength,
      s->grid.zlength);
  printf("\tCells (x, y, z): %d, %d, %d\n", s->grid.imax, s->grid.jmax, s->grid.kmax);
  printf("\tCell size (dx, dy, dz): %f, %f, %f\n", s->grid.dx, s->grid.dy, s->grid.dz);
  printf("Timestep parameters:\n");
  printf("\tDefault stepsize: %.2f, Final time %.2f\n", s->dt, s->te);
  printf("\tdt bound: %.6f\n", s->dtBound);
  printf("\tTau factor: %.2f\n", s->tau);
  printf("Iterative parameters:\n");
  printf("\tMax iterations: %d\n", s->itermax);
  printf("\tepsilon (stopping tolerance) : %f\n", s->eps);
  printf("\tgamma factor: %f\n", s->gamma);
  printf("\tomega (SOR relaxation): %f\n", s->omega);
}

}  // namespace

extern "C" {

// initDiscretization, reference src/discretization.c:49-117
void initDiscretization(Discretization *s, Parameter *params)
{
  if (!s || !params) {
    fail(NUSIF_ERR_ARG, "initDiscretization: null argument");
    return;
  }
  if (params->imax < 1 || params->jmax < 1 || params->kmax < 1) {
    fail(NUSIF_ERR_ARG, "initDiscretization: grid %d x %d x %d is empty", params->imax,
        params->jmax, params->kmax);
    return;
  }
  const int64_t padded = (int64_t)(params->imax + 2) * (params->jmax + 2) * (params->kmax + 2);
  if (padded >= ((int64_t)1 << 31)) {
    fail(NUSIF_ERR_ARG, "initDiscretization: %lld padded cells exceed the 2^31 index range",
        (long long)padded);
    return;
  }
  if (disc_state(s)) nusifFreeDiscretization(s);

  s->problem = params->name;
  s->bcLeft = params->bcLeft;
  s->bcRight = params->bcRight;
  s->bcBottom = params->bcBottom;
  s->bcTop = params->bcTop;
  s->bcFront = params->bcFront;
  s->bcBack = params->bcBack;

  s->grid.imax = params->imax;
  s->grid.jmax = params->jmax;
  s->grid.kmax = params->kmax;
  s->grid.xlength = params->xlength;
  s->grid.ylength = params->ylength;
  s->grid.zlength = params->zlength;
  s->grid.dx = params->xlength / params->imax;
  s->grid.dy = params->ylength / params->jmax;
  s->grid.dz = params->zlength / params->kmax;

  s->eps = params->eps;
  s->omega = params->omg;
  s->itermax = params->itermax;
  s->re = params->re;
  s->gx = params->gx;
  s->gy = params->gy;
  s->gz = params->gz;
  s->dt = params->dt;
  s->te = params->te;
  s->tau = params->tau;
  s->gamma = params->gamma;

  DiscState *st = disc_state_create(s);
  st->dims = make_dims(params->imax, params->jmax, params->kmax);
  const Extras *x = extras_for(params, false);
  st->ext = x ? *x : Extras();

  const size_t bytes = sizeof(double) * (size_t)padded;
  double **fields[8] = { &s->u, &s->v, &s->w, &s->p, &s->rhs, &s->f, &s->g, &s->h };
  for (int q = 0; q < 8; q++) {
    *fields[q] = nullptr;
    if (st->ext.host_fields) {
      // host_fields: managed memory kept in HBM, so that host code (the
      // reference's output stage) can read the fields through these pointers
      if (!cuda_ok(cudaMallocManaged(fields[q], bytes, cudaMemAttachGlobal),
              "cudaMallocManaged(field)"))
        return;
      int dev = 0;
      cudaGetDevice(&dev);
      cudaMemLocation loc = {};
      loc.type = cudaMemLocationTypeDevice;
      loc.id = dev;
      if (!cuda_ok(cudaMemAdvise(*fields[q], bytes, cudaMemAdviseSetPreferredLocation, loc),
              "cudaMemAdvise(field)"))
        return;
    } else if (!cuda_ok(cudaMalloc(fields[q], bytes), "cudaMalloc(field)")) {
      return;
    }
  }
  if (!cuda_ok(cudaMalloc(&st->d_scalars, 8 * sizeof(double)), "cudaMalloc(scalars)")) return;
  const size_t amax_bytes = 3 * kAmaxSlots * sizeof(unsigned long long);
  if (!cuda_ok(cudaMalloc(&st->d_amax, amax_bytes), "cudaMalloc(amax)")) return;
  if (!cuda_ok(cudaMemsetAsync(st->d_amax, 0, amax_bytes, stream()), "cudaMemsetAsync(amax)"))
    return;
  st->amax = kAmaxReset;
  if (!cuda_ok(cudaMallocHost(&st->h_scalars, 8 * sizeof(double)), "cudaMallocHost(scalars)"))
    return;
  const double init[4] = { params->u_init, params->v_init, params->w_init, params->p_init };
  for (int q = 0; q < 4; q++)
    if (!launch_fill(*fields[q], padded, init[q])) return;
  for (int q = 4; q < 8; q++)
    if (!cuda_ok(cudaMemsetAsync(*fields[q], 0, bytes, stream()), "cudaMemsetAsync(field)"))
      return;
  cuda_ok(cudaStreamSynchronize(stream()), "initDiscretization sync");

  const double dx = s->grid.dx, dy = s->grid.dy, dz = s->grid.dz;
  const double invSqrSum = 1.0 / (dx * dx) + 1.0 / (dy * dy) + 1.0 / (dz * dz);
  s->dtBound = 0.5 * s->re * 1.0 / invSqrSum;
  if (verbose()) print_config(s);
}

// computeTimestep, reference src/discretization.c:431-453: the three maxima
// come from the device, the dt arithmetic stays on the host.
void computeTimestep(Discretization *s)
{
  DiscState *st = need_state(s, "computeTimestep");
  if (!st || !await_arrays({ s->u, s->v, s->w }, {})) return;
  if (st->ext.fuse_dt && st->amax == kAmaxValid) {
    // the interior maxima came with the last adaptUV: read the ghost shell only
    if (!launch_shell_max3(st->dims, s->u, s->v, s->w, st->d_amax, st->red, st->d_scalars))
      return;
    st->dt_shell++;
  } else {
    if (!launch_max3(st->dims, s->u, s->v, s->w, st->red, st->d_scalars)) return;
    st->dt_full++;
    if (st->amax != kAmaxReset &&
        !cuda_ok(cudaMemsetAsync(st->d_amax, 0, 3 * kAmaxSlots * sizeof(unsigned long long),
                     stream()),
            "computeTimestep reset"))
      return;
  }
  st->amax = kAmaxReset;
  if (!cuda_ok(cudaMemcpyAsync(st->h_scalars, st->d_scalars, 3 * sizeof(double),
                   cudaMemcpyDeviceToHost, stream()),
          "computeTimestep copy"))
    return;
  if (!cuda_ok(cudaStreamSynchronize(stream()), "computeTimestep sync")) return;
  const double umax = st->h_scalars[0], vmax = st->h_scalars[1], wmax = st->h_scalars[2];
  double dt = s->dtBound;
  const double dx = s->grid.dx, dy = s->grid.dy, dz = s->grid.dz;
  if (umax > 0) dt = (dt > dx / umax) ? dx / umax : dt;
  if (vmax > 0) dt = (dt > dy / vmax) ? dy / vmax : dt;
  if (wmax > 0) dt = (dt > dz / wmax) ? dz / wmax : dt;
  s->dt = dt * s->tau;
}

void setBoundaryConditions(Discretization *s)
{
  DiscState *st = need_state(s, "setBoundaryConditions");
  if (!st || !await_arrays({}, { s->u, s->v, s->w })) return;
  const int bc[6] = { s->bcLeft, s->bcRight, s->bcBottom, s->bcTop, s->bcFront, s->bcBack };
  velocity_written(st);
  launch_bc(st->dims, bc, PROBLEM_NONE, 0.0, 0.0, s->u, s->v, s->w);
}

// the problem is matched by name at every call, as in the reference
void setSpecialBoundaryCondition(Discretization *s)
{
  DiscState *st = need_state(s, "setSpecialBoundaryCondition");
  if (!st || !await_arrays({}, { s->u })) return;
  velocity_written(st);
  launch_special(st->dims, problem_code(s->problem), st->ext.lid, st->ext.inflow, s->u);
}

void computeFG(Discretization *s)
{
  DiscState *st = need_state(s, "computeFG");
  if (!st || !await_arrays({ s->u, s->v, s->w }, { s->f, s->g, s->h })) return;
  launch_fgh(st->dims, s->re, s->gamma, s->gx, s->gy, s->gz, s->dt, s->grid.dx, s->grid.dy,
      s->grid.dz, s->u, s->v, s->w, s->f, s->g, s->h, nullptr, 0, st->ext.fg_fp64 != 0);
}

void computeRHS(Discretization *s)
{
  DiscState *st = need_state(s, "computeRHS");
  if (!st || !await_arrays({ s->f, s->g, s->h }, { s->rhs })) return;
  launch_rhs(st->dims, s->dt, s->grid.dx, s->grid.dy, s->grid.dz, s->f, s->g, s->h, s->rhs);
}

void normalizePressure(Discretization *s)
{
  DiscState *st = need_state(s, "normalizePressure");
  if (!st || !await_arrays({}, { s->p })) return;
  if (!launch_interior_sum(st->dims, s->p, st->red, st->d_scalars + 3)) return;
  launch_subtract_mean(st->dims, s->p, st->d_scalars + 4);
}

void adaptUV(Discretization *s)
{
  DiscState *st = need_state(s, "adaptUV");
  if (!st || !await_arrays({ s->f, s->g, s->h, s->p }, { s->u, s->v, s->w })) return;
  // fuse_dt: the first adaptUV after computeTimestep keeps the maxima of what it writes
  // (not with host_fields, whose arrays host code may write directly)
  const bool keep = st->ext.fuse_dt && !st->ext.host_fields && st->amax == kAmaxReset;
  if (!launch_adapt_uv(st->dims, s->dt, s->grid.dx, s->grid.dy, s->grid.dz, s->f, s->g, s->h,
          s->p, s->u, s->v, s->w, nullptr, keep ? st->d_amax : nullptr))
    return;
  if (keep) st->amax = kAmaxValid;
  else velocity_written(st);
}

int nusifTimestepCounts(const Discretization *s, long long *shell, long long *full)
{
  const DiscState *st = disc_state(s);
  if (!st) {
    fail(NUSIF_ERR_ARG, "nusifTimestepCounts: unknown discretization");
    return NUSIF_ERR_ARG;
  }
  if (shell) *shell = st->dt_shell;
  if (full) *full = st->dt_full;
  return NUSIF_OK;
}

void nusifFreeDiscretization(Discretization *s)
{
  DiscState *st = disc_state(s);
  if (!st) return;
  await_fields(s);
  cudaStreamSynchronize(stream());
  double **fields[8] = { &s->u, &s->v, &s->w, &s->p, &s->rhs, &s->f, &s->g, &s->h };
  for (int q = 0; q < 8; q++) {
    if (*fields[q]) cudaFree(*fields[q]);
    *fields[q] = nullptr;
  }
  if (st->d_scalars) cudaFree(st->d_scalars);
  if (st->d_amax) cudaFree(st->d_amax);
  if (st->h_scalars) cudaFreeHost(st->h_scalars);
  reduce_scratch_free(st->red);
  disc_state_erase(s);
}

}  // extern "C"
