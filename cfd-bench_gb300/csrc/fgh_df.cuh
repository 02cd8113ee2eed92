// computeFG face fluxes in double-float arithmetic (df32.cuh).
//
// The same flux form as the FP64 kernel (discretization.cu): the donor-cell
// convective term and the viscous term of one component across one face are
// A*q_a + B*q_b with A = cp*(c1 +- c2) + nu, B = cp*(c1 -+ c2) - nu, cp the
// doubled transport velocity on the face, the signs picked by the sign of cp
// (reference src/discretization.c:488-597: du2dx, duvdy, duwdz, ... and the
// second differences). Every term of F, G, H is a difference of such fluxes,
// except the z-convection of G, whose "minus" half keeps the reference's
// V(i,j,k+1) (discretization.c:543-550).
//
// Host and device: the CPU checks of the arithmetic call the same functions.
#pragma once

#include "df32.cuh"

namespace nusif {
namespace df {

// per-axis constants of the face fluxes as pairs: P = c1 + c2, M = c1 - c2,
// nu = (1/Re)/h^2, with c1 = 0.25/h, c2 = gamma*0.25/h
struct AxisCoef {
  f2 P, M, nu, mnu;
};

DF_FN AxisCoef axis_coef(double P, double M, double nu)
{
  AxisCoef a;
  a.P = from_double_rn(P);
  a.M = from_double_rn(M);
  a.nu = from_double_rn(nu);
  a.mnu = neg(a.nu);
  return a;
}

// total flux of q across a face between qa (minus side) and qb (plus side),
// transported by the doubled velocity cp
DF_FN f2 face_flux(const AxisCoef &a, f2 cp, f2 qa, f2 qb)
{
  const bool negative = f32_bits(cp.hi) >> 31;  // cp is renormalised: hi carries the sign
  const f2 A = fma_u(cp, negative ? a.M : a.P, a.nu);
  const f2 B = fma_u(cp, negative ? a.P : a.M, a.mnu);
  return dot2_u(A, qa, B, qb);
}

// the three components' fluxes across one x-, y- or z-face
struct Face {
  f2 f, g, h;
};

// G's z-face: viscous part and transport velocity (the convective part needs
// the cell's own v on both sides, the dvwdz quirk)
struct ZFaceG {
  f2 gv, gc;
};

// the 2 x 2 x 2 neighbourhood a cell's plus faces read: q[c], q[c+1], q[c+sj], q[c+sk]
struct Quad {
  f2 c, x, y, z;
};

DF_FN Face x_face(const AxisCoef &a, const Quad &u, const Quad &v, const Quad &w)
{
  Face r;
  r.f = face_flux(a, add(u.c, u.x), u.c, u.x);
  r.g = face_flux(a, add(u.c, u.y), v.c, v.x);
  r.h = face_flux(a, add(u.c, u.z), w.c, w.x);
  return r;
}

DF_FN Face y_face(const AxisCoef &a, const Quad &u, const Quad &v, const Quad &w)
{
  Face r;
  r.f = face_flux(a, add(v.c, v.x), u.c, u.y);
  r.g = face_flux(a, add(v.c, v.y), v.c, v.y);
  r.h = face_flux(a, add(v.c, v.z), w.c, w.y);
  return r;
}

// F and H fluxes across the z-face, and G's viscous flux and transport velocity
DF_FN Face z_face(const AxisCoef &a, const Quad &u, const Quad &v, const Quad &w, ZFaceG &gz)
{
  Face r;
  r.f = face_flux(a, add(w.c, w.x), u.c, u.z);
  r.h = face_flux(a, add(w.c, w.z), w.c, w.z);
  r.g = f2{ 0.0f, 0.0f };
  gz.gv = mul_u(a.nu, sub_u(v.c, v.z));
  gz.gc = add(w.c, w.y);
  return r;
}

// G's z-convection: c1*(vc + vt)*(gp - gm) + c2*(vc - vt)*(|gp| + |gm|) as
// gp*Xp - gm*Xm, Xp and Xm weighted sums of vc and vt (vt = v[c+sk]) chosen
// by the signs of gp and gm
DF_FN f2 g_zconv(const AxisCoef &a, f2 gp, f2 gm, f2 vc, f2 vt)
{
  const bool np = f32_bits(gp.hi) >> 31, nm = f32_bits(gm.hi) >> 31;
  const f2 xp = dot2_u(np ? a.M : a.P, vc, np ? a.P : a.M, vt);
  const f2 xm = dot2_u(nm ? a.P : a.M, vc, nm ? a.M : a.P, vt);
  return dot2_u(gp, xp, neg(gm), xm);
}

// q + dt * (g - s) as a binary64 number: the flux sum s and the gravity g as
// pairs, q exact (mdt = -dt as a pair; two FP64 adds)
DF_FN double update(double q, f2 s, f2 g, f2 mdt, bool gravity)
{
  const f2 t = gravity ? sub_u(s, g) : s;
  const f2 d = mul(t, mdt);
  return (q + widen(d.hi)) + widen(d.lo);
}

}  // namespace df
}  // namespace nusif
