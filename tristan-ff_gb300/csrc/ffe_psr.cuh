// ffe_psr.cuh — the rotating-conductor boundary condition of user/user_psr.F90
// as per-cell device functions, shared by the staged kernel (ffe_staged.cu)
// and the fused path's fix-up (ffe_fused.cu).  An accessor a(c, di, dj, dk)
// supplies the (updated, not yet cleaned) fields around the cell.
#pragma once
#include "ffe_physics.cuh"

namespace ffe {

// getDipole (user_psr.F90:345-374); the moment mu is evaluated per step on the host.
template <typename R>
__device__ __forceinline__ void psr_dipole(const PsrBC<R>& q, R x_g, R y_g, R z_g, R& obx, R& oby, R& obz) {
  R nx = x_g - q.xc, ny = y_g - q.yc, nz = z_g - q.zc;
  R rr = R(1.0) / sqrt((nx * nx + ny * ny) + nz * nz);
  nx = nx * rr;
  ny = ny * rr;
  nz = nz * rr;
  rr = (rr * rr) * rr;
  const R mdn = (q.mu[0] * nx + q.mu[1] * ny) + q.mu[2] * nz;
  obx = (R(3.0) * nx * mdn - q.mu[0]) * rr;
  oby = (R(3.0) * ny * mdn - q.mu[1]) * rr;
  obz = (R(3.0) * nz * mdn - q.mu[2]) * rr;
}

// shape() (user_psr.F90:376-383)
template <typename R>
__device__ __forceinline__ R psr_shape(R rad, R rad0) { return R(0.5) * (R(1.0) - tanh((rad - rad0) / R(1.0))); }

// r < 2R test of the BC loops (user_psr.F90:153,311)
template <typename R>
__device__ __forceinline__ bool psr_inside(const PsrBC<R>& q, const Phys& p, int i, int j, int k) {
  const R ig = R(i + p.x0), jg = R(j + p.y0), kg = R(k + p.z0);
  return ((ig - q.xc) * (ig - q.xc) + (jg - q.yc) * (jg - q.yc)) + (kg - q.zc) * (kg - q.zc) < q.sr2;
}

// New B component comp at a staggered point (user_psr.F90:157-214).
template <typename R>
__device__ __forceinline__ R psr_newB(const PsrBC<R>& q, R rx, R ry, R rz, R bint, R bown, int comp) {
  const R rr_sqr = (rx * rx + ry * ry) + rz * rz;
  R bdx, bdy, bdz;
  psr_dipole(q, rx + q.xc, ry + q.yc, rz + q.zc, bdx, bdy, bdz);
  const R bdip = (bdx * rx + bdy * ry) + bdz * rz;
  const R rc = comp == 0 ? rx : (comp == 1 ? ry : rz);
  const R bd = comp == 0 ? bdx : (comp == 1 ? bdy : bdz);
  const R shift_B = R(4.0), scaleBperp = R(0.5), scaleBpar = R(0.25);
  R sc = R(1.0) / scaleBperp;
  R sh = psr_shape(sqrt(rr_sqr) * sc, (q.radius - shift_B) * sc);
  const R v = (bint - bdip) * (rc / rr_sqr) * (R(1.0) - sh);
  sc = R(1.0) / scaleBpar;
  sh = psr_shape(sqrt(rr_sqr) * sc, (q.radius - shift_B) * sc);
  return (v + bd) + ((bown - bint * rc / rr_sqr) - (bd - bdip * rc / rr_sqr)) * (R(1.0) - sh);
}

// New E component comp at a staggered point (user_psr.F90:219-297).
template <typename R>
__device__ __forceinline__ R psr_newE(const PsrBC<R>& q, R rx, R ry, R rz, R eint, R eown, int comp) {
  const R rr_sqr = (rx * rx + ry * ry) + rz * rz;
  R bdx, bdy, bdz;
  psr_dipole(q, rx + q.xc, ry + q.yc, rz + q.zc, bdx, bdy, bdz);
  const R vx = -(q.omega * ry), vy = q.omega * rx, vz = R(0.0);
  const R exd = -(vy * bdz - vz * bdy) * q.ccinv;
  const R eyd = (vx * bdz - vz * bdx) * q.ccinv;
  const R ezd = -(vx * bdy - vy * bdx) * q.ccinv;
  const R edip = (exd * rx + eyd * ry) + ezd * rz;
  const R rc = comp == 0 ? rx : (comp == 1 ? ry : rz);
  const R ed = comp == 0 ? exd : (comp == 1 ? eyd : ezd);
  const R shift_E = R(0.0), scaleEpar = R(0.5), scaleEperp = R(0.25);
  R sc = R(1.0) / scaleEpar;
  R sh = psr_shape(sqrt(rr_sqr) * sc, (q.radius - shift_E) * sc);
  const R v = ed + ((eown - eint * rc / rr_sqr) - (ed - edip * rc / rr_sqr)) * (R(1.0) - sh);
  sc = R(1.0) / scaleEperp;
  sh = psr_shape(sqrt(rr_sqr) * sc, (q.radius - shift_E) * sc);
  return v + (eint - edip) * (rc / rr_sqr) * (R(1.0) - sh);
}

// All six new values of local cell (i, j, k), which must satisfy psr_inside
// (user_psr.F90:155-298).  Output order: ex ey ez bx by bz.
template <typename R, class A>
__device__ __forceinline__ void psr_cell(const PsrBC<R>& q, const Phys& p, const A& a, int i, int j, int k, R o[6]) {
  const R ig = R(i + p.x0), jg = R(j + p.y0), kg = R(k + p.z0), h = R(0.5);
  R rx, ry, rz, in;
  // B_x (:157-174)
  rx = ig - q.xc; ry = (jg + h) - q.yc; rz = (kg + h) - q.zc;
  in = (a(BX, 0, 0, 0) * rx + R(0.25) * (((a(BY, 0, 0, 0) + a(BY, 0, 1, 0)) + a(BY, -1, 0, 0)) + a(BY, -1, 1, 0)) * ry) +
       R(0.25) * (((a(BZ, 0, 0, 0) + a(BZ, 0, 0, 1)) + a(BZ, -1, 0, 0)) + a(BZ, -1, 0, 1)) * rz;
  o[3] = psr_newB(q, rx, ry, rz, in, a(BX, 0, 0, 0), 0);
  // B_y (:177-194)
  rx = (ig + h) - q.xc; ry = jg - q.yc; rz = (kg + h) - q.zc;
  in = (R(0.25) * (((a(BX, 0, 0, 0) + a(BX, 1, 0, 0)) + a(BX, 0, -1, 0)) + a(BX, 1, -1, 0)) * rx + a(BY, 0, 0, 0) * ry) +
       R(0.25) * (((a(BZ, 0, 0, 0) + a(BZ, 0, 0, 1)) + a(BZ, 0, -1, 0)) + a(BZ, 0, -1, 1)) * rz;
  o[4] = psr_newB(q, rx, ry, rz, in, a(BY, 0, 0, 0), 1);
  // B_z (:197-214)
  rx = (ig + h) - q.xc; ry = (jg + h) - q.yc; rz = kg - q.zc;
  in = (R(0.25) * (((a(BX, 0, 0, 0) + a(BX, 1, 0, 0)) + a(BX, 0, 0, -1)) + a(BX, 1, 0, -1)) * rx +
        R(0.25) * (((a(BY, 0, 0, 0) + a(BY, 0, 1, 0)) + a(BY, 0, 0, -1)) + a(BY, 0, 1, -1)) * ry) +
       a(BZ, 0, 0, 0) * rz;
  o[5] = psr_newB(q, rx, ry, rz, in, a(BZ, 0, 0, 0), 2);
  // E_x (:219-243)
  rx = (ig + h) - q.xc; ry = jg - q.yc; rz = kg - q.zc;
  in = (a(EX, 0, 0, 0) * rx + R(0.25) * (((a(EY, 0, 0, 0) + a(EY, 1, 0, 0)) + a(EY, 0, -1, 0)) + a(EY, 1, -1, 0)) * ry) +
       R(0.25) * (((a(EZ, 0, 0, 0) + a(EZ, 1, 0, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 1, 0, -1)) * rz;
  o[0] = psr_newE(q, rx, ry, rz, in, a(EX, 0, 0, 0), 0);
  // E_y (:246-270)
  rx = ig - q.xc; ry = (jg + h) - q.yc; rz = kg - q.zc;
  in = (R(0.25) * (((a(EX, 0, 0, 0) + a(EX, 0, 1, 0)) + a(EX, -1, 0, 0)) + a(EX, -1, 1, 0)) * rx + a(EY, 0, 0, 0) * ry) +
       R(0.25) * (((a(EZ, 0, 0, 0) + a(EZ, 0, 1, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 0, 1, -1)) * rz;
  o[1] = psr_newE(q, rx, ry, rz, in, a(EY, 0, 0, 0), 1);
  // E_z (:273-297)
  rx = ig - q.xc; ry = jg - q.yc; rz = (kg + h) - q.zc;
  in = (R(0.25) * (((a(EX, 0, 0, 0) + a(EX, 0, 0, 1)) + a(EX, -1, 0, 0)) + a(EX, -1, 0, 1)) * rx +
        R(0.25) * (((a(EY, 0, 0, 0) + a(EY, 0, -1, 0)) + a(EY, 0, 0, 1)) + a(EY, 0, -1, 1)) * ry) +
       a(EZ, 0, 0, 0) * rz;
  o[2] = psr_newE(q, rx, ry, rz, in, a(EZ, 0, 0, 0), 2);
}

// The twisted-footpoint BC of user/user_uniform.F90:114-142 at local cell
// (i, j, k): on z_glob <= 0 it sets Ex, Ey to the rotating drive and Bz to the
// tube profile, on z_glob >= gsz it resets Bz and zeroes Ex, Ey.  Pure
// functions of position and time, so it applies to one cell at a time.
template <typename R>
__device__ __forceinline__ void uniform_bc_apply(const UniformBC<R>& u, const Phys& p, int i, int j, int k, R& ex,
                                                 R& ey, R& bz) {
  const R xg = R(i + p.x0), yg = R(j + p.y0), zg = R(k + p.z0), h = R(0.5);
  R rx, ry, rr, omega, ee0;
  if (zg <= R(0)) {
    rx = (xg + h) - u.xc; ry = yg - u.yc;
    rr = sqrt((rx * rx + ry * ry) + tiny<R>());
    omega = exp(-rr / u.r0) * u.beta * u.cc / u.r0;
    ee0 = -omega * u.bnorm * u.tanh_t;
    ex = rx * ee0;
    rx = xg - u.xc; ry = (yg + h) - u.yc;
    rr = sqrt((rx * rx + ry * ry) + tiny<R>());
    omega = exp(-rr / u.r0) * u.beta * u.cc / u.r0;
    ee0 = -omega * u.bnorm * u.tanh_t;
    ey = ry * ee0;
    rx = (xg + h) - u.xc; ry = (yg + h) - u.yc;
    rr = sqrt((rx * rx + ry * ry) + tiny<R>());
    bz = u.bnorm / (R(1.0) + (rr / u.r0));
  }
  if (zg >= R(p.gsz)) {
    rx = (xg + h) - u.xc; ry = (yg + h) - u.yc;
    rr = sqrt((rx * rx + ry * ry) + tiny<R>());
    bz = u.bnorm / (R(1.0) + (rr / u.r0));
    ex = R(0.0);
    ey = R(0.0);
  }
}

}  // namespace ffe
