// ffe_physics.cuh — per-cell arithmetic of the force-free update, written once
// and used by both kernel families:
//   * the staged kernels (ffe_staged.cu, one launch per reference procedure,
//     compiled without multiply-add contraction so that they reproduce the
//     reference's rounding), and
//   * the fused stage kernels (ffe_fused.cu), which read the same neighbours
//     from shared-memory tiles.
// A kernel supplies an accessor `a` with a(F, di, dj, dk) -> value of field F
// at offset (di, dj, dk) from the current cell and a.rho(di, dj, dk).
//
// Every expression keeps the Fortran association of
// src/algorithms/field_solver.F90 (left to right); line numbers cite that file.
#pragma once
#include "ffe_common.cuh"

namespace ffe {

enum { EX = 0, EY, EZ, BX, BY, BZ, B0X, B0Y, B0Z };

template <typename R> __host__ __device__ __forceinline__ R tiny() { return R(1e-7); }
template <> __host__ __device__ __forceinline__ float tiny<float>() { return 1e-7f; }  // src/defs.F90:4

// rho = div E at offset d (field_solver.F90:57-59)
template <typename R, class A>
__device__ __forceinline__ R rho_at(const A& a, int di, int dj, int dk) {
  return ((a(EX, di, dj, dk) - a(EX, di - 1, dj, dk)) + (a(EY, di, dj, dk) - a(EY, di, dj - 1, dk))) +
         (a(EZ, di, dj, dk) - a(EZ, di, dj, dk - 1));
}

// Quotient x / y: correctly rounded, or (FD, float only) the two-instruction
// reciprocal-multiply of __fdividef (<= 2 ulp) used by the fast fused path.
template <typename R, bool FD>
__device__ __forceinline__ R qdiv(R x, R y) {
  if constexpr (FD && sizeof(R) == 4) return __fdividef(x, y);
  else return x / y;
}

// J = CC rho (E x B) / (B^2 + TINY) with the denominator in R, or in double (FP32C).
template <typename R, int C, bool FD = false>
__device__ __forceinline__ R jdiv(R cc, R bmag, R bx, R by, R bz, R num) {
  if (C == 2) {
    const double bd = ((double)bx * (double)bx + (double)by * (double)by) + (double)bz * (double)bz;
    return (R)((double)cc / (bd + (double)tiny<float>()) * (double)num);
  }
  return qdiv<R, FD>(cc, bmag + tiny<R>()) * num;
}

// rk3Push (field_solver.F90:81-162): writes dE (with -J) and dB of one cell.
template <typename R, int C, bool B0, class A, bool FD = false>
__device__ __forceinline__ void push_cell(const A& a, R cc, R d[6]) {
  const R ey0 = a(EY, 0, 0, 0), ez0 = a(EZ, 0, 0, 0), ex0 = a(EX, 0, 0, 0);
  const R bx0 = a(BX, 0, 0, 0), by0 = a(BY, 0, 0, 0), bz0 = a(BZ, 0, 0, 0);
  d[3] = cc * ((a(EY, 0, 0, 1) - ey0) - (a(EZ, 0, 1, 0) - ez0));
  d[4] = cc * ((a(EZ, 1, 0, 0) - ez0) - (a(EX, 0, 0, 1) - ex0));
  d[5] = cc * ((a(EX, 0, 1, 0) - ex0) - (a(EY, 1, 0, 0) - ey0));
  R cbx = (by0 - a(BY, 0, 0, -1)) - (bz0 - a(BZ, 0, -1, 0));
  R cby = (bz0 - a(BZ, -1, 0, 0)) - (bx0 - a(BX, 0, 0, -1));
  R cbz = (bx0 - a(BX, 0, -1, 0)) - (by0 - a(BY, -1, 0, 0));
  if (B0) {
    cbx = cbx - ((a(B0Y, 0, 0, 0) - a(B0Y, 0, 0, -1)) - (a(B0Z, 0, 0, 0) - a(B0Z, 0, -1, 0)));
    cby = cby - ((a(B0Z, 0, 0, 0) - a(B0Z, -1, 0, 0)) - (a(B0X, 0, 0, 0) - a(B0X, 0, 0, -1)));
    cbz = cbz - ((a(B0X, 0, 0, 0) - a(B0X, 0, -1, 0)) - (a(B0Y, 0, 0, 0) - a(B0Y, -1, 0, 0)));
  }
  // -CC * (X) is -(CC*X); the value equals (-CC)*X exactly.
  d[0] = -(cc * cbx);
  d[1] = -(cc * cby);
  d[2] = -(cc * cbz);

  const R r0 = a.rho(0, 0, 0);
  R intrho, intex, intey, intez, intbx, intby, intbz, bmag, emag;
  // X current (:91-111)
  intrho = R(0.5) * (a.rho(1, 0, 0) + r0);
  intex = ex0;
  intey = R(0.25) * (((ey0 + a(EY, 1, 0, 0)) + a(EY, 0, -1, 0)) + a(EY, 1, -1, 0));
  intez = R(0.25) * (((ez0 + a(EZ, 1, 0, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 1, 0, -1));
  intbx = R(0.125) * (((((((bx0 + a(BX, 0, -1, 0)) + a(BX, 1, -1, 0)) + a(BX, 1, 0, 0)) + a(BX, 0, 0, -1)) +
                        a(BX, 0, -1, -1)) + a(BX, 1, -1, -1)) + a(BX, 1, 0, -1));
  intby = R(0.5) * (by0 + a(BY, 0, 0, -1));
  intbz = R(0.5) * (bz0 + a(BZ, 0, -1, 0));
  bmag = (intbx * intbx + intby * intby) + intbz * intbz;
  emag = (intex * intex + intey * intey) + intez * intez;
  if (emag > bmag) {
    const R corr = sqrt(qdiv<R, FD>(bmag, emag));
    intey = intey * corr;
    intez = intez * corr;
  }
  const R jx = jdiv<R, C, FD>(cc, bmag, intbx, intby, intbz, intrho * (intey * intbz - intby * intez));
  // Y current (:114-134)
  intrho = R(0.5) * (a.rho(0, 1, 0) + r0);
  intex = R(0.25) * (((ex0 + a(EX, -1, 0, 0)) + a(EX, 0, 1, 0)) + a(EX, -1, 1, 0));
  intey = ey0;
  intez = R(0.25) * (((ez0 + a(EZ, 0, 1, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 0, 1, -1));
  intbx = R(0.5) * (bx0 + a(BX, 0, 0, -1));
  intby = R(0.125) * (((((((by0 + a(BY, -1, 0, 0)) + a(BY, -1, 1, 0)) + a(BY, 0, 1, 0)) + a(BY, 0, 0, -1)) +
                        a(BY, -1, 0, -1)) + a(BY, -1, 1, -1)) + a(BY, 0, 1, -1));
  intbz = R(0.5) * (bz0 + a(BZ, -1, 0, 0));
  bmag = (intbx * intbx + intby * intby) + intbz * intbz;
  emag = (intex * intex + intey * intey) + intez * intez;
  if (emag > bmag) {
    const R corr = sqrt(qdiv<R, FD>(bmag, emag));
    intex = intex * corr;
    intez = intez * corr;
  }
  const R jy = jdiv<R, C, FD>(cc, bmag, intbx, intby, intbz, intrho * (intez * intbx - intex * intbz));
  // Z current (:137-157)
  intrho = R(0.5) * (r0 + a.rho(0, 0, 1));
  intex = R(0.25) * (((ex0 + a(EX, -1, 0, 0)) + a(EX, 0, 0, 1)) + a(EX, -1, 0, 1));
  intey = R(0.25) * (((ey0 + a(EY, 0, -1, 0)) + a(EY, 0, 0, 1)) + a(EY, 0, -1, 1));
  intez = ez0;
  intbx = R(0.5) * (bx0 + a(BX, 0, -1, 0));
  intby = R(0.5) * (by0 + a(BY, -1, 0, 0));
  intbz = R(0.125) * (((((((bz0 + a(BZ, -1, 0, 0)) + a(BZ, -1, -1, 0)) + a(BZ, 0, -1, 0)) + a(BZ, 0, 0, 1)) +
                        a(BZ, -1, 0, 1)) + a(BZ, -1, -1, 1)) + a(BZ, 0, -1, 1));
  bmag = (intbx * intbx + intby * intby) + intbz * intbz;
  emag = (intex * intex + intey * intey) + intez * intez;
  if (emag > bmag) {
    const R corr = sqrt(qdiv<R, FD>(bmag, emag));
    intex = intex * corr;
    intey = intey * corr;
  }
  const R jz = jdiv<R, C, FD>(cc, bmag, intbx, intby, intbz, intrho * (intex * intby - intbx * intey));
  d[0] = d[0] - jx;
  d[1] = d[1] - jy;
  d[2] = d[2] - jz;
}

// RK combination (field_solver.F90:187-193): (c1*fn + c2*f) + c3*df, or the
// FP32C increment form fn + (c2*(f - fn) + c3*df), used when c1 + c2 == 1.
template <typename R, int C>
__device__ __forceinline__ R combine(R c1, R c2, R c3, R fn, R f, R df, bool incr) {
  if (C && incr) return fn + (c2 * (f - fn) + c3 * df);
  return (c1 * fn + c2 * f) + c3 * df;
}

// Absorbing shell (field_solver.F90:210-265) applied to the six updated
// components of a cell at global (ig_i, jg_i, kg_i).  Callers pass
// jg_i = i + y0 as the reference does (:211), or j + y0 under
// FFE_FLAG_ABSORB_TRUE_Y (see shell_jg).
// The y coordinate the shell's radius uses for local cell (i, j).
template <typename R>
__device__ __forceinline__ int shell_jg(const Absorb<R>& ab, int i, int j, int y0) { return (ab.true_y ? j : i) + y0; }

template <typename R>
__device__ __forceinline__ void absorb_cell(const Absorb<R>& ab, int ig_i, int jg_i, int kg_i, R v[6]) {
  const R ig = R(ig_i), jg = R(jg_i), kg = R(kg_i);
  R r = sqrt(((ig - ab.xc) * (ig - ab.xc) + (jg - ab.yc) * (jg - ab.yc)) + (kg - ab.zc) * (kg - ab.zc));
  if (!(r > ab.rabsorb - R(1.0))) return;
  const R h = R(0.5);
  const R gx[2] = {ig - ab.xc, (ig + h) - ab.xc};
  const R gy[2] = {jg - ab.yc, (jg + h) - ab.yc};
  const R gz[2] = {kg - ab.zc, (kg + h) - ab.zc};
  // staggering of Ex, Ey, Ez, Bx, By, Bz: (1,0,0) (0,1,0) (0,0,1) (0,1,1) (1,0,1) (1,1,0)
  const int sxo[6] = {1, 0, 0, 0, 1, 1}, syo[6] = {0, 1, 0, 1, 0, 1}, szo[6] = {0, 0, 1, 1, 1, 0};
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const R dx = gx[sxo[c]], dy = gy[syo[c]], dz = gz[szo[c]];
    r = sqrt((dx * dx + dy * dy) + dz * dz);
    R dr = (r - ab.rabsorb) / ab.buff;
    if (ab.clamp && dr > R(1.0)) dr = R(1.0);
    if (dr > R(0.0)) v[c] = (R(1.0) - (dr * dr) * dr) * v[c];
  }
}

// The absorbing shell on the FP32 fast path: the same factors with the
// hardware square-root approximation, depth (r - rabsorb) * (1 / buff), and
// the cell test r > rabsorb - 1 made on r^2 (no root for cells inside).
__device__ __forceinline__ float sqrt_approx(float x);
__device__ __forceinline__ void absorb_cell_fast(const Absorb<float>& ab, int ig_i, int jg_i, int kg_i, float v[6]) {
  const float ig = float(ig_i), jg = float(jg_i), kg = float(kg_i);
  const float x = ig - ab.xc, y = jg - ab.yc, z = kg - ab.zc;
  const float t = ab.rabsorb - 1.f;
  if (t >= 0.f && !((x * x + y * y) + z * z > t * t)) return;
  const float gx[2] = {x, x + 0.5f}, gy[2] = {y, y + 0.5f}, gz[2] = {z, z + 0.5f};
  const int sxo[6] = {1, 0, 0, 0, 1, 1}, syo[6] = {0, 1, 0, 1, 0, 1}, szo[6] = {0, 0, 1, 1, 1, 0};
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const float dx = gx[sxo[c]], dy = gy[syo[c]], dz = gz[szo[c]];
    float dr = (sqrt_approx((dx * dx + dy * dy) + dz * dz) - ab.rabsorb) * ab.inv_buff;
    if (ab.clamp && dr > 1.f) dr = 1.f;
    if (dr > 0.f) v[c] = (1.f - (dr * dr) * dr) * v[c];
  }
}

// cleanEpar (field_solver.F90:288-328): E - (E.B) B / B^2 at the three E points.
template <typename R, int C, bool FD = false>
__device__ __forceinline__ R clean_div(R epar, R bi, R bmag, R bx, R by, R bz, R ct) {
  // ct = 0 (the reference) or TINY (FFE_FLAG_CLEAN_TINY); bmag + 0 == bmag exactly
  if (C == 2) {
    const double bd = ((double)bx * (double)bx + (double)by * (double)by) + (double)bz * (double)bz;
    return (R)((double)(epar * bi) / (bd + (double)ct));
  }
  return qdiv<R, FD>(epar * bi, bmag + ct);
}

template <typename R, int C, class A, bool FD = false>
__device__ __forceinline__ void clean_cell(const A& a, R e[3], R ct = R(0)) {
  const R ex0 = a(EX, 0, 0, 0), ey0 = a(EY, 0, 0, 0), ez0 = a(EZ, 0, 0, 0);
  const R bx0 = a(BX, 0, 0, 0), by0 = a(BY, 0, 0, 0), bz0 = a(BZ, 0, 0, 0);
  R intex, intey, intez, intbx, intby, intbz, bmag, epar;
  intex = ex0;
  intey = R(0.25) * (((ey0 + a(EY, 1, 0, 0)) + a(EY, 0, -1, 0)) + a(EY, 1, -1, 0));
  intez = R(0.25) * (((ez0 + a(EZ, 1, 0, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 1, 0, -1));
  intbx = R(0.125) * (((((((bx0 + a(BX, 0, -1, 0)) + a(BX, 1, -1, 0)) + a(BX, 1, 0, 0)) + a(BX, 0, 0, -1)) +
                        a(BX, 0, -1, -1)) + a(BX, 1, -1, -1)) + a(BX, 1, 0, -1));
  intby = R(0.5) * (by0 + a(BY, 0, 0, -1));
  intbz = R(0.5) * (bz0 + a(BZ, 0, -1, 0));
  bmag = (intbx * intbx + intby * intby) + intbz * intbz;
  epar = (intex * intbx + intey * intby) + intez * intbz;
  e[0] = ex0 - clean_div<R, C, FD>(epar, intbx, bmag, intbx, intby, intbz, ct);

  intex = R(0.25) * (((ex0 + a(EX, -1, 0, 0)) + a(EX, 0, 1, 0)) + a(EX, -1, 1, 0));
  intey = ey0;
  intez = R(0.25) * (((ez0 + a(EZ, 0, 1, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 0, 1, -1));
  intbx = R(0.5) * (bx0 + a(BX, 0, 0, -1));
  intby = R(0.125) * (((((((by0 + a(BY, -1, 0, 0)) + a(BY, -1, 1, 0)) + a(BY, 0, 1, 0)) + a(BY, 0, 0, -1)) +
                        a(BY, -1, 0, -1)) + a(BY, -1, 1, -1)) + a(BY, 0, 1, -1));
  intbz = R(0.5) * (bz0 + a(BZ, -1, 0, 0));
  bmag = (intbx * intbx + intby * intby) + intbz * intbz;
  epar = (intex * intbx + intey * intby) + intez * intbz;
  e[1] = ey0 - clean_div<R, C, FD>(epar, intby, bmag, intbx, intby, intbz, ct);

  intex = R(0.25) * (((ex0 + a(EX, -1, 0, 0)) + a(EX, 0, 0, 1)) + a(EX, -1, 0, 1));
  intey = R(0.25) * (((ey0 + a(EY, 0, -1, 0)) + a(EY, 0, 0, 1)) + a(EY, 0, -1, 1));
  intez = ez0;
  intbx = R(0.5) * (bx0 + a(BX, 0, -1, 0));
  intby = R(0.5) * (by0 + a(BY, -1, 0, 0));
  intbz = R(0.125) * (((((((bz0 + a(BZ, -1, 0, 0)) + a(BZ, -1, -1, 0)) + a(BZ, 0, -1, 0)) + a(BZ, 0, 0, 1)) +
                        a(BZ, -1, 0, 1)) + a(BZ, -1, -1, 1)) + a(BZ, 0, -1, 1));
  bmag = (intbx * intbx + intby * intby) + intbz * intbz;
  epar = (intex * intbx + intey * intby) + intez * intbz;
  e[2] = ez0 - clean_div<R, C, FD>(epar, intbz, bmag, intbx, intby, intbz, ct);
}

// ---------------------------------------------------------------------------
// FP32 fast-path forms of push_cell / clean_cell.  The reference averages are
// sums times 1/2, 1/4 or 1/8; those power-of-two factors are moved out of the
// products and gathered into one constant per quotient, which is exact in
// binary arithmetic (no rounding changes, barring subnormals) and removes
// about a dozen multiplies per cell.  With S the bare sums:
//   64 B^2 = S8^2 + 16 (S2a^2 + S2b^2),   64 E^2 = 64 e0^2 + 4 (S4a^2 + S4b^2),
//   J_i    = 4 CC / (64 B^2 + 64 TINY) * Srho * (cross product of bare sums),
//   clean:   E_i -= (S.B-sums dot) * S8 / (64 B^2 + 64 ct).
// With TREE the four- and eight-term sums are added as balanced trees
// (dependency depth 2 and 3 instead of 3 and 7) grouped by y row: the sub-sum
// of one row is the same expression for the two cells that share the row when
// a thread updates two cells stacked in y, so it is evaluated once.  This
// changes the association of the reference's sums (rounding differences of
// an ulp or so per average).  Without TREE the sums keep the reference's
// left-to-right order (fewer live registers for one cell per thread).
// ---------------------------------------------------------------------------
// The hardware square-root approximation (PTX sqrt.approx.f32; +0 -> +0),
// for the limiter's ratio in the fast path.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Row-grouped partial sums of field c around the cell:
//   xpair(c, dx, dj, dk) = F(0, dj, dk) + F(dx, dj, dk)
//   zpair(c, dj, dz)     = F(0, dj, 0) + F(0, dj, dz)
//   quad(c, dx, dj, dz)  = xpair(c, dx, dj, 0) + xpair(c, dx, dj, dz)
//   oct(c, dx, dy, dz)   = quad(c, dx, 0, dz) + quad(c, dx, dy, dz)
template <class A>
__device__ __forceinline__ float xpair(const A& a, int c, int dx, int dj, int dk) {
  return a(c, 0, dj, dk) + a(c, dx, dj, dk);
}
template <class A>
__device__ __forceinline__ float zpair(const A& a, int c, int dj, int dz) {
  return a(c, 0, dj, 0) + a(c, 0, dj, dz);
}
template <class A>
__device__ __forceinline__ float quad(const A& a, int c, int dx, int dj, int dz) {
  return xpair(a, c, dx, dj, 0) + xpair(a, c, dx, dj, dz);
}
template <class A>
__device__ __forceinline__ float oct(const A& a, int c, int dx, int dy, int dz) {
  return quad(a, c, dx, 0, dz) + quad(a, c, dx, dy, dz);
}

// The bare sums of the averages at the three E points (field_solver.F90
// :93-99, :116-122, :139-145 for the push; :290-295, :304-309, :318-323 for
// the cleaning, which averages the same neighbours): the two 4-point sums of
// the other E components (sa, sb), the 8-point sum of the B component along
// the point (s8) and the 2-point sums of the other two B components (s2a, s2b).
struct PointSums {
  float sa, sb, s8, s2a, s2b;
};
template <bool TREE, class A>
__device__ __forceinline__ PointSums sums_x(const A& a) {  // Ex point: Ey, Ez; Bx; By, Bz
  const float s2a = a(BY, 0, 0, 0) + a(BY, 0, 0, -1), s2b = a(BZ, 0, 0, 0) + a(BZ, 0, -1, 0);
  if constexpr (TREE)
    return {xpair(a, EY, 1, 0, 0) + xpair(a, EY, 1, -1, 0), xpair(a, EZ, 1, 0, 0) + xpair(a, EZ, 1, 0, -1),
            oct(a, BX, 1, -1, -1), s2a, s2b};
  return {((a(EY, 0, 0, 0) + a(EY, 1, 0, 0)) + a(EY, 0, -1, 0)) + a(EY, 1, -1, 0),
          ((a(EZ, 0, 0, 0) + a(EZ, 1, 0, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 1, 0, -1),
          ((((((a(BX, 0, 0, 0) + a(BX, 0, -1, 0)) + a(BX, 1, -1, 0)) + a(BX, 1, 0, 0)) + a(BX, 0, 0, -1)) +
            a(BX, 0, -1, -1)) + a(BX, 1, -1, -1)) + a(BX, 1, 0, -1),
          s2a, s2b};
}
template <bool TREE, class A>
__device__ __forceinline__ PointSums sums_y(const A& a) {  // Ey point: Ex, Ez; By; Bx, Bz
  const float s2a = a(BX, 0, 0, 0) + a(BX, 0, 0, -1), s2b = a(BZ, 0, 0, 0) + a(BZ, -1, 0, 0);
  if constexpr (TREE)
    return {xpair(a, EX, -1, 0, 0) + xpair(a, EX, -1, 1, 0), zpair(a, EZ, 0, -1) + zpair(a, EZ, 1, -1),
            oct(a, BY, -1, 1, -1), s2a, s2b};
  return {((a(EX, 0, 0, 0) + a(EX, -1, 0, 0)) + a(EX, 0, 1, 0)) + a(EX, -1, 1, 0),
          ((a(EZ, 0, 0, 0) + a(EZ, 0, 1, 0)) + a(EZ, 0, 0, -1)) + a(EZ, 0, 1, -1),
          ((((((a(BY, 0, 0, 0) + a(BY, -1, 0, 0)) + a(BY, -1, 1, 0)) + a(BY, 0, 1, 0)) + a(BY, 0, 0, -1)) +
            a(BY, -1, 0, -1)) + a(BY, -1, 1, -1)) + a(BY, 0, 1, -1),
          s2a, s2b};
}
template <bool TREE, class A>
__device__ __forceinline__ PointSums sums_z(const A& a) {  // Ez point: Ex, Ey; Bz; Bx, By
  const float s2a = a(BX, 0, 0, 0) + a(BX, 0, -1, 0), s2b = a(BY, 0, 0, 0) + a(BY, -1, 0, 0);
  if constexpr (TREE)
    return {xpair(a, EX, -1, 0, 0) + xpair(a, EX, -1, 0, 1), zpair(a, EY, 0, 1) + zpair(a, EY, -1, 1),
            oct(a, BZ, -1, -1, 1), s2a, s2b};
  return {((a(EX, 0, 0, 0) + a(EX, -1, 0, 0)) + a(EX, 0, 0, 1)) + a(EX, -1, 0, 1),
          ((a(EY, 0, 0, 0) + a(EY, 0, -1, 0)) + a(EY, 0, 0, 1)) + a(EY, 0, -1, 1),
          ((((((a(BZ, 0, 0, 0) + a(BZ, -1, 0, 0)) + a(BZ, -1, -1, 0)) + a(BZ, 0, -1, 0)) + a(BZ, 0, 0, 1)) +
            a(BZ, -1, 0, 1)) + a(BZ, -1, -1, 1)) + a(BZ, 0, -1, 1),
          s2a, s2b};
}

// FP32CD on the fast path, one cell: the B^2 denominators as double-float
// values (hi + lo, 48 significant bits; Dekker 1971): exact products by the
// FMA, Knuth's TwoSum, one Newton step on the quotient.  Written with the
// round-to-nearest intrinsics so that no add or multiply is contracted into
// an FMA, which would break the error terms.
struct DF1 {
  float hi, lo;
};
__device__ __forceinline__ void two_sum1(float a, float b, float& s, float& t) {  // s + t == a + b
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// 64 B^2 + t from the bare sums (every term >= 0); `bm` receives 64 B^2 as a float
__device__ __forceinline__ DF1 bmag64_df1(const PointSums& s, float t, float& bm) {
  const float u = __fmul_rn(4.f, s.s2a), w = __fmul_rn(4.f, s.s2b);  // 16 s^2 == (4 s)^2 exactly
  const float p1 = __fmul_rn(s.s8, s.s8), p2 = __fmul_rn(u, u), p3 = __fmul_rn(w, w);
  const float e1 = __fmaf_rn(s.s8, s.s8, -p1), e2 = __fmaf_rn(u, u, -p2), e3 = __fmaf_rn(w, w, -p3);
  float a, ta, tb, c, tc;
  two_sum1(p1, p2, a, ta);
  two_sum1(a, p3, bm, tb);
  two_sum1(bm, t, c, tc);
  const float lo = __fadd_rn(__fadd_rn(__fadd_rn(ta, tb), tc), __fadd_rn(__fadd_rn(e1, e2), e3));
  DF1 r;
  r.hi = __fadd_rn(c, lo);
  r.lo = __fsub_rn(lo, __fsub_rn(r.hi, c));
  return r;
}
// n / (d.hi + d.lo)
__device__ __forceinline__ float df_div1(float n, const DF1& d) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d.hi));
  const float q = __fmul_rn(n, r);
  const float res = __fmaf_rn(-q, d.lo, __fmaf_rn(-q, d.hi, n));
  return __fmaf_rn(res, r, q);
}

template <bool DF = false>
__device__ __forceinline__ float fast_current(float cc4, float t64, float sr, float e0, const PointSums& s,
                                              float& ea, float& eb) {
  float bm;
  DF1 den;
  if constexpr (DF) den = bmag64_df1(s, t64, bm);
  else bm = s.s8 * s.s8 + 16.f * (s.s2a * s.s2a + s.s2b * s.s2b);
  const float em = 64.f * (e0 * e0) + 4.f * (s.sa * s.sa + s.sb * s.sb);
  // limiter as a select: corr = 1 leaves the values unchanged exactly
  const float corr = em > bm ? sqrt_approx(__fdividef(bm, em)) : 1.f;
  ea = s.sa * corr;
  eb = s.sb * corr;
  if constexpr (DF) return df_div1(cc4, den) * sr;
  return __fdividef(cc4, bm + t64) * sr;
}

// DF: the denominators of FP32CD
template <bool B0, bool TREE, class A, bool DF = false>
__device__ __forceinline__ void push_cell_fast(const A& a, float cc, float d[6]) {
  const float ey0 = a(EY, 0, 0, 0), ez0 = a(EZ, 0, 0, 0), ex0 = a(EX, 0, 0, 0);
  const float bx0 = a(BX, 0, 0, 0), by0 = a(BY, 0, 0, 0), bz0 = a(BZ, 0, 0, 0);
  d[3] = cc * ((a(EY, 0, 0, 1) - ey0) - (a(EZ, 0, 1, 0) - ez0));
  d[4] = cc * ((a(EZ, 1, 0, 0) - ez0) - (a(EX, 0, 0, 1) - ex0));
  d[5] = cc * ((a(EX, 0, 1, 0) - ex0) - (a(EY, 1, 0, 0) - ey0));
  float cbx = (by0 - a(BY, 0, 0, -1)) - (bz0 - a(BZ, 0, -1, 0));
  float cby = (bz0 - a(BZ, -1, 0, 0)) - (bx0 - a(BX, 0, 0, -1));
  float cbz = (bx0 - a(BX, 0, -1, 0)) - (by0 - a(BY, -1, 0, 0));
  if (B0) {
    cbx = cbx - ((a(B0Y, 0, 0, 0) - a(B0Y, 0, 0, -1)) - (a(B0Z, 0, 0, 0) - a(B0Z, 0, -1, 0)));
    cby = cby - ((a(B0Z, 0, 0, 0) - a(B0Z, -1, 0, 0)) - (a(B0X, 0, 0, 0) - a(B0X, 0, 0, -1)));
    cbz = cbz - ((a(B0X, 0, 0, 0) - a(B0X, 0, -1, 0)) - (a(B0Y, 0, 0, 0) - a(B0Y, -1, 0, 0)));
  }
  const float r0 = a.rho(0, 0, 0);
  const float cc4 = 4.f * cc, t64 = 64.f * tiny<float>();
  float ea, eb, k;
  {  // X current at the Ex point (field_solver.F90:91-111)
    const PointSums s = sums_x<TREE>(a);
    k = fast_current<DF>(cc4, t64, a.rho(1, 0, 0) + r0, ex0, s, ea, eb);
    d[0] = -(cc * cbx) - k * (ea * s.s2b - s.s2a * eb);
  }
  {  // Y current at the Ey point (:114-134)
    const PointSums s = sums_y<TREE>(a);
    k = fast_current<DF>(cc4, t64, a.rho(0, 1, 0) + r0, ey0, s, ea, eb);
    d[1] = -(cc * cby) - k * (eb * s.s2a - ea * s.s2b);
  }
  {  // Z current at the Ez point (:137-157)
    const PointSums s = sums_z<TREE>(a);
    k = fast_current<DF>(cc4, t64, r0 + a.rho(0, 0, 1), ez0, s, ea, eb);
    d[2] = -(cc * cbz) - k * (ea * s.s2b - s.s2a * eb);
  }
}

// E_i - ep S8 / (64 B^2 + c64) at one E point of one cell
template <bool DF>
__device__ __forceinline__ float clean_quot1(float ep, const PointSums& s, float c64, float e0) {
  if constexpr (DF) {
    float bm;
    return e0 - df_div1(ep * s.s8, bmag64_df1(s, c64, bm));
  }
  const float bm = s.s8 * s.s8 + 16.f * (s.s2a * s.s2a + s.s2b * s.s2b);
  return e0 - __fdividef(ep * s.s8, bm + c64);
}

template <bool TREE, class A, bool DF = false>
__device__ __forceinline__ void clean_cell_fast(const A& a, float e[3], float ct) {
  const float ex0 = a(EX, 0, 0, 0), ey0 = a(EY, 0, 0, 0), ez0 = a(EZ, 0, 0, 0);
  const float c64 = 64.f * ct;
  {  // Ex point (:289-300)
    const PointSums s = sums_x<TREE>(a);
    const float ep = ex0 * s.s8 + s.sa * s.s2a + s.sb * s.s2b;
    e[0] = clean_quot1<DF>(ep, s, c64, ex0);
  }
  {  // Ey point (:303-314)
    const PointSums s = sums_y<TREE>(a);
    const float ep = s.sa * s.s2a + ey0 * s.s8 + s.sb * s.s2b;
    e[1] = clean_quot1<DF>(ep, s, c64, ey0);
  }
  {  // Ez point (:317-328)
    const PointSums s = sums_z<TREE>(a);
    const float ep = s.sa * s.s2a + s.sb * s.s2b + ez0 * s.s8;
    e[2] = clean_quot1<DF>(ep, s, c64, ez0);
  }
}

// ---------------------------------------------------------------------------
// Packed forms for two cells at once (FP32 fast path of the plain variant).
// A thread that updates and cleans two cells stacked in y keeps each quantity
// of both cells in one float2 (x: the lower cell, y: the upper) and evaluates
// the same expressions with the paired FP32 instructions of sm_100+
// (add/mul/fma.f32x2: one issue slot for two lanes' worth of work, each half
// rounded exactly as its scalar instruction).  The accessor returns
// float2 {value at the lower cell, value at the upper cell}.  Quotients and
// square roots have no paired form and run per half.  The four- and
// eight-term sums are added as balanced trees grouped by z plane.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b as fma(b, -1, a): the product is exact, so it rounds as a - b does
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2s(float s) { return make_float2(s, s); }
// hardware reciprocal approximation (PTX rcp.approx.ftz.f32), per half
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float2 f2rcp(float2 a) { return make_float2(rcp_approx(a.x), rcp_approx(a.y)); }
// -1 / x per half
__device__ __forceinline__ float2 f2nrcp(float2 a) { return make_float2(rcp_approx(-a.x), rcp_approx(-a.y)); }

template <class A>
__device__ __forceinline__ float2 rho2(const A& a, int di, int dj, int dk) {
  return f2add(f2add(f2sub(a(EX, di, dj, dk), a(EX, di - 1, dj, dk)), f2sub(a(EY, di, dj, dk), a(EY, di, dj - 1, dk))),
               f2sub(a(EZ, di, dj, dk), a(EZ, di, dj, dk - 1)));
}
// F(0,dj,dk) + F(dx,dj,dk)
template <class A>
__device__ __forceinline__ float2 xpair2(const A& a, int c, int dx, int dj, int dk) {
  return f2add(a(c, 0, dj, dk), a(c, dx, dj, dk));
}

struct PointSums2 {
  float2 sa, sb, s8, s2a, s2b;
};
// 64 B^2 of a point from its bare sums
__device__ __forceinline__ float2 bmag64_2(const PointSums2& s) {
  return f2fma(s.s8, s.s8, f2mul(f2s(16.f), f2fma(s.s2a, s.s2a, f2mul(s.s2b, s.s2b))));
}

// FP32CD on the fast path: the B^2 denominators as double-float values, the
// unevaluated sum hi + lo of two floats (48 significant bits; Dekker 1971):
// exact products by the FMA (p = a b, e = fma(a, b, -p)), sums by Knuth's
// TwoSum, and the quotient by one Newton step on the reciprocal estimate of
// hi.  All of it is FP32 arithmetic in the paired instructions, where FP64
// arithmetic runs at a small fraction of the FP32 rate.
struct DF2 {
  float2 hi, lo;
};
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
// s + t == a + b exactly (TwoSum)
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& t) {
  s = f2add(a, b);
  const float2 bb = f2sub(s, a);
  t = f2add(f2sub(a, f2sub(s, bb)), f2sub(b, bb));
}
// 64 B^2 + t of a point from its bare sums as a double-float (every term is
// >= 0); `bm` receives 64 B^2 as a float (for the limiter)
__device__ __forceinline__ DF2 bmag64_df(const PointSums2& s, float2 t, float2& bm) {
  const float2 u = f2mul(f2s(4.f), s.s2a), w = f2mul(f2s(4.f), s.s2b);  // 16 s^2 == (4 s)^2 exactly
  const float2 p1 = f2mul(s.s8, s.s8), p2 = f2mul(u, u), p3 = f2mul(w, w);
  const float2 e1 = f2fma(s.s8, s.s8, f2neg(p1)), e2 = f2fma(u, u, f2neg(p2)), e3 = f2fma(w, w, f2neg(p3));
  float2 a, ta, tb, c, tc;
  two_sum2(p1, p2, a, ta);
  two_sum2(a, p3, bm, tb);
  two_sum2(bm, t, c, tc);
  const float2 lo = f2add(f2add(f2add(ta, tb), tc), f2add(f2add(e1, e2), e3));
  DF2 r;
  r.hi = f2add(c, lo);
  r.lo = f2sub(lo, f2sub(r.hi, c));
  return r;
}
// n / (d.hi + d.lo)
__device__ __forceinline__ float2 df_div(float2 n, const DF2& d) {
  const float2 r = f2rcp(d.hi);
  const float2 q = f2mul(n, r);
  const float2 res = f2fma(f2neg(q), d.lo, f2fma(f2neg(q), d.hi, n));
  return f2fma(res, r, q);
}

// The current factor k = 4 CC Srho / (64 B^2 + 64 TINY) of a point and its
// limited transverse E sums (ea, eb).  The limiter factor is min(1,
// sqrt(B^2 / E^2)): 1 where E^2 <= B^2 (and where E = 0), the reference's
// sqrt(B^2/E^2) where E^2 > B^2.
template <bool DF>
__device__ __forceinline__ float2 fast_current2(float cc4, float t64, float2 sr, float2 e0, const PointSums2& s,
                                                float2& ea, float2& eb) {
  float2 bm;
  DF2 den;
  if constexpr (DF) den = bmag64_df(s, f2s(t64), bm);
  else bm = bmag64_2(s);
  const float2 em = f2fma(f2mul(f2s(64.f), e0), e0, f2mul(f2s(4.f), f2fma(s.sa, s.sa, f2mul(s.sb, s.sb))));
  const float2 q = f2mul(bm, f2rcp(em));
  const float2 corr = make_float2(fminf(1.f, sqrt_approx(q.x)), fminf(1.f, sqrt_approx(q.y)));
  ea = f2mul(s.sa, corr);
  eb = f2mul(s.sb, corr);
  if constexpr (DF) return df_div(f2mul(f2s(cc4), sr), den);
  return f2mul(f2mul(f2s(cc4), sr), f2rcp(f2add(bm, f2s(t64))));
}

// Sums carried from plane to plane along the z march.  The eight-point B sum
// at a point is the sum of two four-point quads in neighbouring z planes, and
// rho at (0,0,1) is next plane's rho at (0,0,0): each is computed once, with
// the same expression, and reused by the next plane (bit for bit the value a
// recomputation would give).  The quads are those of Bx at the Ex point
// (planes p, p-1), By at the Ey point (p, p-1) and Bz at the Ez point
// (p, p+1).
struct PushCarry {
  float2 r0;          // rho at this plane
  float2 qx, qy, qz;  // Bx, By quads of plane p-1; Bz quad of plane p
};
struct CleanCarry {
  float2 qx, qy, qz;
};
template <class A>
__device__ __forceinline__ float2 quad_x(const A& a, int dz) {  // Bx over x 0..1, y -1..0 at plane dz
  return f2add(xpair2(a, BX, 1, 0, dz), xpair2(a, BX, 1, -1, dz));
}
template <class A>
__device__ __forceinline__ float2 quad_y(const A& a, int dz) {  // By over x -1..0, y 0..1
  return f2add(xpair2(a, BY, -1, 0, dz), xpair2(a, BY, -1, 1, dz));
}
template <class A>
__device__ __forceinline__ float2 quad_z(const A& a, int dz) {  // Bz over x -1..0, y -1..0
  return f2add(xpair2(a, BZ, -1, 0, dz), xpair2(a, BZ, -1, -1, dz));
}
// the carried values of a plane from its own neighbourhood (first plane of a run)
template <class A>
__device__ __forceinline__ void push_carry_prime(const A& a, PushCarry& c) {
  c.r0 = rho2(a, 0, 0, 0);
  c.qx = quad_x(a, -1);
  c.qy = quad_y(a, -1);
  c.qz = quad_z(a, 0);
}
template <class A>
__device__ __forceinline__ void clean_carry_prime(const A& a, CleanCarry& c) {
  c.qx = quad_x(a, -1);
  c.qy = quad_y(a, -1);
  c.qz = quad_z(a, 0);
}

// push_cell_fast (no B0) for two cells; `cy` holds this plane's carried values
// on entry and the next plane's on return; DF: the denominators of FP32CD
template <bool DF, class A>
__device__ __forceinline__ void push_pair_fast(const A& a, float cc, float2 d[6], PushCarry& cy) {
  const float2 ey0 = a(EY, 0, 0, 0), ez0 = a(EZ, 0, 0, 0), ex0 = a(EX, 0, 0, 0);
  const float2 bx0 = a(BX, 0, 0, 0), by0 = a(BY, 0, 0, 0), bz0 = a(BZ, 0, 0, 0);
  const float2 c2 = f2s(cc);
  d[3] = f2mul(c2, f2sub(f2sub(a(EY, 0, 0, 1), ey0), f2sub(a(EZ, 0, 1, 0), ez0)));
  d[4] = f2mul(c2, f2sub(f2sub(a(EZ, 1, 0, 0), ez0), f2sub(a(EX, 0, 0, 1), ex0)));
  d[5] = f2mul(c2, f2sub(f2sub(a(EX, 0, 1, 0), ex0), f2sub(a(EY, 1, 0, 0), ey0)));
  const float2 mcc = f2s(-cc);  // -(CC*X) == (-CC)*X exactly
  const float2 cbx = f2mul(mcc, f2sub(f2sub(by0, a(BY, 0, 0, -1)), f2sub(bz0, a(BZ, 0, -1, 0))));
  const float2 cby = f2mul(mcc, f2sub(f2sub(bz0, a(BZ, -1, 0, 0)), f2sub(bx0, a(BX, 0, 0, -1))));
  const float2 cbz = f2mul(mcc, f2sub(f2sub(bx0, a(BX, 0, -1, 0)), f2sub(by0, a(BY, -1, 0, 0))));
  const float2 r0 = cy.r0;
  const float cc4 = 4.f * cc, t64 = 64.f * tiny<float>();
  float2 ea, eb, k;
  {  // X current at the Ex point (field_solver.F90:91-111): dE_x = -CC curl - k (ea s2b - s2a eb)
    PointSums2 s;
    s.s2a = f2add(a(BY, 0, 0, 0), a(BY, 0, 0, -1));
    s.s2b = f2add(a(BZ, 0, 0, 0), a(BZ, 0, -1, 0));
    s.sa = f2add(xpair2(a, EY, 1, 0, 0), xpair2(a, EY, 1, -1, 0));
    s.sb = f2add(xpair2(a, EZ, 1, 0, 0), xpair2(a, EZ, 1, 0, -1));
    const float2 q0 = quad_x(a, 0);
    s.s8 = f2add(q0, cy.qx);
    cy.qx = q0;
    k = fast_current2<DF>(cc4, t64, f2add(rho2(a, 1, 0, 0), r0), ex0, s, ea, eb);
    d[0] = f2fma(k, f2sub(f2mul(s.s2a, eb), f2mul(ea, s.s2b)), cbx);
  }
  {  // Y current at the Ey point (:114-134): - k (eb s2a - ea s2b)
    PointSums2 s;
    s.s2a = f2add(a(BX, 0, 0, 0), a(BX, 0, 0, -1));
    s.s2b = f2add(a(BZ, 0, 0, 0), a(BZ, -1, 0, 0));
    s.sa = f2add(xpair2(a, EX, -1, 0, 0), xpair2(a, EX, -1, 1, 0));
    s.sb = f2add(f2add(a(EZ, 0, 0, 0), a(EZ, 0, 1, 0)), f2add(a(EZ, 0, 0, -1), a(EZ, 0, 1, -1)));
    const float2 q0 = quad_y(a, 0);
    s.s8 = f2add(q0, cy.qy);
    cy.qy = q0;
    k = fast_current2<DF>(cc4, t64, f2add(rho2(a, 0, 1, 0), r0), ey0, s, ea, eb);
    d[1] = f2fma(k, f2sub(f2mul(ea, s.s2b), f2mul(eb, s.s2a)), cby);
  }
  {  // Z current at the Ez point (:137-157): - k (ea s2b - s2a eb)
    PointSums2 s;
    s.s2a = f2add(a(BX, 0, 0, 0), a(BX, 0, -1, 0));
    s.s2b = f2add(a(BY, 0, 0, 0), a(BY, -1, 0, 0));
    s.sa = f2add(xpair2(a, EX, -1, 0, 0), xpair2(a, EX, -1, 0, 1));
    s.sb = f2add(f2add(a(EY, 0, 0, 0), a(EY, 0, -1, 0)), f2add(a(EY, 0, 0, 1), a(EY, 0, -1, 1)));
    const float2 q1 = quad_z(a, 1);
    s.s8 = f2add(cy.qz, q1);
    cy.qz = q1;
    const float2 r1 = rho2(a, 0, 0, 1);
    cy.r0 = r1;
    k = fast_current2<DF>(cc4, t64, f2add(r0, r1), ez0, s, ea, eb);
    d[2] = f2fma(k, f2sub(f2mul(s.s2a, eb), f2mul(ea, s.s2b)), cbz);
  }
}

// E_i - ep S8 / (64 B^2 + c64) at one E point of two cells
template <bool DF>
__device__ __forceinline__ float2 clean_quot(float2 ep, const PointSums2& s, float2 c64, float2 e0) {
  if constexpr (DF) {
    float2 bm;
    return f2sub(e0, df_div(f2mul(ep, s.s8), bmag64_df(s, c64, bm)));
  }
  return f2fma(f2mul(ep, s.s8), f2nrcp(f2add(bmag64_2(s), c64)), e0);
}

// clean_cell_fast for two cells (ct64 = 64 x the cleaning's TINY, 0 by default):
// E_i - (E.B-sums) S8 / (64 B^2 + ct64); `cy` and DF as in push_pair_fast
template <bool DF, class A>
__device__ __forceinline__ void clean_pair_fast(const A& a, float2 e[3], float ct64, CleanCarry& cy) {
  const float2 ex0 = a(EX, 0, 0, 0), ey0 = a(EY, 0, 0, 0), ez0 = a(EZ, 0, 0, 0);
  const float2 c64 = f2s(ct64);
  {  // Ex point (:289-300)
    PointSums2 s;
    s.s2a = f2add(a(BY, 0, 0, 0), a(BY, 0, 0, -1));
    s.s2b = f2add(a(BZ, 0, 0, 0), a(BZ, 0, -1, 0));
    s.sa = f2add(xpair2(a, EY, 1, 0, 0), xpair2(a, EY, 1, -1, 0));
    s.sb = f2add(xpair2(a, EZ, 1, 0, 0), xpair2(a, EZ, 1, 0, -1));
    const float2 q0 = quad_x(a, 0);
    s.s8 = f2add(q0, cy.qx);
    cy.qx = q0;
    const float2 ep = f2fma(ex0, s.s8, f2fma(s.sa, s.s2a, f2mul(s.sb, s.s2b)));
    e[0] = clean_quot<DF>(ep, s, c64, ex0);
  }
  {  // Ey point (:303-314)
    PointSums2 s;
    s.s2a = f2add(a(BX, 0, 0, 0), a(BX, 0, 0, -1));
    s.s2b = f2add(a(BZ, 0, 0, 0), a(BZ, -1, 0, 0));
    s.sa = f2add(xpair2(a, EX, -1, 0, 0), xpair2(a, EX, -1, 1, 0));
    s.sb = f2add(f2add(a(EZ, 0, 0, 0), a(EZ, 0, 1, 0)), f2add(a(EZ, 0, 0, -1), a(EZ, 0, 1, -1)));
    const float2 q0 = quad_y(a, 0);
    s.s8 = f2add(q0, cy.qy);
    cy.qy = q0;
    const float2 ep = f2fma(ey0, s.s8, f2fma(s.sa, s.s2a, f2mul(s.sb, s.s2b)));
    e[1] = clean_quot<DF>(ep, s, c64, ey0);
  }
  {  // Ez point (:317-328)
    PointSums2 s;
    s.s2a = f2add(a(BX, 0, 0, 0), a(BX, 0, -1, 0));
    s.s2b = f2add(a(BY, 0, 0, 0), a(BY, -1, 0, 0));
    s.sa = f2add(xpair2(a, EX, -1, 0, 0), xpair2(a, EX, -1, 0, 1));
    s.sb = f2add(f2add(a(EY, 0, 0, 0), a(EY, 0, -1, 0)), f2add(a(EY, 0, 0, 1), a(EY, 0, -1, 1)));
    const float2 q1 = quad_z(a, 1);
    s.s8 = f2add(cy.qz, q1);
    cy.qz = q1;
    const float2 ep = f2fma(ez0, s.s8, f2fma(s.sa, s.s2a, f2mul(s.sb, s.s2b)));
    e[2] = clean_quot<DF>(ep, s, c64, ez0);
  }
}

// RK combination for two cells (see combine)
template <int C>
__device__ __forceinline__ float2 combine2(float c1, float c2, float c3, float2 fn, float2 f, float2 df, bool incr) {
  if (C && incr) return f2add(fn, f2fma(f2s(c2), f2sub(f, fn), f2mul(f2s(c3), df)));
  return f2fma(f2s(c3), df, f2fma(f2s(c1), fn, f2mul(f2s(c2), f)));
}

}  // namespace ffe
