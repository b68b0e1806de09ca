// ffe_common.cuh — device layout and parameter blocks shared by the kernels.
//
// Device layout of one field array (one allocation per array inside one arena):
//   * index (i, j, k) with i, j, k in [-2, s+1] (NGHOST = 2, as the reference's
//     allocation, src/logistics/initialize.F90:192-199), x fastest;
//   * each x-row is padded to a pitch of px elements (a multiple of 128 bytes)
//     and cell i = 0 sits at element OX = 2 of its row, so that ghost cell
//     i = -2 starts the row: a tile whose first cell is x0 - 2 (x0 a multiple
//     of 32) then starts on a 128-byte boundary, as TMA boxes must;
//   * rows per plane py = sy + 4, planes sz + 4.
// A reference-layout host array (sx+4 contiguous values per row) maps onto this
// with one pitched 2-D copy (ffe_api.cu).
//
// Since a row holds cells -2 .. s+1 from element 0, the TMA tensor coordinate of
// cell (i, j, k) is (i + 2, j + 2, k + 2).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ffe {

constexpr int NG = 2;

template <typename R> struct Layout;
template <> struct Layout<float> { static constexpr int OX = 2; static constexpr int PXA = 32; };
template <> struct Layout<double> { static constexpr int OX = 2; static constexpr int PXA = 16; };

struct Geom {
  int sx, sy, sz;     // interior cells
  int px;             // row pitch (elements)
  int py;             // rows per plane (sy + 4)
  int ox;             // element offset of cell i = 0 in its row
  long long plane;    // px * py
  long long nelem;    // px * py * (sz + 4)
  __host__ __device__ __forceinline__ long long idx(int i, int j, int k) const {
    return (long long)(k + NG) * plane + (long long)(j + NG) * px + (i + ox);
  }
};

// Global placement and physics constants of one meshblock.
struct Phys {
  int x0, y0, z0;      // meshblock corner in the global mesh
  int gsx, gsy, gsz;   // global mesh
  int bnd[3];          // 0 open, 1 periodic, 2 absorbing
  int absorb_buff;
  int withhold_copy;   // FFE_FLAG_TEST_WITHHOLD_COPY (failure-detection tests only)
  double cc;
};

// Field pointer bundles.
template <typename R> struct EB { R* c[6]; };           // ex ey ez bx by bz
template <typename R> struct CEB { const R* c[6]; };

// Absorbing-layer constants (field_solver.F90:200-204), in precision R.
template <typename R> struct Absorb {
  R xc, yc, zc, rabsorb, buff;
  R inv_buff;  // 1 / buff (the fast path's quotient)
  int clamp;   // FFE_FLAG_ABSORB_CLAMP: delta_r <- min(delta_r, 1)
  int true_y;  // FFE_FLAG_ABSORB_TRUE_Y: jg = j + y0 instead of the reference's i + y0
};

// psr boundary-condition constants (user/user_psr.F90:26-37,345-374) in R.
template <typename R> struct PsrBC {
  R radius, omega, ccinv, xc, yc, zc, sr2;  // sr2 = (2 R)^2
  R mu[3];                                   // dipole moment at this step
  int i_lo, i_hi, j_lo, j_hi, k_lo, k_hi;    // bounding box (local, interior)
  int bx, by, bz;                            // box extents
};

// user_uniform constants (user/user_uniform.F90:27-41) in R.
template <typename R> struct UniformBC {
  R xc, yc, r0, beta, bnorm, cc, tanh_t;  // tanh(time / t0) for this step
};

}  // namespace ffe
