// ffe_fused_types.cuh — parameter blocks of the fused stage kernels, shared by
// the kernels (ffe_fused.cu) and the host drivers that fill them (ffe_api.cu).
#pragma once
#include <cuda.h>
#include "ffe_common.cuh"

namespace ffe {

// Tile of the fused stage kernel: TX x TY cells per block, TX fixed at one warp
// width.  The tile height TY is a template parameter (8 or 16).
constexpr int FUSED_TX = 32;
constexpr int FUSED_TY = 8;  // tile height of the single-grid stage kernel
// tile height of the single-grid stage kernel's plain FP32 variant (no B0, no
// absorbing layer): its lean rings at this height still fit two blocks per SM
// and the halo recompute falls from 1.33x (32 x 8 tile) to 1.24x (32 x 12)
constexpr int PLAIN_TY = 12;

struct Maps {  // one 3-D tensor map per component: stage input (OLD) and step start (EN)
  CUtensorMap in[6];
  CUtensorMap en[6];
};

template <typename R>
struct Params {
  Geom g;
  Phys p;
  Absorb<R> ab;
  R cc, c1, c2, c3;
  R ct;  // TINY in the cleaning denominator (opt-in), else 0
  int incr;
  int kz;  // planes per block
  const R* b0[3];
  // The six arrays of a set lie at a fixed stride: component c of the stage
  // input, step-start and output sets starts at in0, en0, out0 + c * fs.
  const R* in0;
  const R* en0;
  R* out0;
  long long fs;
  int* err;
  int ubc;  // apply the user_uniform BC inline (this step's constants in ub)
  UniformBC<R> ub;
};

// One grid of a batched stage launch: its parameters, the tensor maps of its
// stage-input and step-start sets (in global memory, 64-byte aligned), and
// the two block-uniform switches of the kernel body.
template <typename R>
struct alignas(16) BatchBox {
  Params<R> P;
  const CUtensorMap* mi;
  const CUtensorMap* me;
  int has_b0, absorb;
};

// The entries of one batched stage launch, passed by value as the kernel's
// parameter (at most 32 KB: 64 entries of 384 bytes in FP32, 448 in FP64).
constexpr int BATCH_MAX = 64;
template <typename R>
struct BoxTable {
  BatchBox<R> b[BATCH_MAX];
};

// A block's work in a batched launch: tile (tx, ty), z-chunk tz of grid `box`
// (an index into the launch's BoxTable).
struct BatchItem {
  int box, tx, ty, tz;
};

// Pulsar-BC fix-up of one grid (see ffe_fused.cu): U = the BC's box dilated by
// two cells, S1/S2 compact 6-component work arrays over U.
template <typename R>
struct FixParams {
  Geom g;
  Phys p;
  Absorb<R> ab;
  PsrBC<R> q;
  R cc, c1, c2, c3, ct;
  int incr;
  int ui, uj, uk, ux, uy, uz;  // U: first cell and extents
  const R* in[6];
  const R* en[6];
  const R* b0[3];
  R* out[6];
  R* s1;
  R* s2;
  int has_b0, absorb;
};

// A block's work in a batched fix-up or ghost-plane launch: grid `box`,
// block (bx, by) of a plane, plane index bz.
struct FixItem {
  int box, bx, by, bz;
};

// U = the pulsar BC's bounding box dilated by two cells, clipped to the array:
// u = {first i, first j, first k, extent x, extent y, extent z}.
inline void psr_fix_box(const Geom& g, int i_lo, int i_hi, int j_lo, int j_hi, int k_lo, int k_hi, int u[6]) {
  u[0] = i_lo - 2 > -NG ? i_lo - 2 : -NG;
  u[1] = j_lo - 2 > -NG ? j_lo - 2 : -NG;
  u[2] = k_lo - 2 > -NG ? k_lo - 2 : -NG;
  u[3] = (i_hi + 2 < g.sx + NG - 1 ? i_hi + 2 : g.sx + NG - 1) - u[0] + 1;
  u[4] = (j_hi + 2 < g.sy + NG - 1 ? j_hi + 2 : g.sy + NG - 1) - u[1] + 1;
  u[5] = (k_hi + 2 < g.sz + NG - 1 ? k_hi + 2 : g.sz + NG - 1) - u[2] + 1;
}

}  // namespace ffe
