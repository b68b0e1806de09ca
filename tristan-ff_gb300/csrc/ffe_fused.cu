// ffe_fused.cu — one launch per SSP-RK3 stage: computeRho + rk3Push +
// rk3Update (+ absorbing shell) + ghost fill + cleanEpar + ghost fill.
//
// Data flow of one launch (block = TX x TY column of cells, marching in z
// through a chunk of planes):
//   OLD ring   : stage-input E,B on 3 planes over the tile + 2 halo cells
//   NEW ring   : updated (not yet cleaned) E,B on 3 planes over tile + 1 halo
//   per plane k: load OLD(k+2); compute NEW(k+1) on tile+1 (push + update);
//                clean plane k on the tile from NEW(k-1..k+1); store.
// The halo-1 ring of NEW is recomputed by neighbouring blocks (1.33x push
// work for a 32x8 tile) instead of a second pass over memory, so a stage
// reads E,B (+ step-start E,B for stages 2-3) once and writes E,B once.
//
// Ghosts.  The reference refreshes ghosts by exchangeFields after the update
// and after the cleaning (src/tristanmainloop.F90:59-61).  Here a cell lying
// within 2 cells of a periodic face is also stored at its periodic image in
// the ghost shell, so the output arrays leave the kernel with valid ghosts
// and the next stage reads plain indices.  On open / absorbing axes ghosts
// keep the values they were given at set-up (no neighbour sends them,
// src/tools/helpers.F90:27-45), and the halo cells of NEW that lie there take
// those frozen values.
//
// Compiled twice: normally (multiply-add contraction on; the fast path) and
// with -fmad=false under FFE_FUSED_EXACT (bit-comparable with the oracle).
#include "ffe_kernels.h"
#include "ffe_physics.cuh"

#ifdef FFE_FUSED_EXACT
#define FFE_FUSED_NS fused_exact
#else
#define FFE_FUSED_NS fused_fast
#endif

namespace ffe {
namespace FFE_FUSED_NS {

constexpr int TX = 32, TY = 8;
constexpr int HX = TX + 4, HY = TY + 4;  // OLD tile incl. 2 halo
constexpr int NX = TX + 2, NY = TY + 2;  // NEW tile incl. 1 halo
constexpr int NT = TX * TY;

template <typename R>
struct Params {
  Geom g;
  Phys p;
  Absorb<R> ab;
  R cc, c1, c2, c3;
  int incr;
  int kz;               // planes per block
  const R* in[6];
  const R* en[6];
  const R* b0[3];
  R* out[6];
};

template <typename R>
struct SmemOld {  // accessor over the OLD ring for push_cell
  const R* old;   // [3][6][HY][HX]
  const R* const* b0;
  long long gs, dj, dk;  // global index of the cell (for B0)
  int x, y;              // local position in OLD coordinates
  int s[3];              // ring slot of plane offset -1, 0, +1
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    if (c >= 6) return __ldg(b0[c - 6] + gs + di + djj * dj + dkk * dk);
    return old[((s[dkk + 1] * 6 + c) * HY + (y + djj)) * HX + (x + di)];
  }
  __device__ __forceinline__ R rho(int di, int djj, int dkk) const { return rho_at<R>(*this, di, djj, dkk); }
};

template <typename R>
struct SmemNew {  // accessor over the NEW ring for clean_cell
  const R* nw;    // [3][6][NY][NX]
  int x, y;
  int s[3];
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    return nw[((s[dkk + 1] * 6 + c) * NY + (y + djj)) * NX + (x + di)];
  }
};

__device__ __forceinline__ int slot(int p) { return (p + 3000) % 3; }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <typename R, bool C, bool B0, bool ABS, bool STAGE1>
__global__ void __launch_bounds__(NT) k_fused(const Params<R> P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* old = reinterpret_cast<R*>(smem_raw);  // 3*6*HY*HX
  R* nw = old + 3 * 6 * HY * HX;            // 3*6*NY*NX
  const Geom& g = P.g;
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int kb = blockIdx.z * P.kz;
  const int ke = min(kb + P.kz, g.sz);
  const bool per_x = P.p.bnd[0] == 1, per_y = P.p.bnd[1] == 1, per_z = P.p.bnd[2] == 1;

  auto load_old = [&](int p) {
    const int sl = slot(p);
    const int pz = clampi(p, -NG, g.sz + NG - 1);
    for (int e = tid; e < HX * HY; e += NT) {
      const int lx = e % HX, ly = e / HX;
      const int gi = clampi(x0 - 2 + lx, -NG, g.sx + NG - 1);
      const int gj = clampi(y0 - 2 + ly, -NG, g.sy + NG - 1);
      const long long gidx = g.idx(gi, gj, pz);
#pragma unroll
      for (int c = 0; c < 6; ++c) old[((sl * 6 + c) * HY + ly) * HX + lx] = P.in[c][gidx];
    }
  };

  auto compute_new = [&](int p) {
    const int sl = slot(p);
    for (int e = tid; e < NX * NY; e += NT) {
      const int nxl = e % NX, nyl = e / NX;
      const int gi = x0 - 1 + nxl, gj = y0 - 1 + nyl;
      R v[6];
      const bool in_range = gi >= -1 && gi <= g.sx && gj >= -1 && gj <= g.sy && p >= -1 && p <= g.sz;
      const bool out_x = gi < 0 || gi >= g.sx, out_y = gj < 0 || gj >= g.sy, out_z = p < 0 || p >= g.sz;
      const bool frozen = (out_x && !per_x) || (out_y && !per_y) || (out_z && !per_z);
      const int ox = nxl + 1, oy = nyl + 1;  // OLD coordinates
      if (!in_range) {
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = R(0);
      } else if (frozen) {
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = old[((sl * 6 + c) * HY + oy) * HX + ox];
      } else {
        SmemOld<R> a;
        a.old = old;
        a.b0 = P.b0;
        a.gs = g.idx(gi, gj, p);
        a.dj = g.px;
        a.dk = g.plane;
        a.x = ox;
        a.y = oy;
        a.s[0] = slot(p - 1);
        a.s[1] = sl;
        a.s[2] = slot(p + 1);
        R d[6];
        push_cell<R, C, B0>(a, P.cc, d);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const R f = old[((sl * 6 + c) * HY + oy) * HX + ox];
          const R fn = STAGE1 ? f : P.en[c][a.gs];
          v[c] = combine<R, C>(P.c1, P.c2, P.c3, fn, f, d[c], P.incr != 0);
        }
        if (ABS) absorb_cell<R>(P.ab, gi + P.p.x0, gi + P.p.y0, p + P.p.z0, v);
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) nw[((sl * 6 + c) * NY + nyl) * NX + nxl] = v[c];
    }
  };

  auto clean_store = [&](int k) {
    const int lx = tid % TX, ly = tid / TX;
    const int gi = x0 + lx, gj = y0 + ly;
    if (gi >= g.sx || gj >= g.sy) return;
    SmemNew<R> a;
    a.nw = nw;
    a.x = lx + 1;
    a.y = ly + 1;
    a.s[0] = slot(k - 1);
    a.s[1] = slot(k);
    a.s[2] = slot(k + 1);
    R e[3];
    clean_cell<R, C>(a, e);
    R v[6] = {e[0], e[1], e[2], a(BX, 0, 0, 0), a(BY, 0, 0, 0), a(BZ, 0, 0, 0)};
    // the cell and its periodic images in the ghost shell (two per axis when s < 4)
    int xs[3] = {gi, gi, gi}, ys[3] = {gj, gj, gj}, zs[3] = {k, k, k};
    int nxs = 1, nys = 1, nzs = 1;
    if (per_x && gi < NG) xs[nxs++] = gi + g.sx;
    if (per_x && gi >= g.sx - NG) xs[nxs++] = gi - g.sx;
    if (per_y && gj < NG) ys[nys++] = gj + g.sy;
    if (per_y && gj >= g.sy - NG) ys[nys++] = gj - g.sy;
    if (per_z && k < NG) zs[nzs++] = k + g.sz;
    if (per_z && k >= g.sz - NG) zs[nzs++] = k - g.sz;
    for (int a2 = 0; a2 < nzs; ++a2)
      for (int a1 = 0; a1 < nys; ++a1)
        for (int a0 = 0; a0 < nxs; ++a0) {
          const long long o = g.idx(xs[a0], ys[a1], zs[a2]);
#pragma unroll
          for (int c = 0; c < 6; ++c) P.out[c][o] = v[c];
        }
  };

  load_old(kb - 2);
  load_old(kb - 1);
  load_old(kb);
  __syncthreads();
  compute_new(kb - 1);
  __syncthreads();
  load_old(kb + 1);
  __syncthreads();
  compute_new(kb);
  __syncthreads();  // compute_new(kb) reads OLD(kb-1), whose slot load_old(kb+2) reuses
  for (int k = kb; k < ke; ++k) {
    load_old(k + 2);
    __syncthreads();
    compute_new(k + 1);
    __syncthreads();
    clean_store(k);
  }
}

}  // namespace FFE_FUSED_NS

#ifdef FFE_FUSED_EXACT
#define FFE_LAUNCH_NAME launch_fused_stage_exact
#else
#define FFE_LAUNCH_NAME launch_fused_stage
#endif

template <typename R, bool C>
void FFE_LAUNCH_NAME(const Geom& g, const Phys& p, const Absorb<R>& ab, R cc, R c1, R c2, R c3, bool incr, int stage,
                     const CEB<R>& in, const CEB<R>& en, const CEB<R>& b0, bool has_b0, const EB<R>& out,
                     cudaStream_t st) {
  using namespace FFE_FUSED_NS;
  Params<R> P;
  P.g = g;
  P.p = p;
  P.ab = ab;
  P.cc = cc;
  P.c1 = c1;
  P.c2 = c2;
  P.c3 = c3;
  P.incr = incr ? 1 : 0;
  for (int c = 0; c < 6; ++c) {
    P.in[c] = in.c[c];
    P.en[c] = en.c[c];
    P.out[c] = out.c[c];
  }
  for (int c = 0; c < 3; ++c) P.b0[c] = b0.c[c];
  const int tiles_x = (g.sx + TX - 1) / TX, tiles_y = (g.sy + TY - 1) / TY;
  // enough blocks for ~16 per SM on 152 SMs, at least 4 planes per block
  long long want = 152LL * 16;
  int kz = (int)std::max(4LL, std::min<long long>(64, ((long long)g.sz * tiles_x * tiles_y + want - 1) / want));
  kz = std::min(kz, g.sz);
  P.kz = kz;
  const dim3 grid(tiles_x, tiles_y, (g.sz + kz - 1) / kz);
  const size_t smem = sizeof(R) * (3 * 6 * HY * HX + 3 * 6 * NY * NX);
  const bool abs = p.bnd[0] == 2;
  const bool s1 = stage == 1;
#define FFE_GO(B0V, ABSV, S1V)                                                                    \
  do {                                                                                            \
    auto kf = k_fused<R, C, B0V, ABSV, S1V>;                                                      \
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);             \
    kf<<<grid, NT, smem, st>>>(P);                                                                \
  } while (0)
  if (has_b0) {
    if (abs) { if (s1) FFE_GO(true, true, true); else FFE_GO(true, true, false); }
    else { if (s1) FFE_GO(true, false, true); else FFE_GO(true, false, false); }
  } else {
    if (abs) { if (s1) FFE_GO(false, true, true); else FFE_GO(false, true, false); }
    else { if (s1) FFE_GO(false, false, true); else FFE_GO(false, false, false); }
  }
#undef FFE_GO
}

#ifndef FFE_FUSED_EXACT
void fused_tile_shape(int* tx, int* ty) {
  *tx = fused_fast::TX;
  *ty = fused_fast::TY;
}
#endif

#define FFE_INST_F(R, C)                                                                                          \
  template void FFE_LAUNCH_NAME<R, C>(const Geom&, const Phys&, const Absorb<R>&, R, R, R, R, bool, int,         \
                                      const CEB<R>&, const CEB<R>&, const CEB<R>&, bool, const EB<R>&, cudaStream_t);
FFE_INST_F(float, false)
FFE_INST_F(float, true)
FFE_INST_F(double, false)

}  // namespace ffe
