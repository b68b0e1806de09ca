// ffe_fused.cu — one launch per SSP-RK3 stage: computeRho + rk3Push +
// rk3Update (+ absorbing shell) + ghost fill + cleanEpar + ghost fill.
//
// A block owns a TX x TY column of cells and marches in z through a chunk of
// planes.  Shared memory holds the plane rings (standard layout; the lean
// layout of the plain FP32 variant is described at Rings):
//   OLD (depth 5): stage-input E,B over the tile + 2 halo cells, one TMA box
//                  per component and plane, fetched two planes ahead;
//   EN  (depth 2): step-start E,B over the tile + 1 halo (stages 2 and 3),
//                  fetched one plane ahead;
//   NEW (depth 4): updated, not yet cleaned E,B over the tile + 1 halo.
// Per plane k:  one thread issues TMA for OLD(k+3..k+4), EN(k+2);
//               wait OLD(k+2), EN(k+1) -> NEW(k+1) = push + update on
//               tile+1 (the 34 x (TY+2) region, one or two cells per
//               thread) -> barrier -> clean plane k on the tile from
//               NEW(k-1..k+1), store E'' and B'.
// With four NEW slots the clean of plane k and the push of plane k+2 touch
// different slots, so one barrier per plane suffices and warps that have no
// clean work move on to the next push.  A stage reads E,B (and the
// step-start E,B for stages 2-3) once from HBM and writes E,B once; the halo
// ring of NEW (1.24x the push work of a 32 x 12 tile, 1.33x of 32 x 8) is
// recomputed instead of making a second pass over memory.  The plain FP32
// variant's fast path evaluates the two cells a thread owns as float2 pairs
// with the paired FP32 instructions (see Body, ffe_physics.cuh).
//
// Ghosts.  The reference refreshes ghosts by exchangeFields after the update
// and after the cleaning (src/tristanmainloop.F90:59-61).  Here a cell lying
// within 2 cells of a periodic face is also stored at its periodic images in
// the ghost shell, so the output arrays leave the kernel with valid ghosts
// and the next stage reads plain indices.  On open / absorbing axes ghosts
// keep the values they were given at set-up (no neighbour sends them,
// src/tools/helpers.F90:27-45), and NEW takes those frozen values there.
//
// Waits on the TMA barriers are bounded: a block that gives up sets the error
// word (read by ffe_synchronize as FFE_ETIMEOUT), drains its copies in flight
// with bounded waits and returns.
//
// Compiled twice: normally (multiply-add contraction and, in FP32, the
// reciprocal-multiply quotient) as the fast path, and with -fmad=false under
// FFE_FUSED_EXACT with correctly rounded division (bit-comparable with the
// oracle).  Compiled a third and fourth time with -DFFE_BATCH_TY=8 / 16 for the
// batched launches (many grids per launch, see k_fused_batch), and a fifth
// time with -DFFE_BATCH_TY=8 -DFFE_BATCH_SPEC for the batched launches whose
// grids all share one B0 / absorbing-layer variant (k_fused_batch_var).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <climits>
#include <cstring>
#include "ffe_kernels.h"
#include "ffe_fused_types.cuh"
#include "ffe_physics.cuh"
#include "ffe_psr.cuh"

#if defined(FFE_BATCH_TY)
#define FFE_CAT2(a, b) a##b
#define FFE_CAT(a, b) FFE_CAT2(a, b)
#if defined(FFE_BATCH_SPEC)
#define FFE_FUSED_NS FFE_CAT(FFE_CAT(fused_batch, FFE_BATCH_TY), s)
#else
#define FFE_FUSED_NS FFE_CAT(fused_batch, FFE_BATCH_TY)
#endif
#define FFE_FAST true
#elif defined(FFE_FUSED_EXACT)
#define FFE_FUSED_NS fused_exact
#define FFE_FAST false
#else
#define FFE_FUSED_NS fused_fast
#define FFE_FAST true
#endif

namespace ffe {
namespace FFE_FUSED_NS {

constexpr int TX = FUSED_TX;
constexpr int OW = TX + 4;               // OLD/EN box width (cells x0-2 .. x0+TX+1)
constexpr int NX = TX + 2;               // NEW tile width (tile + 1 halo)
constexpr int DN = 4;                    // NEW ring depth
constexpr long long WAIT_LIMIT = 1LL << 22;
// Periodic images of the cleaned cells: written by the batched kernels as they
// clean (one launch covers many grids).  The single-grid kernels store
// without a branch, through predicated stores: every cleaning thread stores
// its cells (predicate: the cell lies in the grid) and, as a second set, their
// x image (predicate: the cell lies within NG of a periodic x face; the ghost
// columns share their 32-byte sectors with the cells stored next to them).
// The ghost rows and planes of periodic y and z (and a second x image, when
// sx < 2 NG) are copied by the ghost fill that follows each stage launch
// (k_fill, whole rows).
#if defined(FFE_FUSED_EXACT)
constexpr bool FFE_FUSED_EXACT_BUILD = true;
#else
constexpr bool FFE_FUSED_EXACT_BUILD = false;
#endif

// The six components of a cell at q, q + st, ..., q + 5 st, stored only when
// p holds (one predicate, six predicated st.global; no branch).  No memory
// clobber: nothing in the stage kernel reads the arrays it stores to, so the
// stores may be scheduled among the next plane's shared-memory loads.
__device__ __forceinline__ void store6_if(bool p, float* q, long long st, const float (&v)[6]) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %0, 0;\n\t"
      "@p st.global.f32 [%1], %7;\n\t@p st.global.f32 [%2], %8;\n\t@p st.global.f32 [%3], %9;\n\t"
      "@p st.global.f32 [%4], %10;\n\t@p st.global.f32 [%5], %11;\n\t@p st.global.f32 [%6], %12;\n\t}"
      ::"r"((int)p), "l"(q), "l"(q + st), "l"(q + 2 * st), "l"(q + 3 * st), "l"(q + 4 * st), "l"(q + 5 * st),
      "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]));
}
__device__ __forceinline__ void store6_if(bool p, double* q, long long st, const double (&v)[6]) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %0, 0;\n\t"
      "@p st.global.f64 [%1], %7;\n\t@p st.global.f64 [%2], %8;\n\t@p st.global.f64 [%3], %9;\n\t"
      "@p st.global.f64 [%4], %10;\n\t@p st.global.f64 [%5], %11;\n\t@p st.global.f64 [%6], %12;\n\t}"
      ::"r"((int)p), "l"(q), "l"(q + st), "l"(q + 2 * st), "l"(q + 3 * st), "l"(q + 4 * st), "l"(q + 5 * st),
      "d"(v[0]), "d"(v[1]), "d"(v[2]), "d"(v[3]), "d"(v[4]), "d"(v[5]));
}
// probes of a wait when the test flag withholds a copy (FFE_FLAG_TEST_WITHHOLD_COPY)
constexpr long long TEST_WAIT_LIMIT = 1LL << 14;

// Tile of height TY: OLD boxes of OH rows (y0-2 .. y0+TY+1), EN boxes of EH
// rows (y0-1 .. y0+TY), NEW planes of NY rows; OLD and EN rows are OW words,
// NEW rows NX words.  A thread owns CPT cells stacked in y (rows CPT*q .. CPT*q +
// CPT-1 of the NEW region for the update, of the tile for the cleaning), so
// the per-plane bookkeeping and the neighbour loads the cells share are paid
// once for CPT cells.  The update threads are laid out on rows of TP (thread
// t at x = t % TP, row group q = t / TP; lanes at x >= NX have no cell): TP =
// OW for two cells per thread, so that a warp's lanes fall on consecutive
// words of an OLD row; TP = NX for one, so that no lane idles.
// TY = 8, CPT = 2: 34 x 10 = 340 cells on 5 row pairs, 192 threads (128 of
// them also clean 32 x 8); CPT = 1: 340 cells, 352 threads.
// With two cells per thread the update threads are laid out one warp per
// row pair (WR): warp w < NY/2 takes x = 0..31 of the NEW region's row pair w,
// so that its 32 lanes read 32 consecutive words of each OLD row and write 32
// consecutive words of each NEW row (no shared-memory bank conflict), and the
// lanes of the last warp take the two remaining columns of every row pair.
template <int TY, int CPT = 1>
struct Tile {
  static constexpr int OH = TY + 4, EH = TY + 2, NY = TY + 2;
  static_assert(NY % CPT == 0 && TY % CPT == 0, "cells per thread must divide the tile rows");
  static constexpr bool WR = CPT == 2;
  static constexpr int RG = NY / CPT;  // row groups of the NEW region
  static constexpr int TP = CPT == 1 ? NX : OW;
  static constexpr int NT = WR ? (RG + (2 * RG + 31) / 32) * 32 : (TP * RG + 31) / 32 * 32;
  static constexpr int NCLEAN = TX * TY / CPT;  // threads that clean
};
// The batched kernel that switches variants per grid inlines the four B0 /
// absorbing-layer variants of the body; with one cell per thread it stays at
// two blocks per SM (TY = 8).
constexpr int BATCH_CPT = 1;

// Ring layout by kind RK.  0, standard (FP64, the B0 and absorbing-layer
// variants, the per-grid-switch batched kernel): OLD ring of 5 planes (two
// planes of copies ahead of use), step-start fields in a 2-plane TMA ring.
// 1, lean (the plain FP32 variant): OLD ring of 4 planes (one plane ahead),
// step-start fields in a single TMA slot, refilled as soon as every thread has
// finished the update that read it and waited for just before the next
// update's RK combination, so that the push hides the copy: 83 KB of shared
// memory at TY = 8, 111 KB at TY = 12 (two blocks per SM).  NEW rows are NX
// words in both.
template <int RK>
struct Rings {
  static constexpr int DO = RK == 1 ? 4 : 5, DE = RK == 0 ? 2 : 1;
  static constexpr int NP = NX;  // NEW row pitch
};

template <typename R, int TY, int RK = 0> struct Sizes {
  static constexpr int OLDBOX = ((OW * Tile<TY>::OH * (int)sizeof(R) + 127) / 128) * 128 / (int)sizeof(R);
  static constexpr int ENBOX = ((OW * Tile<TY>::EH * (int)sizeof(R) + 127) / 128) * 128 / (int)sizeof(R);
  static constexpr int NEWPL = Tile<TY>::NY * Rings<RK>::NP;  // one component of one NEW plane
  static constexpr int OLD = Rings<RK>::DO * 6 * OLDBOX;
  static constexpr int EN = Rings<RK>::DE * 6 * ENBOX;
  static constexpr int NEW = DN * 6 * NEWPL;
  static constexpr int BARS = Rings<RK>::DO + Rings<RK>::DE;
  static constexpr size_t BYTES = sizeof(R) * (size_t)(OLD + EN + NEW) + 8 * BARS;
};

// Configuration of the single-variant kernels (k_fused, k_fused_batch_var)
// by element type, precision mode C, variant and tile height: the plain FP32
// variant (no B0, no absorbing layer) takes two cells per thread and the lean
// rings; on the fast path it evaluates both cells at once with the paired
// FP32 instructions (PK; FP32CD with double-float denominators), which needs
// up to 168 registers (two blocks
// per SM); the single-grid kernel runs it at tile height PLAIN_TY (12: two
// blocks per SM by shared memory), the batched kernels at 8, where the exact
// path and FP32CD run at three blocks per SM (96 registers); the B0 and
// absorbing-layer variants, measured slower with two
// cells per thread (a 160^3 pulsar stage: 321 us against 215 us), and FP64
// take one cell per thread and the standard rings (two blocks per SM in FP32,
// one in FP64).
template <typename R, int C, bool B0, bool ABS, int TY>
struct Body {
  static constexpr bool LEAN = sizeof(R) == 4 && !B0 && !ABS;
  static constexpr int CPT = LEAN ? 2 : 1;
  static constexpr bool PK = LEAN && FFE_FAST;
  static constexpr int RK = LEAN ? 1 : 0;
  static constexpr int NT = Tile<TY, CPT>::NT;
  static constexpr int MINB = (PK || (LEAN && TY > 8)) ? 2 : (LEAN ? 3 : (sizeof(R) == 4 ? 2 : 1));
  static constexpr size_t SMEM = Sizes<R, TY, RK>::BYTES;
};

// Accessor over global arrays around linear index s (used for halo cells that
// are computed at their periodic image).
template <typename R>
struct GlobalAcc {
  const R* f[6];
  const R* const* b0;
  long long s, dj, dk;
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    const long long o = s + di + djj * dj + dkk * dk;
    return c >= 6 ? __ldg(b0[c - 6] + o) : __ldg(f[c] + o);
  }
  __device__ __forceinline__ R rho(int di, int djj, int dkk) const { return rho_at<R>(*this, di, djj, dkk); }
};

// ---- PTX helpers: mbarrier + TMA ------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: true when the phase completed (one probe in the common
// case), false after `limit` probes
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, long long limit = WAIT_LIMIT) {
  if (__builtin_expect(mbar_try_wait(bar, parity), 1)) return true;
  for (long long it = 1; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap* map, int x, int y, int z, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// Accessor over the OLD ring for push_cell: b[dk+1] points at this thread's
// cell in plane p+dk, so every (component, di, dj) offset is a constant.
template <typename R, int TY>
struct SmemOld {
  const R* b[3];
  const R* const* b0;
  long long gs, dj, dk;  // global index of the cell (for B0)
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    if (c >= 6) return __ldg(b0[c - 6] + gs + di + djj * dj + dkk * dk);
    return b[dkk + 1][c * Sizes<R, TY>::OLDBOX + djj * OW + di];
  }
  __device__ __forceinline__ R rho(int di, int djj, int dkk) const { return rho_at<R>(*this, di, djj, dkk); }
};

// Accessor over the NEW ring for clean_cell.
template <typename R, int TY, int RK>
struct SmemNew {
  const R* b[3];
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    return b[dkk + 1][c * Sizes<R, TY, RK>::NEWPL + djj * Rings<RK>::NP + di];
  }
};

// Accessors over the OLD and NEW rings for the packed two-cell forms:
// float2 {value at the thread's lower cell, value at its upper cell}.
template <int TY>
struct SmemOldPair {
  const float* b[3];
  __device__ __forceinline__ float2 operator()(int c, int di, int djj, int dkk) const {
    const float* q = b[dkk + 1] + (c * Sizes<float, TY>::OLDBOX + djj * OW + di);
    return make_float2(q[0], q[OW]);
  }
};
template <int TY>
struct SmemNewPair {
  const float* b[3];
  __device__ __forceinline__ float2 operator()(int c, int di, int djj, int dkk) const {
    const float* q = b[dkk + 1] + (c * Sizes<float, TY, 1>::NEWPL + djj * Rings<1>::NP + di);
    return make_float2(q[0], q[Rings<1>::NP]);
  }
};

// One block's work: the TX x TY column (tile_x, tile_y) of a grid, planes of
// z-chunk `chunk`.  Shared by the single-grid kernel and the batched kernel.
// mi / me: the six tensor maps of the stage-input and step-start sets.
// RK: ring kind (0 standard, 1 lean; see Rings).
// Returns false when a wait on a copy gave up (the error word is set).
// PER: a grid periodic on every axis with no user BC (every plane of every
// tile takes the uniform update path; the per-cell boundary path and the
// twisted-footpoint BC are compiled out).
template <typename R, int C, bool B0, bool ABS, bool STAGE1, int TY, int CPT, int RK, bool PER = false>
__device__ __forceinline__ bool stage_body(const CUtensorMap* mi, const CUtensorMap* me, const Params<R>& P,
                                           int tile_x, int tile_y, int chunk) {
  constexpr bool LEAN = RK == 1;
  using S = Sizes<R, TY, RK>;
  using T = Tile<TY, CPT>;
  constexpr int DO = Rings<RK>::DO, DE = Rings<RK>::DE, NP = Rings<RK>::NP;
  constexpr int OH = T::OH, EH = T::EH;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  R* old = reinterpret_cast<R*>(smem_raw);
  R* en = old + S::OLD;
  R* nw = en + S::EN;
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(nw + S::NEW);
  const Geom g = P.g;
  const int tid = threadIdx.x;
  // the copy-issuing thread: first thread of the last warp, which has the
  // least work (it cleans nothing, and part of its lanes have no cell)
  constexpr int PRODUCER = T::NT - 32;
  const int x0 = tile_x * TX, y0 = tile_y * TY;
  const int kb = chunk * P.kz;
  const int ke = min(kb + P.kz, g.sz);
  const bool per_x = P.p.bnd[0] == 1, per_y = P.p.bnd[1] == 1, per_z = P.p.bnd[2] == 1;
  constexpr bool FD = FFE_FAST && sizeof(R) == 4;
  constexpr bool DF = C == 2;  // FP32CD: double-float denominators
  // fast-path sums as row-grouped trees in the plain variant (whatever the
  // kernel), in the reference's order in the B0 and absorbing-layer variants
  constexpr bool TREE = !B0 && !ABS;
  // the plain FP32 variant's fast path: the two cells of a thread as float2
  // pairs through the paired FP32 instructions
  // (FP32CD too, with DF)
  constexpr bool PK = FD && LEAN && CPT == 2;
  const R cc = P.cc, c1 = P.c1, c2 = P.c2, c3 = P.c3, ct = P.ct;
  const bool incr = P.incr != 0;
  R* const out0 = P.out0;
  const long long fs = P.fs;

  const unsigned bar_old = smem_u32(bars), bar_en = smem_u32(bars + DO);

  // ---- producer (thread PRODUCER): TMA copies of whole planes -----------
  // OLD plane p lives in slot (p - kb + 2) % DO, EN plane p in (p - kb + 1) % DE.
  int old_next = kb - 2, en_next = kb - 1;
  const int old_last = ke + 1, en_last = ke;
  // failure-detection test: the copy of OLD plane kb+1 is left out, so the
  // wait for it runs out after TEST_WAIT_LIMIT probes
  const int withheld = P.p.withhold_copy ? kb + 1 : INT_MIN;
  const long long wlim = P.p.withhold_copy ? TEST_WAIT_LIMIT : WAIT_LIMIT;
  auto issue_old = [&](int p) {
    if (p == withheld) return;
    const int s = (p - kb + 2) % DO;
    const unsigned bar = bar_old + 8 * s;
    mbar_expect_tx(bar, 6u * OW * OH * sizeof(R));
#pragma unroll
    for (int c = 0; c < 6; ++c)
      tma_load_3d(smem_u32(old + (s * 6 + c) * S::OLDBOX), mi + c, x0, y0, p + NG, bar);
  };
  auto issue_en = [&](int p) {
    const int s = (p - kb + 1) % (DE > 0 ? DE : 1);
    const unsigned bar = bar_en + 8 * s;
    mbar_expect_tx(bar, 6u * OW * EH * sizeof(R));
#pragma unroll
    for (int c = 0; c < 6; ++c)
      tma_load_3d(smem_u32(en + (s * 6 + c) * S::ENBOX), me + c, x0, y0 + 1, p + NG, bar);
  };
  if (tid == PRODUCER) {
    for (int s = 0; s < DO + DE; ++s) mbar_init(smem_u32(bars + s), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == PRODUCER) {  // prologue fetch: OLD kb-2 .. kb+DO-3, EN kb-1 .. kb+DE-2
    for (; old_next <= min(kb + DO - 3, old_last); ++old_next) issue_old(old_next);
    if (!STAGE1 && DE > 0)
      for (; en_next <= min(kb + DE - 2, en_last); ++en_next) issue_en(en_next);
  }
  // Once every thread has finished compute_new(k), the OLD slots of planes up
  // to k-1 and the EN slot of plane k are free, so OLD may run to k+DO-1 and
  // EN to k+DE.
  auto refill = [&](int k) {
    if (tid != PRODUCER) return;
    while (old_next <= old_last && old_next <= k + DO - 1) issue_old(old_next++);
    if (!STAGE1 && DE > 0)
      while (en_next <= en_last && en_next <= k + DE) issue_en(en_next++);
  };

  // ---- consumers: rolling ring state, uniform across the block ------------
  // Planes are waited for in order, each exactly once.
  int ow_slot = 0;         // slot of the next OLD plane to wait for (kb-2 first)
  unsigned ow_par = 0;     // its phase parity
  int ew = 0;              // EN planes waited so far (kb-1 first)
  auto wait_old = [&]() {
    const bool ok = mbar_wait(bar_old + 8 * ow_slot, ow_par, wlim);
    if (++ow_slot == DO) { ow_slot = 0; ow_par ^= 1u; }
    return ok;
  };
  // the single EN slot of the lean rings is waited for inside compute_new
  constexpr bool EN_INNER = LEAN && !STAGE1;
  auto wait_en_slot = [&]() {
    if constexpr (STAGE1 || DE == 0) return true;
    const bool ok = mbar_wait(bar_en + 8 * (ew % DE), (unsigned)((ew / DE) & 1), wlim);
    ++ew;
    return ok;
  };
  auto wait_en = [&]() {
    if constexpr (EN_INNER) return true;
    return wait_en_slot();
  };

  // ---- per-thread constants --------------------------------------------------
  // update cells of this thread: (nxl, CPT * nq + r) of the NEW region, r < CPT
  int nxl, nq;
  if constexpr (T::WR) {
    const int w = tid >> 5, l = tid & 31;
    if (w < T::RG) {
      nq = w;
      nxl = l;
    } else {  // the last warp: columns TX, TX+1 of every row group
      const int e = (w - T::RG) * 32 + l;
      nq = e >> 1;
      nxl = TX + (e & 1);
    }
  } else {
    nxl = tid % T::TP;
    nq = tid / T::TP;
  }
  const bool cell_thread = nxl < NX && nq < T::NY / CPT;
  const int gi = x0 - 1 + nxl, gj0 = y0 - 1 + CPT * nq;
  const bool out_x = gi < 0 || gi >= g.sx;
  const R* oth = old + (CPT * nq + 1) * OW + (nxl + 1);  // cell 0 in OLD slot 0; cell r at + r * OW
  const R* enth = en + CPT * nq * OW + (nxl + 1);        // in EN slot 0
  R* nwth = nw + CPT * nq * NP + nxl;                    // in NEW slot 0; cell r at + r * NP
  // sums carried from plane to plane by the paired forms (push_pair_fast,
  // clean_pair_fast); primed at the first plane of the chunk and after a
  // plane that took the per-cell path
  PushCarry pcar;
  bool pcar_ok = false;
  CleanCarry ccar;
  bool ccar_ok = false;
  // B0 is read from global memory around the cell; cells of a partial tile
  // beyond the grid read around the nearest halo cell instead (their values
  // are computed but never used)
  long long gbase[CPT];
#pragma unroll
  for (int r = 0; r < CPT; ++r)
    gbase[r] = B0 ? g.idx(min(max(gi, -1), g.sx), min(max(gj0 + r, -1), g.sy), 0) : 0;
  // No cell of the 34x(TY+2) region is a frozen ghost in x, y: every axis is
  // periodic or the region lies inside [-1, s].  On a periodic axis a partial
  // tile qualifies too: its cells beyond the halo (index > s) compute values
  // from the zero-filled or padded part of the boxes that no cleaning reads.
  const bool simple_xy = (per_x || (x0 >= 1 && x0 + TX + 1 <= g.sx)) &&
                         (per_y || (y0 >= 1 && y0 + TY + 1 <= g.sy));
  // periodic and open axes together: a halo cell outside a periodic face whose
  // image lies next to an open face takes the per-cell path (see below); such
  // cells exist only where the tile (or plane) touches a periodic face and
  // reaches an open face's boundary layer
  const bool mixed = (per_x || per_y || per_z) && !(per_x && per_y && per_z);
  const bool touch_per_xy = (per_x && (x0 == 0 || x0 + TX >= g.sx)) || (per_y && (y0 == 0 || y0 + TY >= g.sy));
  const bool near_open_xy = (!per_x && (x0 <= 1 || x0 + TX >= g.sx - 1)) ||
                            (!per_y && (y0 <= 1 || y0 + TY >= g.sy - 1));
  // no cell of the tile has a periodic image in x or y
  [[maybe_unused]] const bool no_xy_images = (!per_x || (x0 >= NG && x0 + TX <= g.sx - NG)) &&
                            (!per_y || (y0 >= NG && y0 + TY <= g.sy - NG));

  // NEW(p): push + update on this thread's cells.  so = OLD slot of plane
  // p-1, m = p - (kb - 1) (EN slot m % DE, NEW slot m % 4).  Returns false if
  // the wait for the step-start fields (lean rings) gave up.
  auto compute_new = [&](int p, int so, int m) -> bool {
    if (!cell_thread) return true;
    bool en_ready = true;
    if constexpr (EN_INNER && !PK) en_ready = wait_en_slot();
    const int s1 = so == DO - 1 ? 0 : so + 1;
    const int s2 = s1 == DO - 1 ? 0 : s1 + 1;
    const R* o0 = oth + so * (6 * S::OLDBOX);
    const R* o1 = oth + s1 * (6 * S::OLDBOX);
    const R* o2 = oth + s2 * (6 * S::OLDBOX);
    const R* e1 = enth + (m & (DE > 0 ? DE - 1 : 0)) * (6 * S::ENBOX);
    R* dst = nwth + (m & (DN - 1)) * (6 * S::NEWPL);
    // push + update (+ absorbing shell) of cell r from the OLD and EN rings.
    // Only shared-memory loads: the loads the CPT cells share are made once.
    auto push_update = [&](int r, R w[6]) {
      SmemOld<R, TY> a;
      a.b[0] = o0 + r * OW;
      a.b[1] = o1 + r * OW;
      a.b[2] = o2 + r * OW;
      a.b0 = P.b0;
      a.gs = gbase[r] + (long long)p * g.plane;
      a.dj = g.px;
      a.dk = g.plane;
      R d[6];
      if constexpr (FD) push_cell_fast<B0, TREE, SmemOld<R, TY>, DF>(a, cc, d);
      else push_cell<R, C, B0, SmemOld<R, TY>, false>(a, cc, d);
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const R f = a.b[1][c * S::OLDBOX];
        R fn;
        if constexpr (STAGE1) fn = f;
        else fn = e1[c * S::ENBOX + r * OW];
        w[c] = combine<R, C>(c1, c2, c3, fn, f, d[c], incr);
      }
      if constexpr (ABS && FD)
        absorb_cell_fast(P.ab, gi + P.p.x0, shell_jg(P.ab, gi, gj0 + r, P.p.y0), p + P.p.z0, w);
      else if constexpr (ABS)
        absorb_cell<R>(P.ab, gi + P.p.x0, shell_jg(P.ab, gi, gj0 + r, P.p.y0), p + P.p.z0, w);
    };
    R v[CPT][6];
    bool frozen_cell[CPT];
    // block-uniform common case: every cell of the region is computed
    const bool all_push = PER || (simple_xy && (per_z || (p >= 0 && p < g.sz)) &&
                          !(mixed && (touch_per_xy || (per_z && (p < 0 || p >= g.sz))) &&
                            (near_open_xy || (!per_z && (p <= 0 || p >= g.sz - 1)))));
    if (all_push) {
      if constexpr (PK) {
        SmemOldPair<TY> a;
        a.b[0] = reinterpret_cast<const float*>(o0);
        a.b[1] = reinterpret_cast<const float*>(o1);
        a.b[2] = reinterpret_cast<const float*>(o2);
        float2 d[6];
        if (!pcar_ok) push_carry_prime(a, pcar);
        push_pair_fast<DF>(a, (float)cc, d, pcar);
        pcar_ok = true;
        if constexpr (EN_INNER) en_ready = wait_en_slot();
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const float2 f = a(c, 0, 0, 0);
          float2 fn = f;
          if constexpr (!STAGE1) {
            const float* q = reinterpret_cast<const float*>(e1) + c * S::ENBOX;
            fn = make_float2(q[0], q[OW]);
          }
          const float2 w = combine2<C>((float)c1, (float)c2, (float)c3, fn, f, d[c], incr);
          v[0][c] = (R)w.x;
          v[CPT - 1][c] = (R)w.y;
        }
#pragma unroll
        for (int r = 0; r < CPT; ++r) frozen_cell[r] = false;
      } else {
#pragma unroll
        for (int r = 0; r < CPT; ++r) {
          push_update(r, v[r]);
          frozen_cell[r] = false;
        }
      }
    } else {
      pcar_ok = false;
      if constexpr (EN_INNER && PK) en_ready = wait_en_slot();
#pragma unroll
      for (int r = 0; r < CPT; ++r) {
        const int gj = gj0 + r;
        const bool xy_in = gi >= -1 && gi <= g.sx && gj >= -1 && gj <= g.sy;
        const bool out_y = gj < 0 || gj >= g.sy;
        const bool out_xy_open = (out_x && !per_x) || (out_y && !per_y);
        const bool in_range = xy_in && p >= -1 && p <= g.sz;
        const bool out_z = p < 0 || p >= g.sz;
        const bool frozen = out_xy_open || (out_z && !per_z);
        frozen_cell[r] = in_range && frozen;
        bool push = true;
        if (!in_range || frozen) {
#pragma unroll
          for (int c = 0; c < 6; ++c) v[r][c] = in_range ? o1[r * OW + c * S::OLDBOX] : R(0);
          push = false;
        } else if (out_x || out_y || out_z) {
          // A halo cell outside a periodic face is the periodic image of an
          // interior cell.  If that cell lies next to an open face, its stencil
          // reaches ghosts of the open face at positions whose counterparts here
          // are ghosts of both faces, which keep their own (frozen) values: the
          // copy at this position would differ.  Compute it at the image instead.
          const int wi = gi < 0 ? gi + g.sx : (gi >= g.sx ? gi - g.sx : gi);
          const int wj = gj < 0 ? gj + g.sy : (gj >= g.sy ? gj - g.sy : gj);
          const int wk = p < 0 ? p + g.sz : (p >= g.sz ? p - g.sz : p);
          const bool near_open = (!per_x && (wi == 0 || wi == g.sx - 1)) || (!per_y && (wj == 0 || wj == g.sy - 1)) ||
                                 (!per_z && (wk == 0 || wk == g.sz - 1));
          if (near_open) {
            GlobalAcc<R> a;
            for (int c = 0; c < 6; ++c) a.f[c] = P.in0 + c * fs;
            a.b0 = P.b0;
            a.s = g.idx(wi, wj, wk);
            a.dj = g.px;
            a.dk = g.plane;
            R d[6];
            if constexpr (FD) push_cell_fast<B0, TREE, GlobalAcc<R>, DF>(a, cc, d);
            else push_cell<R, C, B0, GlobalAcc<R>, false>(a, cc, d);
#pragma unroll
            for (int c = 0; c < 6; ++c) {
              const R f = __ldg(P.in0 + (c * fs + a.s));
              const R fn = STAGE1 ? f : __ldg(P.en0 + (c * fs + a.s));
              v[r][c] = combine<R, C>(c1, c2, c3, fn, f, d[c], incr);
            }
            push = false;
          }
        }
        if (push) push_update(r, v[r]);
      }
    }
    // Twisted-footpoint BC (user_uniform) between the update and the cleaning,
    // on the planes z_glob <= 0 and >= gsz.  Frozen ghosts take the formula at
    // their own position; a halo cell on a periodic face is the image of an
    // interior cell, which took the formula at the image position.
    if (!PER && P.ubc && (p + P.p.z0 <= 0 || p + P.p.z0 >= P.p.gsz)) {
#pragma unroll
      for (int r = 0; r < CPT; ++r) {
        int bi = gi, bj = gj0 + r;
        if (!frozen_cell[r]) {
          bi = bi < 0 ? bi + g.sx : (bi >= g.sx ? bi - g.sx : bi);
          bj = bj < 0 ? bj + g.sy : (bj >= g.sy ? bj - g.sy : bj);
        }
        uniform_bc_apply(P.ub, P.p, bi, bj, p, v[r][EX], v[r][EY], v[r][BZ]);
      }
    }
#pragma unroll
    for (int r = 0; r < CPT; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c) dst[r * NP + c * S::NEWPL] = v[r][c];
    return en_ready;
  };

  // cleaned cells of this thread: (lx, CPT * lq + r) of the tile, tid < NCLEAN
  const int lx = tid % TX, lq = tid / TX;
  const bool clean_thread = tid < T::NCLEAN;
  const int ci = x0 + lx, cj0 = y0 + CPT * lq;
  // periodic images of this column in x and y (two per axis when s < 4)
  int xs[3] = {ci, ci, ci}, nxs = 1;
  if (per_x && ci < NG) xs[nxs++] = ci + g.sx;
  if (per_x && ci >= g.sx - NG) xs[nxs++] = ci - g.sx;
  bool c_in[CPT], xy_images[CPT];
  // the x image stored by this thread's cells (single-grid kernels)
  const bool x_image = per_x && (ci < NG || ci >= g.sx - NG);
  const int x_shift = ci < NG ? g.sx : -g.sx;
  // a tile with a cell within NG of a periodic x face (block-uniform)
  const bool x_edge = per_x && (x0 < NG || x0 + TX > g.sx - NG);
  int cbase[CPT];  // in-plane offsets
#pragma unroll
  for (int r = 0; r < CPT; ++r) {
    const int cj = cj0 + r;
    c_in[r] = clean_thread && ci < g.sx && cj < g.sy;
    xy_images[r] = nxs > 1 || (per_y && (cj < NG || cj >= g.sy - NG));
    cbase[r] = c_in[r] ? (cj + NG) * g.px + ci + g.ox : 0;
  }
  const R* cth = nw + (CPT * lq + 1) * NP + (lx + 1);

  // clean plane k (m = k - kb: NEW slots of k-1, k, k+1 are m, m+1, m+2 mod 4)
  auto clean_store = [&](int k, int m) {
    if (!clean_thread) return;
    const R* n0 = cth + (m & (DN - 1)) * (6 * S::NEWPL);
    const R* n1 = cth + ((m + 1) & (DN - 1)) * (6 * S::NEWPL);
    const R* n2 = cth + ((m + 2) & (DN - 1)) * (6 * S::NEWPL);
    // all loads of the CPT cells first (they share neighbours), then the stores
    R v[CPT][6];
    if constexpr (PK) {
      SmemNewPair<TY> a;
      a.b[0] = reinterpret_cast<const float*>(n0);
      a.b[1] = reinterpret_cast<const float*>(n1);
      a.b[2] = reinterpret_cast<const float*>(n2);
      float2 e[3];
      if (!ccar_ok) clean_carry_prime(a, ccar);
      clean_pair_fast<DF>(a, e, 64.f * (float)ct, ccar);
      ccar_ok = true;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        v[0][c] = (R)e[c].x;
        v[CPT - 1][c] = (R)e[c].y;
        const float2 b = a(BX + c, 0, 0, 0);
        v[0][3 + c] = (R)b.x;
        v[CPT - 1][3 + c] = (R)b.y;
      }
    } else {
#pragma unroll
      for (int r = 0; r < CPT; ++r) {
        SmemNew<R, TY, RK> a;
        a.b[0] = n0 + r * NP;
        a.b[1] = n1 + r * NP;
        a.b[2] = n2 + r * NP;
        R e[3];
        if constexpr (FD) clean_cell_fast<TREE, SmemNew<R, TY, RK>, DF>(a, e, ct);
        else clean_cell<R, C, SmemNew<R, TY, RK>, false>(a, e, ct);
        v[r][0] = e[0];
        v[r][1] = e[1];
        v[r][2] = e[2];
        v[r][3] = a(BX, 0, 0, 0);
        v[r][4] = a(BY, 0, 0, 0);
        v[r][5] = a(BZ, 0, 0, 0);
      }
    }
#if !defined(FFE_BATCH_TY)
    const long long po = (long long)(k + NG) * g.plane;
#pragma unroll
    for (int r = 0; r < CPT; ++r) {
      R* const q = out0 + (po + cbase[r]);
      store6_if(c_in[r], q, fs, v[r]);
      if (x_edge) store6_if(c_in[r] && x_image, q + x_shift, fs, v[r]);
    }
#else
    const bool z_image = per_z && (k < NG || k >= g.sz - NG);
#pragma unroll
    for (int r = 0; r < CPT; ++r) {
      if (!c_in[r]) continue;
      if ((no_xy_images || !xy_images[r]) && !z_image) {
        R* q = out0 + ((long long)(k + NG) * g.plane + cbase[r]);
#pragma unroll
        for (int c = 0; c < 6; ++c, q += fs) *q = v[r][c];
        continue;
      }
      const int cj = cj0 + r;
      int ys[3] = {cj, cj, cj}, nys = 1;
      if (per_y && cj < NG) ys[nys++] = cj + g.sy;
      if (per_y && cj >= g.sy - NG) ys[nys++] = cj - g.sy;
      int zs[3] = {k, k, k}, nzs = 1;
      if (per_z && k < NG) zs[nzs++] = k + g.sz;
      if (per_z && k >= g.sz - NG) zs[nzs++] = k - g.sz;
      for (int a2 = 0; a2 < nzs; ++a2)
        for (int a1 = 0; a1 < nys; ++a1)
          for (int a0 = 0; a0 < nxs; ++a0) {
            const long long o = g.idx(xs[a0], ys[a1], zs[a2]);
#pragma unroll
            for (int c = 0; c < 6; ++c) out0[o + c * fs] = v[r][c];
          }
    }
#endif
  };

  // ---- prologue: NEW(kb-1), NEW(kb) ----------------------------------------
  // `failed` is block-uniform: every wait result goes through a barrier-OR.
  bool failed = __syncthreads_or(!(wait_old() & wait_old() & wait_old() & wait_en()));  // OLD kb-2..kb, EN kb-1
  if (!failed) {
    const bool ok0 = compute_new(kb - 1, 0, 0);
    const bool ok1 = wait_old() & wait_en();  // OLD kb+1, EN kb (standard rings)
    failed = __syncthreads_or(!(ok0 & ok1));
    if (!failed) {
      refill(kb - 1);
      failed = __syncthreads_or(!compute_new(kb, 1, 1));
    }
    if (!failed) {
      // ---- march: one barrier per plane ------------------------------------
      int so = 2;  // OLD slot of plane k for compute_new(k+1)
      for (int k = kb, m = 0; k < ke; ++k, ++m) {
        refill(k);
        bool late = !(wait_old() & wait_en());  // OLD k+2, EN k+1 (standard rings)
        if (!late) late = !compute_new(k + 1, so, m + 2);
        if (__syncthreads_or(late)) {
          failed = true;
          break;
        }
        clean_store(k, m);
        so = so == DO - 1 ? 0 : so + 1;
      }
    }
  }
  if (failed) {
    if (tid == PRODUCER) {
      atomicExch(P.err, 1);
      // drain the copies that may still be in flight: the last use of each slot
      for (int p = max(kb - 2, old_next - DO); p < old_next; ++p)
        if (p != withheld) mbar_wait(bar_old + 8 * ((p - kb + 2) % DO), (unsigned)(((p - kb + 2) / DO) & 1), wlim);
      if constexpr (!STAGE1 && DE > 0)
        for (int p = max(kb - 1, en_next - DE); p < en_next; ++p)
          mbar_wait(bar_en + 8 * ((p - kb + 1) % DE), (unsigned)(((p - kb + 1) / DE) & 1), wlim);
    }
    __syncthreads();
    return false;
  }
  // Every wait of this chunk has completed: invalidate the barriers so that a
  // persistent block may initialise them again for its next work item.
  __syncthreads();
  if (tid == PRODUCER)
    for (int s = 0; s < S::BARS; ++s) mbar_inval(smem_u32(bars + s));
  return true;
}

#if !defined(FFE_BATCH_TY)
// One grid: block (x, y, z) = (tile_x, tile_y, z-chunk), tile height TY
// (PLAIN_TY for the plain FP32 variant, FUSED_TY otherwise).
template <typename R, int C, bool B0, bool ABS, bool STAGE1, int TY, bool PER>
__global__ void __launch_bounds__(Body<R, C, B0, ABS, TY>::NT, Body<R, C, B0, ABS, TY>::MINB)
    k_fused(const __grid_constant__ Maps maps, const Params<R> P) {
  using CF = Body<R, C, B0, ABS, TY>;
  stage_body<R, C, B0, ABS, STAGE1, TY, CF::CPT, CF::RK, PER>(maps.in, maps.en, P, blockIdx.x, blockIdx.y,
                                                               blockIdx.z);
}
#else
// Many grids in one launch.  Work item w = (grid, tile_x, tile_y, z-chunk);
// the grids' parameters and tensor-map pointers come in the kernel's
// parameter space (a table of up to BATCH_MAX entries), so that, as in
// k_fused, every per-grid constant is read from the constant bank where it is
// used instead of occupying registers.  The B0 / absorbing-layer variant is
// chosen per grid.  With fewer blocks than items the blocks are persistent:
// block b takes items b, b + gridDim.x, ... (the host orders items by
// decreasing work).
template <typename R, int C, bool STAGE1, int TY>
__global__ void __launch_bounds__(Tile<TY, BATCH_CPT>::NT, (sizeof(R) == 4 && TY == 8) ? 2 : 1)
    k_fused_batch(const BatchItem* __restrict__ items, int nitems, const __grid_constant__ BoxTable<R> T) {
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const BatchItem it = items[w];
    const BatchBox<R>& e = T.b[it.box];
    bool ok;
    if (e.has_b0) {
      if (e.absorb)
        ok = stage_body<R, C, true, true, STAGE1, TY, BATCH_CPT, 0>(e.mi, e.me, e.P, it.tx, it.ty, it.tz);
      else
        ok = stage_body<R, C, true, false, STAGE1, TY, BATCH_CPT, 0>(e.mi, e.me, e.P, it.tx, it.ty, it.tz);
    } else {
      if (e.absorb)
        ok = stage_body<R, C, false, true, STAGE1, TY, BATCH_CPT, 0>(e.mi, e.me, e.P, it.tx, it.ty, it.tz);
      else
        ok = stage_body<R, C, false, false, STAGE1, TY, BATCH_CPT, 0>(e.mi, e.me, e.P, it.tx, it.ty, it.tz);
    }
    if (!ok) return;
  }
}

#if defined(FFE_BATCH_SPEC)
// Many grids of one variant (VAR: bit 1 B0, bit 0 absorbing layer) in one
// launch: the body of the single-grid kernel in its configuration for that
// variant (Cfg), items and table as in k_fused_batch.
template <typename R, int C, bool STAGE1, int TY, int VAR>
__global__ void __launch_bounds__(Body<R, C, (VAR & 2) != 0, (VAR & 1) != 0, TY>::NT,
                                  Body<R, C, (VAR & 2) != 0, (VAR & 1) != 0, TY>::MINB)
    k_fused_batch_var(const BatchItem* __restrict__ items, int nitems, const __grid_constant__ BoxTable<R> T) {
  using CF = Body<R, C, (VAR & 2) != 0, (VAR & 1) != 0, TY>;
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const BatchItem it = items[w];
    const BatchBox<R>& e = T.b[it.box];
    if (!stage_body<R, C, (VAR & 2) != 0, (VAR & 1) != 0, STAGE1, TY, CF::CPT, CF::RK>(e.mi, e.me, e.P, it.tx,
                                                                                       it.ty, it.tz))
      return;
  }
}
#endif
#endif

// ---- rotating-conductor boundary condition on the fused path ---------------
// The fused kernel cleans every cell before any boundary condition could act.
// For the pulsar setup the BC (user/user_psr.F90:72-332) modifies the cells of
// its bounding box B between the update and the cleaning, and the cleaning of
// a cell reads its neighbours, so the cells of B+1 (B dilated by one cell) are
// redone after the fused launch:
//   k_fix_update: uncleaned update (push + combine [+ shell]) on U = B+2 -> S1
//   k_fix_bc:     S2 = S1 with the BC applied inside r < 2R (reads S1 neighbours)
//   k_fix_clean:  clean the interior cells of B+1 from S2, store E'' and B'
// S1, S2 are compact U-shaped arrays (6 components).  Only for grids with no
// periodic axis (the pulsar runs open or absorbing), so U holds no image.
// Each step is a per-cell function of U coordinates (bi, bj, bk), launched
// over one grid (k_fix_*) or over many grids at once (k_fix_*_batch).

template <typename R>
struct BoxAcc {  // accessor over a compact U array around a cell
  const R* base;
  long long n, s, dj, dk;
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    return base[c * n + s + di + djj * dj + dkk * dk];
  }
};

// Only cells near the sphere S (r < 2R) of the BC matter: the cleaning is
// redone on S dilated by one cell (node distance < 2R + sqrt 3), which reads
// updated values on S dilated by two (< 2R + 2 sqrt 3).  The rest of the
// bounding box is skipped: its fused results stand.
struct FixMargin {
  static constexpr float clean = 1.8f, update = 3.6f;
};
template <typename R>
__device__ __forceinline__ bool fix_near(const FixParams<R>& F, int i, int j, int k, float margin) {
  const R ig = R(i + F.p.x0) - F.q.xc, jg = R(j + F.p.y0) - F.q.yc, kg = R(k + F.p.z0) - F.q.zc;
  const R lim = R(2) * F.q.radius + R(margin);
  return (ig * ig + jg * jg) + kg * kg < lim * lim;
}

template <typename R, int C, bool B0, bool ABS, bool STAGE1>
__device__ __forceinline__ void fix_update_cell(const FixParams<R>& F, int bi, int bj, int bk) {
  constexpr bool FD = FFE_FAST && sizeof(R) == 4;
  constexpr bool DF = C == 2;  // FP32CD: double-float denominators
  if (bi >= F.ux || bj >= F.uy || bk >= F.uz) return;
  const int i = F.ui + bi, j = F.uj + bj, k = F.uk + bk;
  if (!fix_near(F, i, j, k, FixMargin::update)) return;
  const Geom& g = F.g;
  const long long n = (long long)F.ux * F.uy * F.uz;
  const long long o = bi + (long long)F.ux * (bj + (long long)F.uy * bk);
  const long long s = g.idx(i, j, k);
  R v[6];
  if (i < 0 || i >= g.sx || j < 0 || j >= g.sy || k < 0 || k >= g.sz) {
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] = __ldg(F.in[c] + s);  // frozen ghost
  } else {
    GlobalAcc<R> a;
    for (int c = 0; c < 6; ++c) a.f[c] = F.in[c];
    a.b0 = F.b0;
    a.s = s;
    a.dj = g.px;
    a.dk = g.plane;
    R d[6];
    if constexpr (FD) push_cell_fast<B0, false, GlobalAcc<R>, DF>(a, F.cc, d);  // the reference's order of the sums
    else push_cell<R, C, B0, GlobalAcc<R>, false>(a, F.cc, d);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const R f = __ldg(F.in[c] + s);
      const R fn = STAGE1 ? f : __ldg(F.en[c] + s);
      v[c] = combine<R, C>(F.c1, F.c2, F.c3, fn, f, d[c], F.incr != 0);
    }
    if constexpr (ABS && FD)
      absorb_cell_fast(F.ab, i + F.p.x0, shell_jg(F.ab, i, j, F.p.y0), k + F.p.z0, v);
    else if constexpr (ABS)
      absorb_cell<R>(F.ab, i + F.p.x0, shell_jg(F.ab, i, j, F.p.y0), k + F.p.z0, v);
  }
#pragma unroll
  for (int c = 0; c < 6; ++c) F.s1[c * n + o] = v[c];
}

template <typename R>
__device__ __forceinline__ void fix_bc_cell(const FixParams<R>& F, int bi, int bj, int bk) {
  if (bi >= F.ux || bj >= F.uy || bk >= F.uz) return;
  const int i = F.ui + bi, j = F.uj + bj, k = F.uk + bk;
  if (!fix_near(F, i, j, k, FixMargin::update)) return;
  const long long n = (long long)F.ux * F.uy * F.uz;
  const long long o = bi + (long long)F.ux * (bj + (long long)F.uy * bk);
  const bool in_b = i >= F.q.i_lo && i <= F.q.i_hi && j >= F.q.j_lo && j <= F.q.j_hi && k >= F.q.k_lo &&
                    k <= F.q.k_hi;
  if (in_b && psr_inside(F.q, F.p, i, j, k)) {
    BoxAcc<R> a;
    a.base = F.s1;
    a.n = n;
    a.s = o;
    a.dj = F.ux;
    a.dk = (long long)F.ux * F.uy;
    R v[6];
    psr_cell(F.q, F.p, a, i, j, k, v);
#pragma unroll
    for (int c = 0; c < 6; ++c) F.s2[c * n + o] = v[c];
  } else {
#pragma unroll
    for (int c = 0; c < 6; ++c) F.s2[c * n + o] = F.s1[c * n + o];
  }
}

// (bi, bj, bk): U coordinates less one (the cells of B+1 start at U + 1).
template <typename R, int C>
__device__ __forceinline__ void fix_clean_cell(const FixParams<R>& F, int bi, int bj, int bk) {
  constexpr bool FD = FFE_FAST && sizeof(R) == 4;
  constexpr bool DF = C == 2;  // FP32CD: double-float denominators
  ++bi;
  ++bj;
  ++bk;
  if (bi >= F.ux - 1 || bj >= F.uy - 1 || bk >= F.uz - 1) return;
  const int i = F.ui + bi, j = F.uj + bj, k = F.uk + bk;
  const Geom& g = F.g;
  if (i < 0 || i >= g.sx || j < 0 || j >= g.sy || k < 0 || k >= g.sz) return;
  if (!fix_near(F, i, j, k, FixMargin::clean)) return;
  const long long n = (long long)F.ux * F.uy * F.uz;
  const long long o = bi + (long long)F.ux * (bj + (long long)F.uy * bk);
  BoxAcc<R> a;
  a.base = F.s2;
  a.n = n;
  a.s = o;
  a.dj = F.ux;
  a.dk = (long long)F.ux * F.uy;
  R e[3];
  if constexpr (FD) clean_cell_fast<false, BoxAcc<R>, DF>(a, e, F.ct);
  else clean_cell<R, C, BoxAcc<R>, false>(a, e, F.ct);
  const long long s = g.idx(i, j, k);
  F.out[0][s] = e[0];
  F.out[1][s] = e[1];
  F.out[2][s] = e[2];
  F.out[3][s] = a(BX, 0, 0, 0);
  F.out[4][s] = a(BY, 0, 0, 0);
  F.out[5][s] = a(BZ, 0, 0, 0);
}

#if !defined(FFE_BATCH_TY)
// One grid: block (x, y) covers 32 x 8 cells of a U plane, blockIdx.z the plane.
template <typename R, int C, bool B0, bool ABS, bool STAGE1>
__global__ void k_fix_update(const FixParams<R> F) {
  fix_update_cell<R, C, B0, ABS, STAGE1>(F, blockIdx.x * blockDim.x + threadIdx.x,
                                         blockIdx.y * blockDim.y + threadIdx.y, blockIdx.z);
}
template <typename R>
__global__ void k_fix_bc(const FixParams<R> F) {
  fix_bc_cell<R>(F, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y, blockIdx.z);
}
template <typename R, int C>
__global__ void k_fix_clean(const FixParams<R> F) {
  fix_clean_cell<R, C>(F, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y,
                       blockIdx.z);
}
#elif FFE_BATCH_TY == 8
// Many grids: block b takes item b = (grid, 32-wide x block, 8-high y block,
// plane) of that grid's U box; a 32 x 8 thread block.
template <typename R, int C, bool STAGE1>
__global__ void k_fix_update_batch(const FixItem* __restrict__ items, const FixParams<R>* __restrict__ fp) {
  const FixItem it = items[blockIdx.x];
  const FixParams<R>& F = fp[it.box];
  const int bi = it.bx * 32 + threadIdx.x, bj = it.by * 8 + threadIdx.y;
  if (F.has_b0) {
    if (F.absorb) fix_update_cell<R, C, true, true, STAGE1>(F, bi, bj, it.bz);
    else fix_update_cell<R, C, true, false, STAGE1>(F, bi, bj, it.bz);
  } else {
    if (F.absorb) fix_update_cell<R, C, false, true, STAGE1>(F, bi, bj, it.bz);
    else fix_update_cell<R, C, false, false, STAGE1>(F, bi, bj, it.bz);
  }
}
template <typename R>
__global__ void k_fix_bc_batch(const FixItem* __restrict__ items, const FixParams<R>* __restrict__ fp) {
  const FixItem it = items[blockIdx.x];
  fix_bc_cell<R>(fp[it.box], it.bx * 32 + threadIdx.x, it.by * 8 + threadIdx.y, it.bz);
}
template <typename R, int C>
__global__ void k_fix_clean_batch(const FixItem* __restrict__ items, const FixParams<R>* __restrict__ fp) {
  const FixItem it = items[blockIdx.x];
  fix_clean_cell<R, C>(fp[it.box], it.bx * 32 + threadIdx.x, it.by * 8 + threadIdx.y, it.bz);
}

// user_uniform ghost planes of many grids: item = (grid, x block, y block,
// plane k); the grid's output set, geometry and this step's constants come
// from its stage-launch entry.
template <typename R>
__global__ void k_uniform_ghosts_batch(const FixItem* __restrict__ items, const __grid_constant__ BoxTable<R> T) {
  const FixItem it = items[blockIdx.x];
  const Params<R>& P = T.b[it.box].P;
  const int i = it.bx * 32 + (int)threadIdx.x - NG, j = it.by * 8 + (int)threadIdx.y - NG;
  if (i >= P.g.sx + NG || j >= P.g.sy + NG) return;
  const long long s = P.g.idx(i, j, it.bz);
  uniform_bc_apply(P.ub, P.p, i, j, it.bz, P.out0[s], P.out0[s + P.fs], P.out0[s + 5 * P.fs]);
}
#endif

}  // namespace FFE_FUSED_NS

#if !defined(FFE_BATCH_TY)
#ifdef FFE_FUSED_EXACT
#define FFE_LAUNCH_NAME launch_fused_stage_exact
#else
#define FFE_LAUNCH_NAME launch_fused_stage
#endif

template <typename R, int C>
int FFE_LAUNCH_NAME(const Geom& g, const Phys& p, const Absorb<R>& ab, R cc, R c1, R c2, R c3, bool incr, int stage,
                    const void* maps_in, const void* maps_en, const void* maps_plain, const void* maps_plain_en,
                    const CEB<R>& in_g, const CEB<R>& en_g, const CEB<R>& b0, bool has_b0, const EB<R>& out, R ct,
                    const UniformBC<R>* ub, int* err, cudaStream_t st) {
  using namespace FFE_FUSED_NS;
  const bool abs = p.bnd[0] == 2;
  // the plain FP32 variant takes the taller tile and its own stage-input maps
  const bool plain = sizeof(R) == 4 && !has_b0 && !abs;
  if (plain && (!maps_plain || !maps_plain_en)) return -4;
  Maps M;
  memcpy(M.in, plain ? maps_plain : maps_in, sizeof(M.in));
  memcpy(M.en, plain ? maps_plain_en : maps_en, sizeof(M.en));
  Params<R> P;
  P.g = g;
  P.p = p;
  P.ab = ab;
  P.cc = cc;
  P.c1 = c1;
  P.c2 = c2;
  P.c3 = c3;
  P.ct = ct;
  P.incr = incr ? 1 : 0;
  for (int c = 0; c < 3; ++c) P.b0[c] = b0.c[c];
  // the kernel addresses component c as base + c * fs
  P.in0 = in_g.c[0];
  P.en0 = en_g.c[0];
  P.out0 = out.c[0];
  P.fs = out.c[1] - out.c[0];
  for (int c = 0; c < 6; ++c)
    if (in_g.c[c] != P.in0 + c * P.fs || en_g.c[c] != P.en0 + c * P.fs || out.c[c] != P.out0 + c * P.fs) return -4;
  P.err = err;
  P.ubc = ub ? 1 : 0;
  if (ub) P.ub = *ub;
  constexpr int TYP = sizeof(R) == 4 ? PLAIN_TY : FUSED_TY;
  const int TYL = plain ? TYP : FUSED_TY;
  const int tiles_x = (g.sx + TX - 1) / TX, tiles_y = (g.sy + TYL - 1) / TYL;
  const int kz = fused_planes_per_block(g, TYL);
  P.kz = kz;
  const dim3 grid(tiles_x, tiles_y, (g.sz + kz - 1) / kz);
  const bool s1 = stage == 1;
  // the fully periodic form of the plain FP32 variant (fast path only)
  constexpr bool PER_OK = sizeof(R) == 4 && !FFE_FUSED_EXACT_BUILD;
  const bool per3 = PER_OK && p.bnd[0] == 1 && p.bnd[1] == 1 && p.bnd[2] == 1 && !ub;
#define FFE_GO(B0V, ABSV, S1V, PERV)                                                             \
  do {                                                                                           \
    constexpr int TY = (!B0V && !ABSV) ? TYP : FUSED_TY;                                         \
    auto kf = k_fused<R, C, B0V, ABSV, S1V, TY, PERV>;                                           \
    const size_t smem = Body<R, C, B0V, ABSV, TY>::SMEM;                                         \
    static bool attr_set = false;                                                                \
    if (!attr_set) {                                                                             \
      if (cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=    \
              cudaSuccess ||                                                                     \
          cudaFuncSetAttribute(kf, cudaFuncAttributePreferredSharedMemoryCarveout,               \
                               (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)              \
        return -3;                                                                               \
      attr_set = true;                                                                           \
    }                                                                                            \
    kf<<<grid, Body<R, C, B0V, ABSV, TY>::NT, smem, st>>>(M, P);                                 \
  } while (0)
  if (has_b0) {
    if (abs) { if (s1) FFE_GO(true, true, true, false); else FFE_GO(true, true, false, false); }
    else { if (s1) FFE_GO(true, false, true, false); else FFE_GO(true, false, false, false); }
  } else {
    if (abs) { if (s1) FFE_GO(false, true, true, false); else FFE_GO(false, true, false, false); }
    else if (per3) { if (s1) FFE_GO(false, false, true, PER_OK); else FFE_GO(false, false, false, PER_OK); }
    else { if (s1) FFE_GO(false, false, true, false); else FFE_GO(false, false, false, false); }
  }
#undef FFE_GO
  return 0;
}

#ifdef FFE_FUSED_EXACT
#define FFE_FIX_NAME launch_psr_fixup_exact
#else
#define FFE_FIX_NAME launch_psr_fixup
#endif

template <typename R, int C>
int FFE_FIX_NAME(const Geom& g, const Phys& p, const Absorb<R>& ab, const PsrBC<R>& q, R cc, R c1, R c2, R c3,
                 bool incr, int stage, const CEB<R>& in, const CEB<R>& en, const CEB<R>& b0, bool has_b0,
                 const EB<R>& out, R ct, R* s1, R* s2, cudaStream_t st) {
  using namespace FFE_FUSED_NS;
  if (q.bx <= 0 || q.by <= 0 || q.bz <= 0) return 0;
  FixParams<R> F;
  F.g = g;
  F.p = p;
  F.ab = ab;
  F.q = q;
  F.cc = cc;
  F.c1 = c1;
  F.c2 = c2;
  F.c3 = c3;
  F.ct = ct;
  F.incr = incr ? 1 : 0;
  int u[6];
  psr_fix_box(g, q.i_lo, q.i_hi, q.j_lo, q.j_hi, q.k_lo, q.k_hi, u);
  F.ui = u[0]; F.uj = u[1]; F.uk = u[2]; F.ux = u[3]; F.uy = u[4]; F.uz = u[5];
  for (int c = 0; c < 6; ++c) {
    F.in[c] = in.c[c];
    F.en[c] = en.c[c];
    F.out[c] = out.c[c];
  }
  for (int c = 0; c < 3; ++c) F.b0[c] = b0.c[c];
  F.s1 = s1;
  F.s2 = s2;
  F.has_b0 = has_b0 ? 1 : 0;
  F.absorb = p.bnd[0] == 2 ? 1 : 0;
  const dim3 b(32, 8, 1), gr((F.ux + 31) / 32, (F.uy + 7) / 8, F.uz);
  const bool abs = p.bnd[0] == 2, s1st = stage == 1;
#define FFE_FIXGO(B0V, ABSV, S1V) k_fix_update<R, C, B0V, ABSV, S1V><<<gr, b, 0, st>>>(F)
  if (has_b0) {
    if (abs) { if (s1st) FFE_FIXGO(true, true, true); else FFE_FIXGO(true, true, false); }
    else { if (s1st) FFE_FIXGO(true, false, true); else FFE_FIXGO(true, false, false); }
  } else {
    if (abs) { if (s1st) FFE_FIXGO(false, true, true); else FFE_FIXGO(false, true, false); }
    else { if (s1st) FFE_FIXGO(false, false, true); else FFE_FIXGO(false, false, false); }
  }
#undef FFE_FIXGO
  k_fix_bc<R><<<gr, b, 0, st>>>(F);
  k_fix_clean<R, C><<<gr, b, 0, st>>>(F);
  return 0;
}

#ifndef FFE_FUSED_EXACT
void fused_tile_shape(int* tx, int* ty) {
  *tx = fused_fast::TX;
  *ty = 8;
}

// z-planes per block: enough blocks for ~16 per SM on 152 SMs, at least 8
// planes per block, at most 64.
int fused_planes_per_block(const Geom& g, int ty) {
  const int tiles_x = (g.sx + FUSED_TX - 1) / FUSED_TX, tiles_y = (g.sy + ty - 1) / ty;
  const long long want = 152LL * 16;
  const int kz = (int)std::max(8LL, std::min<long long>(96, ((long long)g.sz * tiles_x * tiles_y + want - 1) / want));
  return std::min(kz, g.sz);
}

// Tensor maps of one array for the fused kernels of tile height ty: the OLD
// box (tile + 2 halo) and the EN box (tile + 1 halo rows; skipped when map_en
// is null).  Coordinates: (i + 2, j + 2, k + 2).
int make_stage_maps(void* map_old, void* map_en, void* base, const Geom& g, int es, int ty) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return -1;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  using namespace fused_fast;
  const cuuint64_t dims[3] = {(cuuint64_t)g.px, (cuuint64_t)g.py, (cuuint64_t)(g.sz + 2 * NG)};
  const cuuint64_t strides[2] = {(cuuint64_t)g.px * es, (cuuint64_t)g.plane * es};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  const cuuint32_t box_old[3] = {(cuuint32_t)OW, (cuuint32_t)(ty + 4), 1};
  const cuuint32_t box_en[3] = {(cuuint32_t)OW, (cuuint32_t)(ty + 2), 1};
  CUresult r = encode((CUtensorMap*)map_old, dt, 3, base, dims, strides, box_old, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return -2;
  if (!map_en) return 0;
  r = encode((CUtensorMap*)map_en, dt, 3, base, dims, strides, box_en, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}
#endif

#define FFE_INST_F(R, C)                                                                                        \
  template int FFE_LAUNCH_NAME<R, C>(const Geom&, const Phys&, const Absorb<R>&, R, R, R, R, bool, int,        \
                                     const void*, const void*, const void*, const void*, const CEB<R>&,         \
                                     const CEB<R>&, const CEB<R>&, bool, const EB<R>&, R, const UniformBC<R>*,  \
                                     int*, cudaStream_t);
#define FFE_INST_X(R, C)                                                                                        \
  template int FFE_FIX_NAME<R, C>(const Geom&, const Phys&, const Absorb<R>&, const PsrBC<R>&, R, R, R, R, bool, \
                                  int, const CEB<R>&, const CEB<R>&, const CEB<R>&, bool, const EB<R>&, R, R*,   \
                                  R*, cudaStream_t);
FFE_INST_F(float, 0)
FFE_INST_F(float, 1)
FFE_INST_F(float, 2)
FFE_INST_F(double, 0)
FFE_INST_X(float, 0)
FFE_INST_X(float, 1)
FFE_INST_X(float, 2)
FFE_INST_X(double, 0)

#elif defined(FFE_BATCH_SPEC)  // batched launches of one variant, tile height 8

// One stage of many grids of variant var (0: plain, 1: absorbing layer, 2:
// B0, 3: B0 and absorbing layer); -1 for any other var.  The shared-memory limit must
// have been raised by fused_batch_prepare_spec_t8.
template <typename R, int C>
int launch_fused_batch_spec_t8(bool stage1, int var, const BatchItem* items, int nitems, const BoxTable<R>& T,
                               int grid, cudaStream_t st) {
  using namespace FFE_FUSED_NS;
  constexpr int TY = FFE_BATCH_TY;
  if (nitems <= 0) return 0;
  if (var == 0) {
    constexpr int NT = Body<R, C, false, false, TY>::NT;
    const size_t smem = Body<R, C, false, false, TY>::SMEM;
    if (stage1) k_fused_batch_var<R, C, true, TY, 0><<<grid, NT, smem, st>>>(items, nitems, T);
    else k_fused_batch_var<R, C, false, TY, 0><<<grid, NT, smem, st>>>(items, nitems, T);
  } else if (var == 1) {
    constexpr int NT = Body<R, C, false, true, TY>::NT;
    const size_t smem = Body<R, C, false, true, TY>::SMEM;
    if (stage1) k_fused_batch_var<R, C, true, TY, 1><<<grid, NT, smem, st>>>(items, nitems, T);
    else k_fused_batch_var<R, C, false, TY, 1><<<grid, NT, smem, st>>>(items, nitems, T);
  } else if (var == 2) {
    constexpr int NT = Body<R, C, true, false, TY>::NT;
    const size_t smem = Body<R, C, true, false, TY>::SMEM;
    if (stage1) k_fused_batch_var<R, C, true, TY, 2><<<grid, NT, smem, st>>>(items, nitems, T);
    else k_fused_batch_var<R, C, false, TY, 2><<<grid, NT, smem, st>>>(items, nitems, T);
  } else if (var == 3) {
    constexpr int NT = Body<R, C, true, true, TY>::NT;
    const size_t smem = Body<R, C, true, true, TY>::SMEM;
    if (stage1) k_fused_batch_var<R, C, true, TY, 3><<<grid, NT, smem, st>>>(items, nitems, T);
    else k_fused_batch_var<R, C, false, TY, 3><<<grid, NT, smem, st>>>(items, nitems, T);
  } else {
    return -1;
  }
  return 0;
}

// Raise the shared-memory limit of the two stage kernels of variant var;
// returns their resident blocks per SM, or 0 on failure.
template <typename R, int C>
int fused_batch_prepare_spec_t8(int var) {
  using namespace FFE_FUSED_NS;
  constexpr int TY = FFE_BATCH_TY;
  // per variant: the lean or the standard body (Body)
  const int NT = var == 0   ? Body<R, C, false, false, TY>::NT
                 : var == 1 ? Body<R, C, false, true, TY>::NT
                 : var == 2 ? Body<R, C, true, false, TY>::NT
                            : Body<R, C, true, true, TY>::NT;
  const size_t smem = var == 0   ? Body<R, C, false, false, TY>::SMEM
                      : var == 1 ? Body<R, C, false, true, TY>::SMEM
                      : var == 2 ? Body<R, C, true, false, TY>::SMEM
                                 : Body<R, C, true, true, TY>::SMEM;
  void (*k1)(const BatchItem*, int, const BoxTable<R>) = nullptr;
  void (*k2)(const BatchItem*, int, const BoxTable<R>) = nullptr;
  if (var == 0) {
    k1 = k_fused_batch_var<R, C, true, TY, 0>;
    k2 = k_fused_batch_var<R, C, false, TY, 0>;
  } else if (var == 1) {
    k1 = k_fused_batch_var<R, C, true, TY, 1>;
    k2 = k_fused_batch_var<R, C, false, TY, 1>;
  } else if (var == 2) {
    k1 = k_fused_batch_var<R, C, true, TY, 2>;
    k2 = k_fused_batch_var<R, C, false, TY, 2>;
  } else if (var == 3) {
    k1 = k_fused_batch_var<R, C, true, TY, 3>;
    k2 = k_fused_batch_var<R, C, false, TY, 3>;
  } else {
    return 0;
  }
  int n[2] = {0, 0};
  for (int i = 0; i < 2; ++i) {
    const void* k = (const void*)(i ? k2 : k1);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n[i], k, NT, smem) != cudaSuccess)
      return 0;
  }
  return n[0] < n[1] ? n[0] : n[1];
}

#define FFE_INST_S(R, C)                                                                                        \
  template int launch_fused_batch_spec_t8<R, C>(bool, int, const BatchItem*, int, const BoxTable<R>&, int,     \
                                                cudaStream_t);                                                  \
  template int fused_batch_prepare_spec_t8<R, C>(int);
FFE_INST_S(float, 0)
FFE_INST_S(float, 1)
FFE_INST_S(double, 0)

#else  // FFE_BATCH_TY: batched launches for tile height FFE_BATCH_TY

#define FFE_BATCH_LAUNCH FFE_CAT(launch_fused_batch_t, FFE_BATCH_TY)
#define FFE_BATCH_PREP FFE_CAT(fused_batch_prepare_t, FFE_BATCH_TY)

// One stage of many grids: `grid` blocks over nitems work items.  The
// shared-memory limit must have been raised by FFE_BATCH_PREP (this launch
// may be captured into a graph, where that call does not belong).
template <typename R, int C>
int FFE_BATCH_LAUNCH(bool stage1, const BatchItem* items, int nitems, const BoxTable<R>& T, int grid,
                     cudaStream_t st) {
  using namespace FFE_FUSED_NS;
  constexpr int TY = FFE_BATCH_TY;
  const size_t smem = Sizes<R, TY>::BYTES;
  if (nitems <= 0) return 0;
  if (stage1) k_fused_batch<R, C, true, TY><<<grid, Tile<TY, BATCH_CPT>::NT, smem, st>>>(items, nitems, T);
  else k_fused_batch<R, C, false, TY><<<grid, Tile<TY, BATCH_CPT>::NT, smem, st>>>(items, nitems, T);
  return 0;
}

// Raise the shared-memory limit of both batched stage kernels; returns their
// resident blocks per SM, or 0 on failure.
template <typename R, int C>
int FFE_BATCH_PREP() {
  using namespace FFE_FUSED_NS;
  constexpr int TY = FFE_BATCH_TY;
  const size_t smem = Sizes<R, TY>::BYTES;
  auto k1 = k_fused_batch<R, C, true, TY>;
  auto k2 = k_fused_batch<R, C, false, TY>;
  if (cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
  if (cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
  int n1 = 0, n2 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n1, k1, Tile<TY, BATCH_CPT>::NT, smem) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k2, Tile<TY, BATCH_CPT>::NT, smem) != cudaSuccess) return 0;
  return n1 < n2 ? n1 : n2;
}

#define FFE_INST_B(R, C)                                                                                 \
  template int FFE_BATCH_LAUNCH<R, C>(bool, const BatchItem*, int, const BoxTable<R>&, int, cudaStream_t); \
  template int FFE_BATCH_PREP<R, C>();
FFE_INST_B(float, 0)
FFE_INST_B(float, 1)
#if FFE_BATCH_TY == 8
FFE_INST_B(double, 0)

// Pulsar fix-up of many grids: the three steps, each one launch over all items.
template <typename R, int C>
int launch_fix_batch(bool stage1, const FixItem* items, int nitems, const FixParams<R>* fp, cudaStream_t st) {
  using namespace FFE_FUSED_NS;
  if (nitems <= 0) return 0;
  const dim3 b(32, 8, 1);
  if (stage1) k_fix_update_batch<R, C, true><<<nitems, b, 0, st>>>(items, fp);
  else k_fix_update_batch<R, C, false><<<nitems, b, 0, st>>>(items, fp);
  k_fix_bc_batch<R><<<nitems, b, 0, st>>>(items, fp);
  k_fix_clean_batch<R, C><<<nitems, b, 0, st>>>(items, fp);
  return 0;
}

template <typename R>
int launch_uniform_ghosts_batch(const FixItem* items, int nitems, const BoxTable<R>& T, cudaStream_t st) {
  using namespace FFE_FUSED_NS;
  if (nitems <= 0) return 0;
  k_uniform_ghosts_batch<R><<<nitems, dim3(32, 8, 1), 0, st>>>(items, T);
  return 0;
}

template int launch_fix_batch<float, 0>(bool, const FixItem*, int, const FixParams<float>*, cudaStream_t);
template int launch_fix_batch<float, 1>(bool, const FixItem*, int, const FixParams<float>*, cudaStream_t);
template int launch_fix_batch<double, 0>(bool, const FixItem*, int, const FixParams<double>*, cudaStream_t);
template int launch_uniform_ghosts_batch<float>(const FixItem*, int, const BoxTable<float>&, cudaStream_t);
template int launch_uniform_ghosts_batch<double>(const FixItem*, int, const BoxTable<double>&, cudaStream_t);
#endif
#endif  // FFE_BATCH_TY

}  // namespace ffe
