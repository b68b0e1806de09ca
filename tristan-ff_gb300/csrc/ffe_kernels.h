// ffe_kernels.h — host-side launchers of the device kernels (internal).
#pragma once
#include <algorithm>
#include <cuda_runtime.h>
#include "ffe_common.cuh"
#include "ffe_fused_types.cuh"

namespace ffe {

// ---- staged kernels (ffe_staged.cu), one per reference procedure -----------
template <typename R>
void launch_rho(const Geom& g, const R* ex, const R* ey, const R* ez, R* rho, cudaStream_t st);
template <typename R, int C>
void launch_push(const Geom& g, R cc, const CEB<R>& eb, const CEB<R>& b0, bool has_b0, const R* rho, const EB<R>& d,
                 cudaStream_t st);
template <typename R, int C>
void launch_update(const Geom& g, const Phys& p, const Absorb<R>& ab, R c1, R c2, R c3, bool incr, const EB<R>& f,
                   const CEB<R>& fn, const CEB<R>& df, cudaStream_t st);
template <typename R, int C>
void launch_clean(const Geom& g, const EB<R>& eb, const EB<R>& d, R ct, cudaStream_t st);
template <typename R>
void launch_fill(const Geom& g, const Phys& p, const EB<R>& f, R* const b0[3], bool with_b0, cudaStream_t st,
                 bool x_done = false);
template <typename R>
void launch_psr_bc(const Geom& g, const Phys& p, const PsrBC<R>& q, const EB<R>& f, R* box, cudaStream_t st);
template <typename R>
void launch_uniform_bc(const Geom& g, const Phys& p, const UniformBC<R>& u, const EB<R>& f, bool ghosts_only,
                       cudaStream_t st);
template <typename R>
void launch_loop_bc(const Geom& g, const Phys& p, const EB<R>& f, cudaStream_t st);
template <typename R>
void launch_psr_init(const Geom& g, const Phys& p, const PsrBC<R>& q, const EB<R>& f, cudaStream_t st);
template <typename R>
void launch_uniform_init(const Geom& g, const Phys& p, const UniformBC<R>& u, R* bz, R* b0z, cudaStream_t st);
template <typename R>
void launch_loop_init(const Geom& g, const Phys& p, const double prm[8], const EB<R>& f, const EB<R>& f0,
                      cudaStream_t st);
// synthetic plane-wave workloads: 11 doubles per mode, see ffe_staged.cu
size_t waves_param_bytes();
template <typename R>
int launch_waves(const Geom& g, const Phys& p, const double bg[3], int n, const double* modes, void* dparam,
                 const EB<R>& f, cudaStream_t st);
// Copy one array between the reference's contiguous layout and the padded one.
template <typename R>
void launch_repack(const Geom& g, const R* src, R* dst, bool to_padded, cudaStream_t st);
template <typename R>
void launch_finite(const Geom& g, const CEB<R>& f, int* bad, cudaStream_t st);

// ---- fused stage kernels (ffe_fused.cu) -------------------------------------
// One launch advances one SSP-RK3 stage AND applies the E-parallel cleaning
// of that stage: reads the stage input E,B (set `in`) and, for stages 2-3,
// the step-start fields (set `en`); writes cleaned E and updated B to `out`.
// maps_in / maps_en: 6 CUtensorMaps each (ex..bz of the input set and of the
// step-start set) made by make_stage_maps; err: device word set on a timeout.
// Returns 0, or -3 if the kernel attribute could not be set.
// ct: TINY added to the cleaning denominators (FFE_FLAG_CLEAN_TINY) or 0.
// ub: the user_uniform BC constants of this step, applied inline (or null).
// in_g / en_g: the same two sets as plain pointers (for halo cells computed at
// their periodic image next to an open face).
// maps_plain / maps_plain_en: the stage-input and step-start maps made for
// tile height PLAIN_TY, used by the plain FP32 variant (no B0, no absorbing
// layer); null for FP64 handles.
template <typename R, int C>
int launch_fused_stage(const Geom& g, const Phys& p, const Absorb<R>& ab, R cc, R c1, R c2, R c3, bool incr,
                       int stage, const void* maps_in, const void* maps_en, const void* maps_plain,
                       const void* maps_plain_en, const CEB<R>& in_g, const CEB<R>& en_g, const CEB<R>& b0,
                       bool has_b0, const EB<R>& out, R ct, const UniformBC<R>* ub, int* err, cudaStream_t st);
template <typename R, int C>
int launch_fused_stage_exact(const Geom& g, const Phys& p, const Absorb<R>& ab, R cc, R c1, R c2, R c3, bool incr,
                             int stage, const void* maps_in, const void* maps_en, const void* maps_plain,
                             const void* maps_plain_en, const CEB<R>& in_g, const CEB<R>& en_g, const CEB<R>& b0,
                             bool has_b0, const EB<R>& out, R ct, const UniformBC<R>* ub, int* err,
                             cudaStream_t st);
// Pulsar BC on the fused path: after a fused stage, redo the cells of the BC's
// bounding box dilated by one (update on box+2 into s1, BC into s2, clean into
// out).  s1, s2: 6 * (bx+4)(by+4)(bz+4) elements each.
template <typename R, int C>
int launch_psr_fixup(const Geom& g, const Phys& p, const Absorb<R>& ab, const PsrBC<R>& q, R cc, R c1, R c2, R c3,
                     bool incr, int stage, const CEB<R>& in, const CEB<R>& en, const CEB<R>& b0, bool has_b0,
                     const EB<R>& out, R ct, R* s1, R* s2, cudaStream_t st);
template <typename R, int C>
int launch_psr_fixup_exact(const Geom& g, const Phys& p, const Absorb<R>& ab, const PsrBC<R>& q, R cc, R c1, R c2,
                           R c3, bool incr, int stage, const CEB<R>& in, const CEB<R>& en, const CEB<R>& b0,
                           bool has_b0, const EB<R>& out, R ct, R* s1, R* s2, cudaStream_t st);
// The two TMA tensor maps (OLD box, EN box) of one field array at `base`, for
// the fused kernels of tile height ty (8 or 16).
int make_stage_maps(void* map_old, void* map_en, void* base, const Geom& g, int es, int ty);
// Tile shape the single-grid fused kernel uses (for reporting).
void fused_tile_shape(int* tx, int* ty);
// Default z-planes per block of the fused kernel for a grid and tile height.
int fused_planes_per_block(const Geom& g, int ty);

// ---- batched launches (ffe_fused.cu with FFE_BATCH_TY = 8 / 16) ------------
// One SSP-RK3 stage of up to BATCH_MAX grids in one launch: `grid` blocks
// take the nitems work items (device memory; grid < nitems: persistent
// blocks).  T: one entry per grid, passed as the kernel's parameter.  (R, C)
// in {(float,0), (float,1), (double,0)}; double only with tile height 8.
template <typename R, int C>
int launch_fused_batch_t8(bool stage1, const BatchItem* items, int nitems, const BoxTable<R>& T, int grid,
                          cudaStream_t st);
template <typename R, int C>
int launch_fused_batch_t16(bool stage1, const BatchItem* items, int nitems, const BoxTable<R>& T, int grid,
                           cudaStream_t st);
// Raise the shared-memory limit of the batched stage kernels (call before any
// launch or capture); returns their resident blocks per SM (0 on failure).
template <typename R, int C> int fused_batch_prepare_t8();
template <typename R, int C> int fused_batch_prepare_t16();
// Tile height 8, all grids of the launch of one B0 / absorbing-layer variant
// var (bit 1: B0, bit 0: absorbing layer), 0 <= var < 4 (launch returns -1,
// prepare 0, for any other var).
template <typename R, int C>
int launch_fused_batch_spec_t8(bool stage1, int var, const BatchItem* items, int nitems, const BoxTable<R>& T,
                               int grid, cudaStream_t st);
template <typename R, int C> int fused_batch_prepare_spec_t8(int var);
// Pulsar fix-up (update, BC, clean) of many grids; items over each grid's U box.
template <typename R, int C>
int launch_fix_batch(bool stage1, const FixItem* items, int nitems, const FixParams<R>* fp, cudaStream_t st);
// user_uniform ghost planes of many grids (items: grid, x block, y block, plane).
template <typename R>
int launch_uniform_ghosts_batch(const FixItem* items, int nitems, const BoxTable<R>& T, cudaStream_t st);

// ---- node output (ffe_output.cu) ------------------------------------------
// Output nodes of a meshblock: i = i0 + i1 * istep for i1 < nx (same in y, z).
struct NodeGrid {
  int istep, i0, j0, k0, nx, ny, nz;
};
NodeGrid node_grid(const Geom& g, const Phys& p, int istep);
// The twelve datasets of writeOutput at the nodes of n into out (device,
// 12 * nx * ny * nz values, dataset-major, x fastest).
template <typename R>
void launch_node_output(const Geom& g, const Phys& p, const NodeGrid& n, bool var2_uniform, const CEB<R>& f, R* out,
                        cudaStream_t st);

// Record a failure without a handle (read back by ffe_last_error(NULL, ...)).
int set_thread_error(int status, const char* msg);

}  // namespace ffe
