/*
 * ffe.h — C ABI of the GB300 force-free field solver (libffe_gb300.so).
 *
 * The reference (tristan-ff, Fortran 2008) exposes its field update as
 * argument-less module procedures acting on module-global arrays.  Each entry
 * point below replaces one of those procedures for ONE meshblock that lives
 * on ONE GPU; the fields stay resident in device memory between calls.
 *
 *   reference procedure                               replaced by
 *   -----------------------------------------------   ------------------------
 *   m_initialize::initializeFields   (src/logistics/initialize.F90:201-229)   ffe_create
 *   m_finalize (deallocation)        (src/logistics/finalize.F90:14-71)        ffe_destroy
 *   m_fldsolver::initRKstep          (src/algorithms/field_solver.F90:15-33)   ffe_init_rk_step
 *   m_fldsolver::rk3Step             (src/algorithms/field_solver.F90:35-42)   ffe_rk3_stage
 *   m_fldsolver::computeRho          (src/algorithms/field_solver.F90:44-63)   ffe_compute_rho
 *   m_fldsolver::rk3Push             (src/algorithms/field_solver.F90:65-166)  ffe_rk3_push
 *   m_fldsolver::rk3Update           (src/algorithms/field_solver.F90:168-271) ffe_rk3_update
 *   m_fldsolver::cleanEpar           (src/algorithms/field_solver.F90:273-335) ffe_clean_epar
 *   m_exchangefields::exchangeFields (src/logistics/exchange_fields.F90:11-197) ffe_exchange_fields
 *   m_userfile::userInitialize       (user/user_psr.F90:20-69,
 *                                     user/user_uniform.F90:20-69,
 *                                     user/user_loop.F90:20-93)               ffe_user_initialize
 *   m_userfile::userFieldBoundaryConditions
 *                                    (user/user_psr.F90:72-332,
 *                                     user/user_uniform.F90:77-147,
 *                                     user/user_loop.F90:101-164)             ffe_user_bc
 *   m_mainloop::mainloop prologue    (src/tristanmainloop.F90:41-42)           ffe_mainloop_prologue
 *   m_mainloop::mainloop step body   (src/tristanmainloop.F90:50-84)           ffe_step
 *   m_writeoutput::writeOutput field datasets
 *                                    (src/io/write_output.F90:270-413)         ffe_output
 *
 * Array contract.  Host arrays passed to ffe_upload / ffe_download have the
 * reference's allocation shape (src/logistics/initialize.F90:192-199):
 * (sx+4) x (sy+4) x (sz+4) values, index range -2..s+1 per axis (NGHOST = 2,
 * src/CMakeLists.txt:18), column-major with x fastest, element type double
 * for FFE_FP64 and float otherwise.  A Fortran caller passes c_loc(ex).
 *
 * Errors.  Every function returns FFE_OK (0) or a negative ffe_status.  The
 * message of the last failure is kept per handle (ffe_last_error) and, for
 * failures without a handle, per host thread (ffe_last_error(NULL, ...)).
 * The reference has no error returns: its fatal paths print and stop
 * (src/tools/error_handling.F90:8-13).
 *
 * Threads and streams.  A handle is used by one host thread at a time; all
 * of its device work is ordered on the stream given at creation (NULL = a
 * stream the library creates).  Distinct handles may run concurrently.
 */
#ifndef FFE_GB300_H
#define FFE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFE_NGHOST 2
#define FFE_ABI_VERSION 1

typedef struct ffe_solver* ffe_t;

typedef enum {
  FFE_OK = 0,
  FFE_EINVAL = -1,      /* bad argument or descriptor                        */
  FFE_ENOMEM = -2,      /* device or host allocation failed                  */
  FFE_ECUDA = -3,       /* a CUDA runtime call failed                        */
  FFE_ESTATE = -4,      /* call not valid in the handle's current state      */
  FFE_ENONFINITE = -5,  /* ffe_check_finite found NaN/Inf                    */
  FFE_ETIMEOUT = -6,    /* a bounded device wait gave up                     */
  FFE_EUNSUPPORTED = -7 /* combination of options not built                  */
} ffe_status;

typedef enum {
  FFE_FP64 = 0,  /* every real is double: what a -fdefault-real-8 build computes */
  FFE_FP32 = 1,  /* every real is float: the arithmetic of the shipped build      */
  FFE_FP32C = 2, /* float storage; increment-form (compensated) RK combination
                    En + (c2 (E - En) + c3 dE): no drift from 1/3 + 2/3 != 1 in float */
  FFE_FP32CD = 3 /* FFE_FP32C with the B^2 denominators of the current and of
                    the cleaning in double precision: FP64 on the exact path,
                    double-float (hi + lo float pairs, 48-bit significand) on
                    the fast path, where FP64 arithmetic is slow (GB300)     */
} ffe_precision;

typedef enum {
  FFE_BOUNDARY_OPEN = 0,     /* ghosts keep their values (no neighbour)   */
  FFE_BOUNDARY_PERIODIC = 1, /* ghosts wrap to the opposite interior      */
  FFE_BOUNDARY_ABSORB = 2    /* spherical absorbing shell, ghosts frozen  */
} ffe_boundary;

typedef enum {
  FFE_EX = 0, FFE_EY, FFE_EZ, FFE_BX, FFE_BY, FFE_BZ,
  FFE_B0X, FFE_B0Y, FFE_B0Z,
  /* the reference's work arrays, readable after the per-procedure calls
     (src/objects/fields.F90:17-24) */
  FFE_DEX, FFE_DEY, FFE_DEZ, FFE_DBX, FFE_DBY, FFE_DBZ,
  FFE_ENX, FFE_ENY, FFE_ENZ, FFE_BNX, FFE_BNY, FFE_BNZ,
  FFE_RHO,
  FFE_NFIELDS
} ffe_field;

typedef enum {
  FFE_SETUP_NONE = 0,    /* no user boundary condition                      */
  FFE_SETUP_PSR = 1,     /* user/user_psr.F90: rotating conducting sphere    */
  FFE_SETUP_UNIFORM = 2, /* user/user_uniform.F90: twisted flux tube         */
  FFE_SETUP_LOOP = 3     /* user/user_loop.F90: magnetic loop                */
} ffe_setup;

/* Index of each setup's parameters in ffe_grid_desc.params[]:
 *  PSR:     0 psr_radius, 1 psr_angle [deg], 2 psr_period [steps],
 *           3 field scale (1 = the shipped |mu| = R^3, user/user_psr.F90:365-367)
 *  UNIFORM: 0 L0, 1 r_L0, 2 t0, 3 beta_twist   (user/user_uniform.F90:29-38)
 *  LOOP:    0 L0, 1 a_L0, 2 h_L0, 3 r_L0, 4 t0, 5 beta_twist
 *                                              (user/user_loop.F90:29-41)   */
#define FFE_MAX_PARAMS 8

typedef enum {
  FFE_PATH_AUTO = 0,      /* fused kernels where the setup allows, else FFE_PATH_STAGED */
  FFE_PATH_STAGED = 1,    /* one kernel per reference procedure, reference order */
  FFE_PATH_FUSED = 2,     /* require the fused stage+clean kernels (error if not possible) */
  FFE_PATH_FUSED_EXACT = 3 /* the fused kernels built without multiply-add contraction:
                              same rounding as FFE_PATH_STAGED, for verification */
} ffe_path;

/* Opt-in deviation from the reference: clamp the absorbing-shell depth
   delta_r to 1.  The reference's factor (1 - delta_r^3) of
   src/algorithms/field_solver.F90:226-263 turns negative and exceeds 1 in
   magnitude where delta_r > 2^(1/3), which happens in the box corners (the
   shell is a sphere inscribed in the box), so fields there grow by up to
   ~100x per stage.  With the clamp the factor stays in [0, 1].            */
#define FFE_FLAG_ABSORB_CLAMP 1
/* Opt-in deviation: add TINY to the B^2 denominators of cleanEpar, as the
   reference does for the current (field_solver.F90:111) but not for the
   cleaning (:300,314,328), where B = 0 gives 0/0 = NaN.  An absorbing shell
   drives B to zero at the box corners, so a run with FFE_FLAG_ABSORB_CLAMP
   needs this flag to stay finite.                                          */
#define FFE_FLAG_CLEAN_TINY 2
/* Opt-in deviation: measure the absorbing shell's radius with the cell's own
   y coordinate.  The reference uses jg = i + y0 (field_solver.F90:211), so
   its shell is a function of (x, x, z): cells near the y faces are not damped
   unless x is far from the centre, and those faces act as open boundaries
   with frozen ghosts.  For the pulsar setup that makes the y faces
   numerically unstable: two FP64 builds that differ only in rounding drift
   apart by 10% (relative L2 of E) within 200 steps.                       */
#define FFE_FLAG_ABSORB_TRUE_Y 4
/* For failure-detection tests only (no counterpart in the reference): in
   every block of the fused stage kernels the thread that issues the TMA plane
   copies leaves out one plane's copy, and the blocks give up waiting for it
   after about 2^14 probes instead of 2^22.  The waits run out, the blocks set
   the error word and return, and the next ffe_synchronize (or
   ffe_batch_synchronize) returns FFE_ETIMEOUT; the CUDA context stays usable.
   Results of a handle with this flag are meaningless.                      */
#define FFE_FLAG_TEST_WITHHOLD_COPY 8

typedef struct {
  int32_t sx, sy, sz;          /* interior cells of this meshblock           */
  int32_t x0, y0, z0;          /* meshblock corner in the global mesh        */
  int32_t gsx, gsy, gsz;       /* global mesh size (mx0, my0, mz0)           */
  int32_t boundary[3];         /* ffe_boundary per axis; 2 on any axis => all */
  int32_t absorb_buff;         /* <grid> absorb_buff (default 20)            */
  int32_t precision;           /* ffe_precision                              */
  int32_t setup;               /* ffe_setup                                  */
  int32_t path;                /* ffe_path                                   */
  int32_t flags;               /* FFE_FLAG_* bits, 0 = the reference's behaviour */
  int32_t reserved;            /* must be 0                                  */
  double cc;                   /* <algorithm> c, the Courant number          */
  double params[FFE_MAX_PARAMS];
  void* stream;                /* cudaStream_t to order work on, or NULL     */
} ffe_grid_desc;

/* Fill *d with the reference's defaults: periodic, c = 0.45, absorb_buff 20
   (src/logistics/initialize.F90:139-148,185-190), the given interior size,
   a single meshblock covering the global mesh, FFE_FP32, FFE_PATH_AUTO.    */
int ffe_desc_default(ffe_grid_desc* d, int32_t sx, int32_t sy, int32_t sz);

/* Allocate device state for one meshblock (all fields zero).  The arena is
   allocated stream-ordered on the handle's stream. */
int ffe_create(ffe_t* out, const ffe_grid_desc* desc);
/* Device bytes ffe_create would allocate for this descriptor (no device call;
   no counterpart in the reference: admission control of a serving loop). */
int ffe_desc_device_bytes(const ffe_grid_desc* desc, size_t* bytes);
int ffe_destroy(ffe_t h);

/* Copy of the last error message; returns the status that produced it. */
int ffe_last_error(ffe_t h, char* buf, size_t len);

/* Number of elements of one ghosted host array: (sx+4)(sy+4)(sz+4). */
int ffe_field_elems(ffe_t h, size_t* nelems);
/* Device bytes the handle holds. */
int ffe_device_bytes(ffe_t h, size_t* bytes);

/* Host <-> device copies of one whole ghosted array (see array contract). */
int ffe_upload(ffe_t h, int32_t field, const void* host, size_t nelems);
int ffe_download(ffe_t h, int32_t field, void* host, size_t nelems);

/* Several whole arrays per call (same shape contract); the host copy of one
   array overlaps the on-device repacking of the previous one.  B0 arrays go
   through ffe_upload.  Both synchronise.  (No counterpart in the reference,
   whose fields live on the host.) */
int ffe_upload_many(ffe_t h, int32_t n, const int32_t* fields, const void* const* host, size_t nelems);
int ffe_download_many(ffe_t h, int32_t n, const int32_t* fields, void* const* host, size_t nelems);

/* --- per-procedure operator API (reference order, one launch each) ---- */
int ffe_init_rk_step(ffe_t h);
int ffe_compute_rho(ffe_t h);
int ffe_rk3_push(ffe_t h);
int ffe_rk3_update(ffe_t h, double c1, double c2, double c3);
int ffe_rk3_stage(ffe_t h, double c1, double c2, double c3);
int ffe_clean_epar(ffe_t h);
int ffe_exchange_fields(ffe_t h, int32_t exchange_b0);
int ffe_user_initialize(ffe_t h);
int ffe_user_bc(ffe_t h, int32_t step);

/* Synthetic plane-wave workload (no counterpart among the reference's user
   files; it builds the Alfven-packet and random-mode grids of the benchmark):
   B = bg + sum_m dB_m, E = sum_m -n_m x dB_m, dB_m(x) = -a_m sin(K_m.x + phi_m) u_m,
   evaluated in double at every staggered point (ghosts included), rounded once
   to the storage precision; B0 is set to zero.  modes holds 11 doubles per mode:
   K[3] (radians per cell), phi, a, u[3] (unit polarisation), n[3]; nmodes <= 64. */
int ffe_init_waves(ffe_t h, const double bg[3], int32_t nmodes, const double* modes);

/* cleanEpar on arrays the caller owns, with no device allocation by the
   library.  No counterpart in the reference: it is for callers that manage
   all of their device memory themselves (arrays reserved once to fill HBM, or
   a run loop where an allocation call, which may synchronise the device or
   fail on fragmented memory, is not acceptable).  ex..bz are device pointers
   to arrays in the reference's layout ((sx+4)(sy+4)(sz+4), x fastest, cell
   -2 first); E is cleaned in place.  The cleaning is the reference's, with
   no TINY in the B^2 denominators: it equals ffe_clean_epar on a handle
   created without FFE_FLAG_CLEAN_TINY.  The out-of-place scratch is a fixed
   24 MiB device array inside the library, so 3*sx*sy*sz values must fit
   (2,097,152 interior cells in FP32, 1,048,576 in FP64); larger sizes
   return FFE_EINVAL.  CUDA loads the library's modules lazily, so the
   scratch takes its 24 MiB of device memory when first needed on a device.
   A call with sx = sy = sz = 0 and every pointer NULL does only that set-up
   on the current device (loads the scratch and the kernels, looks up the
   scratch's device address) and returns FFE_OK.  Make it before reserving
   the rest of HBM and before any stream capture; otherwise the first
   cleaning call on the device does it.  All calls share the scratch: calls
   that overlap on the GPU race.  Asynchronous on `stream` (a cudaStream_t,
   NULL = the default stream); errors read back with
   ffe_last_error(NULL, ...).                                               */
int ffe_clean_epar_noalloc(int32_t sx, int32_t sy, int32_t sz, int32_t precision, void* ex, void* ey, void* ez,
                           const void* bx, const void* by, const void* bz, void* stream);

/* --- output -------------------------------------------------------------- */
/* writeOutput's field datasets (src/io/write_output.F90:336-413) at every
   istep-th node of the meshblock (:270-294): nodes i = i0 + n*istep with
   i0 = ceil(x0/istep)*istep - x0 up to (ceil((x0+sx)/istep) - 1)*istep - x0.
   dims = nodes along x, y, z.  (With istep = 1 the reference also writes the
   outer ghost nodes, whose interpolation reads outside its arrays; here
   istep = 1 gives the interior nodes.) */
int ffe_output_dims(ffe_t h, int32_t istep, int32_t dims[3]);
/* The twelve datasets ex ey ez (interpFromEdges at offset 0), bx by bz
   (interpFromFaces at offset 0; src/tools/helpers.F90:93-257), var1 (rho of
   the current E at the node's cell), var2 (user_uniform: |E x B|_perp /
   (r_perp B^2) at the cell, user/user_uniform.F90:159-170; 0 otherwise),
   var3 (0), xx yy zz (global node coordinates), into host memory: 12 arrays
   of dims[0]*dims[1]*dims[2] values of the storage precision, x fastest, in
   that order.  elems must be 12 * dims[0]*dims[1]*dims[2].  Synchronises the
   handle's stream. */
int ffe_output(ffe_t h, int32_t istep, void* host_out, size_t elems);

/* --- whole steps -------------------------------------------------------- */
/* exchangeFields(exchangeB0=.true.) then userFieldBoundaryConditions(0). */
int ffe_mainloop_prologue(ffe_t h);
/* nsteps repetitions of the main-loop body for timesteps step0 .. step0+nsteps-1:
   initRKstep; 3 x [rk3Step(c); user BC(timestep); exchange; cleanEpar; exchange]
   with c = (1,0,1), (3/4,1/4,1/4), (1/3,2/3,2/3).  Asynchronous on the
   handle's stream. */
int ffe_step(ffe_t h, int32_t nsteps, int32_t step0);
/* Which path ffe_step takes for this handle: FFE_PATH_STAGED or FFE_PATH_FUSED. */
int ffe_step_path(ffe_t h, int32_t* path);
/* Number of kernel launches one ffe_step(h, 1, .) issues. */
int ffe_step_launches(ffe_t h, int32_t* launches);

/* Sets *ok = 1 if E and B are finite over the interior, else 0 and returns
   FFE_ENONFINITE.  Synchronises the handle's stream. */
int ffe_check_finite(ffe_t h, int32_t* ok);
/* Wait for the handle's stream. */
int ffe_synchronize(ffe_t h);
/* Wait for the handle's stream, giving up after timeout_ms (FFE_ETIMEOUT). */
int ffe_synchronize_timeout(ffe_t h, int32_t timeout_ms);

/* --- batches: many meshblocks advanced together ------------------------- */
/* No counterpart in the reference (one meshblock per MPI rank there).  A batch
   groups handles created by ffe_create on the current device, all with the
   same precision (FFE_FP64, FFE_FP32 or FFE_FP32C) and all able to take the
   fused path (path AUTO or FUSED; setup none, uniform, or psr with no
   periodic axis).  The batch does not own the handles; destroy it first.
   Each SSP-RK3 stage of all members is one kernel launch over the tiles of
   every member of one B0 / absorbing-layer variant (tile height 8), or of
   every member (tile height 16), plus one batched launch per stage for
   user_uniform ghost planes and three for the pulsar fix-up; the launches
   of a call are captured into a CUDA graph and replayed.  Members keep
   their own set rotation and step counter: results equal those of ffe_step
   on each member.  stream: a cudaStream_t or NULL (own stream).           */
typedef struct ffe_batch ffe_batch;
typedef ffe_batch* ffe_batch_t;
int ffe_batch_create(ffe_batch_t* out, const ffe_t* members, int32_t n, void* stream);
int ffe_batch_destroy(ffe_batch_t b);
/* Advance every member nsteps steps; member m's first step is step0[m]
   (step0 NULL: 0 for all).  Orders itself after the work queued on each
   member's stream and makes those streams wait for it.  Asynchronous. */
int ffe_batch_step(ffe_batch_t b, int32_t nsteps, const int32_t* step0);
/* Tiling of the batched stage kernel: tile height (8 or 16; 16 needs FP32 or
   FP32C), z-planes per block (0 = per-member default), persistent blocks
   (1: one resident wave of blocks takes the work items in turn). */
int ffe_batch_set_tiling(ffe_batch_t b, int32_t tile_y, int32_t planes, int32_t persistent);
int ffe_batch_get_tiling(ffe_batch_t b, int32_t* tile_y, int32_t* planes, int32_t* persistent);
/* Time every tiling candidate on the members' current fields (a stage launch
   that writes only the set the next step overwrites; member state is
   unchanged), keep the fastest and return its time per stage in *best_ms.
   reps: timed launches per candidate (>= 1). */
int ffe_batch_autotune(ffe_batch_t b, int32_t reps, double* best_ms);
/* Kernel launches per step (nodes of the captured graph per step). */
int ffe_batch_launches(ffe_batch_t b, int32_t* per_step);
/* Wait for the batch's stream; FFE_ETIMEOUT if a stage block gave up waiting
   for its copies. */
int ffe_batch_synchronize(ffe_batch_t b);

int ffe_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* FFE_GB300_H */
