// ffe_noalloc.cu — E-parallel cleaning on caller-owned arrays, with no
// device allocation by the library.
//
// ffe_clean_epar_noalloc is for callers that own all of their device memory
// and cannot let a library allocate: a driver that reserved its arrays up
// front to fill HBM, or a run loop in which a cudaMalloc/cudaFree (which may
// synchronise the device, and may fail once memory is fragmented) is not
// acceptable.  Such a caller passes its own E and B arrays; the out-of-place
// step of the cleaning (the dE copy of the reference, field_solver.F90:300-334)
// uses the fixed array below instead of a handle's arena.
//
// The scratch is one file-scope __device__ array of NOALLOC_SCRATCH_BYTES
// (24 MiB).  CUDA loads a module lazily by default, so the array takes device
// memory on a device when this file's module is first loaded there: at the
// set-up call (all sizes 0, all pointers null), or else at the first cleaning
// call on that device.  From then on the device holds it until the process
// exits.  A caller that is about to reserve all of HBM makes the set-up call
// first.  Host code must not pass the symbol itself to a kernel (on the host
// it is only a stand-in); the device address is looked up with
// cudaGetSymbolAddress with the device current and cached per device and
// CUDA context, so a new context on the device (after cudaDeviceReset, or a
// driver-API context made current) looks it up again.  Every call shares the
// array and leaves its contents behind; the kernel writes every scratch
// element it later reads, so nothing needs clearing.  Two calls whose work
// overlaps on the GPU (different streams, or different host threads on one
// device) race on the array.
//
// The cleaning is the reference's: no TINY in the B^2 denominators
// (field_solver.F90:300,314,328), so B = 0 gives NaN as there; it equals
// ffe_clean_epar on a handle created without FFE_FLAG_CLEAN_TINY.
// Compiled with -fmad=false, like the staged kernels: the result equals
// ffe_clean_epar on such a handle bit for bit.
#include <cuda.h>
#include <mutex>
#include "../../include/ffe.h"
#include "ffe_kernels.h"
#include "ffe_physics.cuh"

namespace ffe {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(24) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
struct ScratchSlot {
  void* ctx;   // the CUDA context the address belongs to
  void* addr;  // device address of g_noalloc_scratch in that context
};
ScratchSlot g_slot[MAX_DEVICES] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);

// Current driver context of this thread (the runtime's primary context of the
// current device once a runtime call has made it current).
int current_context(void** ctx) {
  static CtxGetCurrentFn get = nullptr;
  if (!get) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaGetLastError();
      return set_thread_error(FFE_ECUDA, "clean_epar_noalloc: cuCtxGetCurrent not available");
    }
    get = reinterpret_cast<CtxGetCurrentFn>(fn);
  }
  CUcontext c = nullptr;
  if (get(&c) != CUDA_SUCCESS || !c) return set_thread_error(FFE_ECUDA, "clean_epar_noalloc: no current context");
  *ctx = c;
  return FFE_OK;
}

template <typename R, int C>
__global__ void k_clean_noalloc(Geom g, CEB<R> eb, R* __restrict__ scratch);
template <typename R>
__global__ void k_copy_noalloc(Geom g, const R* __restrict__ scratch, R* __restrict__ ex, R* __restrict__ ey,
                               R* __restrict__ ez);

// Device address of the scratch in the current context; the lookup also loads
// the module (and with it the array) and the cleaning kernels, so that a later
// call takes no device memory.
int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_thread_error(FFE_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= MAX_DEVICES) return set_thread_error(FFE_EUNSUPPORTED, "clean_epar_noalloc: device index >= 64");
  e = cudaFree(nullptr);  // makes the device's primary context current (allocates nothing)
  if (e != cudaSuccess) return set_thread_error(FFE_ECUDA, cudaGetErrorString(e));
  void* ctx = nullptr;
  int rc = current_context(&ctx);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_slot[dev].ctx != ctx || !g_slot[dev].addr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return set_thread_error(FFE_ECUDA, "clean_epar_noalloc: cudaGetSymbolAddress of the scratch failed");
    }
    cudaFuncAttributes fa;
    const void* kernels[] = {(const void*)k_clean_noalloc<float, 0>, (const void*)k_clean_noalloc<float, 2>,
                             (const void*)k_clean_noalloc<double, 0>, (const void*)k_copy_noalloc<float>,
                             (const void*)k_copy_noalloc<double>};
    for (const void* k : kernels)
      if (cudaFuncGetAttributes(&fa, k) != cudaSuccess) {
        cudaGetLastError();
        return set_thread_error(FFE_ECUDA, "clean_epar_noalloc: loading the cleaning kernels failed");
      }
    g_slot[dev].ctx = ctx;
    g_slot[dev].addr = p;
  }
  *out = g_slot[dev].addr;
  return FFE_OK;
}

template <typename R>
struct RefAcc {  // neighbours in a caller's (sx+4)(sy+4)(sz+4) array
  const R* f[6];
  long long s, dj, dk;
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    return f[c][s + di + djj * dj + dkk * dk];
  }
};

// Interior cell o (x fastest) of an sx x sy x sz block.
__device__ __forceinline__ void cell_of(const Geom& g, long long o, int& i, int& j, int& k) {
  i = (int)(o % g.sx);
  const long long r = o / g.sx;
  j = (int)(r % g.sy);
  k = (int)(r / g.sy);
}

// cleanEpar of the interior cells into the compact scratch (3 x sx*sy*sz);
// a grid-stride loop, so any size within the scratch fits the launch limits.
template <typename R, int C>
__global__ void k_clean_noalloc(Geom g, CEB<R> eb, R* __restrict__ scratch) {
  const long long n = (long long)g.sx * g.sy * g.sz;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n; o += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(g, o, i, j, k);
    RefAcc<R> a;
    for (int c = 0; c < 6; ++c) a.f[c] = eb.c[c];
    a.s = g.idx(i, j, k);
    a.dj = g.px;
    a.dk = g.plane;
    R e[3];
    clean_cell<R, C>(a, e);
    scratch[o] = e[0];
    scratch[n + o] = e[1];
    scratch[2 * n + o] = e[2];
  }
}

// ex(interior) = dex (field_solver.F90:332-334), from the scratch.
template <typename R>
__global__ void k_copy_noalloc(Geom g, const R* __restrict__ scratch, R* __restrict__ ex, R* __restrict__ ey,
                               R* __restrict__ ez) {
  const long long n = (long long)g.sx * g.sy * g.sz;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n; o += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    cell_of(g, o, i, j, k);
    const long long s = g.idx(i, j, k);
    ex[s] = scratch[o];
    ey[s] = scratch[n + o];
    ez[s] = scratch[2 * n + o];
  }
}

template <typename R, int C>
int run(const Geom& g, void* ex, void* ey, void* ez, const void* bx, const void* by, const void* bz, void* scratch,
        cudaStream_t st) {
  CEB<R> eb;
  eb.c[0] = (const R*)ex; eb.c[1] = (const R*)ey; eb.c[2] = (const R*)ez;
  eb.c[3] = (const R*)bx; eb.c[4] = (const R*)by; eb.c[5] = (const R*)bz;
  const long long n = (long long)g.sx * g.sy * g.sz;
  const int threads = 256;
  const int blocks = (int)std::min<long long>((n + threads - 1) / threads, 152LL * 8);
  k_clean_noalloc<R, C><<<blocks, threads, 0, st>>>(g, eb, (R*)scratch);
  k_copy_noalloc<R><<<blocks, threads, 0, st>>>(g, (const R*)scratch, (R*)ex, (R*)ey, (R*)ez);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_thread_error(FFE_ECUDA, cudaGetErrorString(e));
  return FFE_OK;
}

}  // namespace
}  // namespace ffe

extern "C" int ffe_clean_epar_noalloc(int32_t sx, int32_t sy, int32_t sz, int32_t precision, void* ex, void* ey,
                                      void* ez, const void* bx, const void* by, const void* bz, void* stream) {
  using namespace ffe;
  if (precision < FFE_FP64 || precision > FFE_FP32CD)
    return set_thread_error(FFE_EINVAL, "clean_epar_noalloc: bad precision");
  void* scratch = nullptr;
  if (sx == 0 && sy == 0 && sz == 0 && !ex && !ey && !ez && !bx && !by && !bz)
    return scratch_address(&scratch);  // set-up only: load the scratch on the current device
  if (sx < FFE_NGHOST || sy < FFE_NGHOST || sz < FFE_NGHOST)
    return set_thread_error(FFE_EINVAL, "clean_epar_noalloc: each size must be >= 2 (NGHOST)");
  if (!ex || !ey || !ez || !bx || !by || !bz) return set_thread_error(FFE_EINVAL, "clean_epar_noalloc: null array");
  const size_t es = precision == FFE_FP64 ? 8 : 4;
  const size_t need = 3 * (size_t)sx * (size_t)sy * (size_t)sz * es;
  if (need > NOALLOC_SCRATCH_BYTES)
    return set_thread_error(FFE_EINVAL,
                            "clean_epar_noalloc: 3 x sx*sy*sz values exceed the 24 MiB scratch "
                            "(at most 2097152 interior cells in FP32, 1048576 in FP64)");
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  Geom g;  // the reference's dense layout: rows of sx+4, cell -2 at element 0
  g.sx = sx; g.sy = sy; g.sz = sz;
  g.ox = FFE_NGHOST;
  g.px = sx + 2 * FFE_NGHOST;
  g.py = sy + 2 * FFE_NGHOST;
  g.plane = (long long)g.px * g.py;
  g.nelem = g.plane * (sz + 2 * FFE_NGHOST);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == FFE_FP64) return run<double, 0>(g, ex, ey, ez, bx, by, bz, scratch, st);
  if (precision == FFE_FP32CD) return run<float, 2>(g, ex, ey, ez, bx, by, bz, scratch, st);
  return run<float, 0>(g, ex, ey, ez, bx, by, bz, scratch, st);  // FP32, FP32C: same cleaning
}
