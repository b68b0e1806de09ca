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
// (24 MiB), present on every GPU where this library is loaded, until the
// process exits.  Host code must not pass the symbol itself to a kernel (on
// the host it is only a stand-in); the device address is looked up once per
// device with cudaGetSymbolAddress, on the first call made with that device
// current, and cached.  Every call shares the array and leaves its contents
// behind; the kernel writes every scratch element it later reads, so nothing
// needs clearing.  Two calls whose work overlaps on the GPU (different
// streams, or different host threads on one device) race on the array.
//
// Compiled with -fmad=false, like the staged kernels: the result equals
// ffe_clean_epar on a handle bit for bit.
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
void* g_scratch_addr[MAX_DEVICES] = {};

// Device address of the scratch on the current device (looked up once).
int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_thread_error(FFE_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= MAX_DEVICES) return set_thread_error(FFE_EUNSUPPORTED, "clean_epar_noalloc: device index >= 64");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return set_thread_error(FFE_ECUDA, "clean_epar_noalloc: cudaGetSymbolAddress of the scratch failed");
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
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

// cleanEpar of one interior cell into the compact scratch (3 x sx*sy*sz).
template <typename R, int C>
__global__ void k_clean_noalloc(Geom g, CEB<R> eb, R* __restrict__ scratch) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  RefAcc<R> a;
  for (int c = 0; c < 6; ++c) a.f[c] = eb.c[c];
  a.s = g.idx(i, j, k);
  a.dj = g.px;
  a.dk = g.plane;
  R e[3];
  clean_cell<R, C>(a, e);
  const long long n = (long long)g.sx * g.sy * g.sz;
  const long long o = i + (long long)g.sx * (j + (long long)g.sy * k);
  scratch[o] = e[0];
  scratch[n + o] = e[1];
  scratch[2 * n + o] = e[2];
}

// ex(interior) = dex (field_solver.F90:332-334), from the scratch.
template <typename R>
__global__ void k_copy_noalloc(Geom g, const R* __restrict__ scratch, R* __restrict__ ex, R* __restrict__ ey,
                               R* __restrict__ ez) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  const long long n = (long long)g.sx * g.sy * g.sz;
  const long long o = i + (long long)g.sx * (j + (long long)g.sy * k);
  const long long s = g.idx(i, j, k);
  ex[s] = scratch[o];
  ey[s] = scratch[n + o];
  ez[s] = scratch[2 * n + o];
}

template <typename R, int C>
int run(const Geom& g, void* ex, void* ey, void* ez, const void* bx, const void* by, const void* bz, void* scratch,
        cudaStream_t st) {
  CEB<R> eb;
  eb.c[0] = (const R*)ex; eb.c[1] = (const R*)ey; eb.c[2] = (const R*)ez;
  eb.c[3] = (const R*)bx; eb.c[4] = (const R*)by; eb.c[5] = (const R*)bz;
  const dim3 b(32, 8, 1), gr((g.sx + 31) / 32, (g.sy + 7) / 8, g.sz);
  k_clean_noalloc<R, C><<<gr, b, 0, st>>>(g, eb, (R*)scratch);
  k_copy_noalloc<R><<<gr, b, 0, st>>>(g, (const R*)scratch, (R*)ex, (R*)ey, (R*)ez);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_thread_error(FFE_ECUDA, cudaGetErrorString(e));
  return FFE_OK;
}

}  // namespace
}  // namespace ffe

extern "C" int ffe_clean_epar_noalloc(int32_t sx, int32_t sy, int32_t sz, int32_t precision, void* ex, void* ey,
                                      void* ez, const void* bx, const void* by, const void* bz, void* stream) {
  using namespace ffe;
  if (sx < FFE_NGHOST || sy < FFE_NGHOST || sz < FFE_NGHOST)
    return set_thread_error(FFE_EINVAL, "clean_epar_noalloc: each size must be >= 2 (NGHOST)");
  if (precision < FFE_FP64 || precision > FFE_FP32CD)
    return set_thread_error(FFE_EINVAL, "clean_epar_noalloc: bad precision");
  if (!ex || !ey || !ez || !bx || !by || !bz) return set_thread_error(FFE_EINVAL, "clean_epar_noalloc: null array");
  const size_t es = precision == FFE_FP64 ? 8 : 4;
  const size_t need = 3 * (size_t)sx * (size_t)sy * (size_t)sz * es;
  if (need > NOALLOC_SCRATCH_BYTES)
    return set_thread_error(FFE_EINVAL,
                            "clean_epar_noalloc: 3 x sx*sy*sz values exceed the 24 MiB scratch "
                            "(at most 2097152 interior cells in FP32, 1048576 in FP64)");
  void* scratch = nullptr;
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
