// ffe_api.cu — the C ABI declared in include/ffe.h.
//
// One handle = one meshblock resident on one GPU.  Device state is a single
// arena holding 22 arrays in the padded layout of ffe_common.cuh:
//   set[0..2][6]  three sets of (ex ey ez bx by bz)
//   b0[3]         the background field B0
//   rho           charge density (staged path only)
// plus, for the pulsar setup, a compact box buffer for its boundary condition.
//
// Two ways through a step share these arrays:
//   staged : the reference's procedures one launch each; E,B live in set[cur],
//            En,Bn in set[cur+1], dE,dB in set[cur+2] (mod 3).
//   fused  : three launches per step; stage s reads one set and writes
//            another: A -> B (stage 1), B (+A as En) -> C, C (+A) -> B, and B
//            becomes the current set.  No En/Bn copy and no separate
//            cleaning or ghost-fill pass.
#include <cstdio>
#include <cstring>
#include <cstdarg>
#include <cmath>
#include <chrono>
#include <thread>
#include <string>
#include <new>
#include <cuda.h>
#include "../../include/ffe.h"
#include "ffe_kernels.h"

using namespace ffe;

namespace {

thread_local std::string t_err;
thread_local int t_status = 0;

int set_thread_err(int st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  t_status = st;
  return st;
}

}  // namespace

int ffe::set_thread_error(int status, const char* msg) { return set_thread_err(status, "%s", msg); }

struct ffe_solver {
  ffe_grid_desc d;
  Geom g;
  Phys p;
  size_t es = 4;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  void* set[3][6] = {};
  void* b0[3] = {};
  void* rho = nullptr;
  void* box = nullptr;
  size_t box_bytes = 0;
  void* param = nullptr;  // device copy of the wave-mode table
  int* dflag = nullptr;   // finite-check word
  int* derr = nullptr;    // fused-kernel timeout word
  bool maps_ok = false;   // TMA tensor maps encoded
  CUtensorMap tm_old[3][6];  // per field array: box of tile + 2 halo (stage input)
  CUtensorMap tm_en[3][6];   // per field array: box of tile + 1 halo rows (step start)
  int cur = 0;
  bool has_b0 = false;
  bool ghosts_synced = false;  // all three sets hold the same ghost values
  std::string err;
  int err_status = 0;
  int device = 0;
};

namespace {

int fail(ffe_t h, int st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) {
    h->err = buf;
    h->err_status = st;
  }
  t_err = buf;
  t_status = st;
  return st;
}

#define FFE_CUDA(h, call)                                                                    \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return fail(h, FFE_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

int check_launch(ffe_t h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, FFE_ECUDA, "%s launch: %s", what, cudaGetErrorString(e));
  return FFE_OK;
}

template <typename R> EB<R> eb_of(ffe_t h, int s) {
  EB<R> r;
  for (int c = 0; c < 6; ++c) r.c[c] = (R*)h->set[s][c];
  return r;
}
template <typename R> CEB<R> ceb_of(ffe_t h, int s) {
  CEB<R> r;
  for (int c = 0; c < 6; ++c) r.c[c] = (const R*)h->set[s][c];
  return r;
}
template <typename R> CEB<R> ceb_b0(ffe_t h) {
  CEB<R> r{};
  for (int c = 0; c < 3; ++c) r.c[c] = (const R*)h->b0[c];
  return r;
}

inline int s_en(ffe_t h) { return (h->cur + 1) % 3; }
inline int s_d(ffe_t h) { return (h->cur + 2) % 3; }

void* field_ptr(ffe_t h, int f) {
  if (f >= FFE_EX && f <= FFE_BZ) return h->set[h->cur][f - FFE_EX];
  if (f >= FFE_B0X && f <= FFE_B0Z) return h->b0[f - FFE_B0X];
  if (f >= FFE_DEX && f <= FFE_DBZ) return h->set[s_d(h)][f - FFE_DEX];
  if (f >= FFE_ENX && f <= FFE_BNZ) return h->set[s_en(h)][f - FFE_ENX];
  if (f == FFE_RHO) return h->rho;
  return nullptr;
}

template <typename R> Absorb<R> absorb_consts(ffe_t h) {
  Absorb<R> a;
  a.xc = R(0.5) * R(h->p.gsx);  // field_solver.F90:200-204
  a.yc = R(0.5) * R(h->p.gsy);
  a.zc = R(0.5) * R(h->p.gsz);
  const R rmax = std::min(std::min(a.xc, a.yc), a.zc);
  a.rabsorb = rmax - R(h->p.absorb_buff);
  a.buff = R(h->p.absorb_buff);
  a.clamp = (h->d.flags & FFE_FLAG_ABSORB_CLAMP) ? 1 : 0;
  return a;
}

// Launches of one ghost-plane pass of the user_uniform BC (below and above).
int uniform_bc_launches(ffe_t h) {
  return (h->p.z0 <= 1 ? 1 : 0) + (h->p.z0 + h->g.sz >= h->p.gsz ? 1 : 0);
}

// TINY added to the cleaning denominators only under FFE_FLAG_CLEAN_TINY.
template <typename R> R clean_tiny(ffe_t h) {
  return (h->d.flags & FFE_FLAG_CLEAN_TINY) ? (sizeof(R) == 4 ? R(1e-7f) : R(1e-7)) : R(0);
}

// user/user_psr.F90:26-37 and :345-374, evaluated in R on the host.
template <typename R> PsrBC<R> psr_consts(ffe_t h, int step) {
  PsrBC<R> q;
  const R pi = sizeof(R) == 8 ? R(3.14159265) : R(3.14159265f);  // user_psr.F90:11
  const double* prm = h->d.params;
  q.radius = R(prm[0]);
  R angle = R(prm[1]);
  angle = angle * pi / R(180.0);
  const R period = R(prm[2] != 0.0 ? prm[2] : 1.0);
  q.omega = R(2.0) * pi / period;
  q.ccinv = R(1.0) / R(h->d.cc);
  q.xc = R(0.5) * R(h->p.gsx);
  q.yc = R(0.5) * R(h->p.gsy);
  q.zc = R(0.5) * R(h->p.gsz);
  q.sr2 = (q.radius * R(2)) * (q.radius * R(2));
  const R scale = R(prm[3] == 0.0 ? 1.0 : prm[3]);
  const R phase = q.omega * R(step);
  const R r3 = ((q.radius * q.radius) * q.radius) * scale;
  q.mu[0] = r3 * std::sin(angle) * std::cos(phase);
  q.mu[1] = r3 * std::sin(angle) * std::sin(phase);
  q.mu[2] = r3 * std::cos(angle);
  // bounding box of r < 2R in local interior indices (conservative by one cell)
  const double rad2 = 2.0 * std::fabs(prm[0]) + 1.0;
  const double cx = 0.5 * h->p.gsx, cy = 0.5 * h->p.gsy, cz = 0.5 * h->p.gsz;
  q.i_lo = std::max(0, (int)std::floor(cx - rad2) - h->p.x0);
  q.i_hi = std::min(h->g.sx - 1, (int)std::ceil(cx + rad2) - h->p.x0);
  q.j_lo = std::max(0, (int)std::floor(cy - rad2) - h->p.y0);
  q.j_hi = std::min(h->g.sy - 1, (int)std::ceil(cy + rad2) - h->p.y0);
  q.k_lo = std::max(0, (int)std::floor(cz - rad2) - h->p.z0);
  q.k_hi = std::min(h->g.sz - 1, (int)std::ceil(cz + rad2) - h->p.z0);
  q.bx = q.i_hi - q.i_lo + 1;
  q.by = q.j_hi - q.j_lo + 1;
  q.bz = q.k_hi - q.k_lo + 1;
  if (q.bx < 0) q.bx = 0;
  if (q.by < 0) q.by = 0;
  if (q.bz < 0) q.bz = 0;
  return q;
}

// user/user_uniform.F90:27-41 and :85-119, evaluated in R on the host.
template <typename R> UniformBC<R> uniform_consts(ffe_t h, int step) {
  UniformBC<R> u;
  const double* prm = h->d.params;
  const R L0 = R(prm[0]);
  u.r0 = R(prm[1]) * L0;
  const R t0 = R(prm[2]);
  u.beta = R(prm[3]);
  u.xc = R(0.5) * R(h->p.gsx);
  u.yc = R(0.5) * R(h->p.gsy);
  u.bnorm = R(1.0);
  u.cc = R(h->d.cc);
  u.tanh_t = std::tanh(R(step) / t0);
  return u;
}

// ---------------------------------------------------------------------------
// precision-dispatched operations
// ---------------------------------------------------------------------------
template <typename R, int C>
int op_rho(ffe_t h) {
  EB<R> e = eb_of<R>(h, h->cur);
  launch_rho<R>(h->g, e.c[0], e.c[1], e.c[2], (R*)h->rho, h->st);
  return check_launch(h, "computeRho");
}

template <typename R, int C>
int op_push(ffe_t h) {
  launch_push<R, C>(h->g, R(h->d.cc), ceb_of<R>(h, h->cur), ceb_b0<R>(h), h->has_b0, (const R*)h->rho,
                    eb_of<R>(h, s_d(h)), h->st);
  return check_launch(h, "rk3Push");
}

template <typename R, int C>
int op_update(ffe_t h, double c1, double c2, double c3) {
  const bool incr = C && std::fabs(c1 + c2 - 1.0) < 1e-6;
  launch_update<R, C>(h->g, h->p, absorb_consts<R>(h), R(c1), R(c2), R(c3), incr, eb_of<R>(h, h->cur),
                      ceb_of<R>(h, s_en(h)), ceb_of<R>(h, s_d(h)), h->st);
  return check_launch(h, "rk3Update");
}

template <typename R, int C>
int op_clean(ffe_t h) {
  launch_clean<R, C>(h->g, eb_of<R>(h, h->cur), eb_of<R>(h, s_d(h)), clean_tiny<R>(h), h->st);
  return check_launch(h, "cleanEpar");
}

template <typename R>
int op_fill(ffe_t h, int s, bool with_b0) {
  R* b0[3] = {(R*)h->b0[0], (R*)h->b0[1], (R*)h->b0[2]};
  launch_fill<R>(h->g, h->p, eb_of<R>(h, s), b0, with_b0, h->st);
  return check_launch(h, "exchangeFields");
}

template <typename R>
int op_bc(ffe_t h, int step) {
  switch (h->d.setup) {
    case FFE_SETUP_PSR:
      launch_psr_bc<R>(h->g, h->p, psr_consts<R>(h, step), eb_of<R>(h, h->cur), (R*)h->box, h->st);
      break;
    case FFE_SETUP_UNIFORM:
      launch_uniform_bc<R>(h->g, h->p, uniform_consts<R>(h, step), eb_of<R>(h, h->cur), false, h->st);
      break;
    case FFE_SETUP_LOOP:
      launch_loop_bc<R>(h->g, h->p, eb_of<R>(h, h->cur), h->st);
      break;
    default:
      return FFE_OK;
  }
  return check_launch(h, "userFieldBoundaryConditions");
}

template <typename R>
int op_user_init(ffe_t h) {
  const size_t bytes = (size_t)h->g.nelem * sizeof(R);
  if (h->d.setup == FFE_SETUP_NONE) return FFE_OK;
  for (int c = 0; c < 6; ++c) FFE_CUDA(h, cudaMemsetAsync(h->set[h->cur][c], 0, bytes, h->st));
  for (int c = 0; c < 3; ++c) FFE_CUDA(h, cudaMemsetAsync(h->b0[c], 0, bytes, h->st));
  h->has_b0 = false;
  EB<R> f = eb_of<R>(h, h->cur);
  if (h->d.setup == FFE_SETUP_PSR) {
    launch_psr_init<R>(h->g, h->p, psr_consts<R>(h, 0), f, h->st);
  } else if (h->d.setup == FFE_SETUP_UNIFORM) {
    launch_uniform_init<R>(h->g, h->p, uniform_consts<R>(h, 0), f.c[5], (R*)h->b0[2], h->st);
    h->has_b0 = true;
  } else if (h->d.setup == FFE_SETUP_LOOP) {
    EB<R> f0{};
    for (int c = 0; c < 3; ++c) f0.c[c] = (R*)h->b0[c];
    launch_loop_init<R>(h->g, h->p, h->d.params, f, f0, h->st);
    h->has_b0 = true;
  }
  h->ghosts_synced = false;
  return check_launch(h, "userInitialize");
}

template <typename R>
int op_init_rk(ffe_t h) {
  const size_t bytes = (size_t)h->g.nelem * sizeof(R);
  for (int c = 0; c < 6; ++c)
    FFE_CUDA(h, cudaMemcpyAsync(h->set[s_en(h)][c], h->set[h->cur][c], bytes, cudaMemcpyDeviceToDevice, h->st));
  for (int c = 0; c < 6; ++c) FFE_CUDA(h, cudaMemsetAsync(h->set[s_d(h)][c], 0, bytes, h->st));
  FFE_CUDA(h, cudaMemsetAsync(h->rho, 0, bytes, h->st));
  h->ghosts_synced = false;
  return FFE_OK;
}

// SSP-RK3 stage coefficients as default-real constants (tristanmainloop.F90:51,62,73)
template <typename R> void stage_coeffs(int s, double c[3]) {
  const R one = R(1.0);
  if (s == 0) { c[0] = 1.0; c[1] = 0.0; c[2] = 1.0; }
  else if (s == 1) { c[0] = double(R(3.0) / R(4.0)); c[1] = double(one / R(4.0)); c[2] = double(one / R(4.0)); }
  else { c[0] = double(one / R(3.0)); c[1] = double(R(2.0) / R(3.0)); c[2] = double(R(2.0) / R(3.0)); }
}

template <typename R, int C>
int step_staged(ffe_t h, int nsteps, int step0) {
  int rc;
  for (int n = 0; n < nsteps; ++n) {
    const int ts = step0 + n;
    if ((rc = op_init_rk<R>(h))) return rc;
    for (int s = 0; s < 3; ++s) {
      double c[3];
      stage_coeffs<R>(s, c);
      if ((rc = op_rho<R, C>(h))) return rc;
      if ((rc = op_push<R, C>(h))) return rc;
      if ((rc = op_update<R, C>(h, c[0], c[1], c[2]))) return rc;
      if ((rc = op_bc<R>(h, ts))) return rc;
      if ((rc = op_fill<R>(h, h->cur, false))) return rc;
      if ((rc = op_clean<R, C>(h))) return rc;
      if ((rc = op_fill<R>(h, h->cur, false))) return rc;
    }
  }
  return FFE_OK;
}

// The fused kernels run every boundary combination (halo cells on a periodic
// face next to an open face are computed at their periodic image).  The pulsar
// BC runs on the fused path through a fix-up of its box when no axis is
// periodic; the other user boundary conditions run staged.
bool fused_possible(ffe_t h) {
  const int* b = h->d.boundary;
  const bool any_per = b[0] == 1 || b[1] == 1 || b[2] == 1;
  return h->maps_ok && (h->d.setup == FFE_SETUP_NONE || h->d.setup == FFE_SETUP_UNIFORM ||
                        (h->d.setup == FFE_SETUP_PSR && !any_per));
}

template <typename R>
int sync_ghosts(ffe_t h) {
  if (h->ghosts_synced) return FFE_OK;
  const size_t bytes = (size_t)h->g.nelem * sizeof(R);
  for (int s = 0; s < 3; ++s) {
    if (s == h->cur) continue;
    for (int c = 0; c < 6; ++c)
      FFE_CUDA(h, cudaMemcpyAsync(h->set[s][c], h->set[h->cur][c], bytes, cudaMemcpyDeviceToDevice, h->st));
  }
  h->ghosts_synced = true;
  return FFE_OK;
}

// Elements of one of the two pulsar fix-up buffers: 6 components over the BC
// box dilated by two cells.
template <typename R> size_t psr_fix_elems(ffe_t h) {
  const PsrBC<R> q = psr_consts<R>(h, 0);
  if (q.bx <= 0 || q.by <= 0 || q.bz <= 0) return 0;
  return (size_t)6 * (q.bx + 4) * (q.by + 4) * (q.bz + 4);
}

template <typename R, int C>
int step_fused(ffe_t h, int nsteps, int step0, bool exact) {
  int rc;
  if ((rc = sync_ghosts<R>(h))) return rc;
  const Absorb<R> ab = absorb_consts<R>(h);
  const CEB<R> b0 = ceb_b0<R>(h);
  const bool psr = h->d.setup == FFE_SETUP_PSR;
  const bool uni = h->d.setup == FFE_SETUP_UNIFORM;
  R* s1 = (R*)h->box;
  R* s2 = psr ? s1 + psr_fix_elems<R>(h) : nullptr;
  for (int n = 0; n < nsteps; ++n) {
    const int A = h->cur, B = (h->cur + 1) % 3, Cs = (h->cur + 2) % 3;
    const int ins[3] = {A, B, Cs}, outs[3] = {B, Cs, B};
    PsrBC<R> q{};
    if (psr) q = psr_consts<R>(h, step0 + n);
    UniformBC<R> ub{};
    if (uni) ub = uniform_consts<R>(h, step0 + n);
    const UniformBC<R>* ubp = uni ? &ub : nullptr;
    for (int s = 0; s < 3; ++s) {
      double c[3];
      stage_coeffs<R>(s, c);
      // c1 + c2 = 1 exactly for SSP-RK3; in FP32 the rounded 1/3 + 2/3 misses by 3e-8
      const bool incr = C && std::fabs(c[0] + c[1] - 1.0) < 1e-6;
      const void* mi = h->tm_old[ins[s]];
      const void* me = h->tm_en[A];
      const R ct = clean_tiny<R>(h);
      int lr;
      if (exact)
        lr = launch_fused_stage_exact<R, C>(h->g, h->p, ab, R(h->d.cc), R(c[0]), R(c[1]), R(c[2]), incr, s + 1, mi,
                                            me, ceb_of<R>(h, ins[s]), ceb_of<R>(h, A), b0, h->has_b0,
                                            eb_of<R>(h, outs[s]), ct, ubp, h->derr, h->st);
      else
        lr = launch_fused_stage<R, C>(h->g, h->p, ab, R(h->d.cc), R(c[0]), R(c[1]), R(c[2]), incr, s + 1, mi, me,
                                      ceb_of<R>(h, ins[s]), ceb_of<R>(h, A), b0, h->has_b0, eb_of<R>(h, outs[s]),
                                      ct, ubp, h->derr, h->st);
      if (lr) return fail(h, FFE_ECUDA, "fused stage: cannot raise the shared-memory limit");
      if ((rc = check_launch(h, "fused stage"))) return rc;
      if (psr) {
        if (exact)
          launch_psr_fixup_exact<R, C>(h->g, h->p, ab, q, R(h->d.cc), R(c[0]), R(c[1]), R(c[2]), incr, s + 1,
                                       ceb_of<R>(h, ins[s]), ceb_of<R>(h, A), b0, h->has_b0, eb_of<R>(h, outs[s]),
                                       ct, s1, s2, h->st);
        else
          launch_psr_fixup<R, C>(h->g, h->p, ab, q, R(h->d.cc), R(c[0]), R(c[1]), R(c[2]), incr, s + 1,
                                 ceb_of<R>(h, ins[s]), ceb_of<R>(h, A), b0, h->has_b0, eb_of<R>(h, outs[s]), ct,
                                 s1, s2, h->st);
        if ((rc = check_launch(h, "pulsar boundary fix-up"))) return rc;
      }
      if (uni) {  // the ghost planes of the output set take this step's BC values
        launch_uniform_bc<R>(h->g, h->p, ub, eb_of<R>(h, outs[s]), true, h->st);
        if ((rc = check_launch(h, "uniform boundary ghosts"))) return rc;
      }
    }
    h->cur = B;
  }
  return FFE_OK;
}

template <typename R, int C>
int do_step(ffe_t h, int nsteps, int step0) {
  const int path = h->d.path;
  if (path == FFE_PATH_STAGED || (path == FFE_PATH_AUTO && !fused_possible(h))) return step_staged<R, C>(h, nsteps, step0);
  if (!fused_possible(h))
    return fail(h, FFE_EUNSUPPORTED,
                "fused path: setup must be none, or psr with no periodic axis (other user BCs run staged)");
  return step_fused<R, C>(h, nsteps, step0, path == FFE_PATH_FUSED_EXACT);
}

// precision -> (storage type, combination/denominator mode): 0 the reference's
// arithmetic, 1 increment-form RK combination, 2 that plus double B^2 denominators
#define DISPATCH(h, FN, ...)                                                             \
  ((h)->d.precision == FFE_FP64     ? FN<double, 0>(__VA_ARGS__)                          \
   : (h)->d.precision == FFE_FP32C  ? FN<float, 1>(__VA_ARGS__)                           \
   : (h)->d.precision == FFE_FP32CD ? FN<float, 2>(__VA_ARGS__)                           \
                                    : FN<float, 0>(__VA_ARGS__))
#define DISPATCH_R(h, FN, ...) ((h)->d.precision == FFE_FP64 ? FN<double>(__VA_ARGS__) : FN<float>(__VA_ARGS__))

int check_handle(ffe_t h) {
  if (!h) return set_thread_err(FFE_EINVAL, "null handle");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return fail(h, FFE_ECUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  return FFE_OK;
}

}  // namespace

extern "C" {

int ffe_abi_version(void) { return FFE_ABI_VERSION; }

int ffe_desc_default(ffe_grid_desc* d, int32_t sx, int32_t sy, int32_t sz) {
  if (!d) return set_thread_err(FFE_EINVAL, "null descriptor");
  memset(d, 0, sizeof *d);
  d->sx = sx; d->sy = sy; d->sz = sz;
  d->gsx = sx; d->gsy = sy; d->gsz = sz;
  d->boundary[0] = d->boundary[1] = d->boundary[2] = FFE_BOUNDARY_PERIODIC;
  d->absorb_buff = 20;
  d->precision = FFE_FP32;
  d->setup = FFE_SETUP_NONE;
  d->path = FFE_PATH_AUTO;
  d->cc = 0.45;
  return FFE_OK;
}

int ffe_create(ffe_t* out, const ffe_grid_desc* din) {
  if (!out || !din) return set_thread_err(FFE_EINVAL, "null argument");
  *out = nullptr;
  ffe_grid_desc d = *din;
  if (d.sx < FFE_NGHOST || d.sy < FFE_NGHOST || d.sz < FFE_NGHOST)
    return set_thread_err(FFE_EINVAL, "ERROR: ghost zones overflow the domain size (s=%d,%d,%d < %d)", d.sx, d.sy,
                          d.sz, FFE_NGHOST);
  if (d.gsx < d.sx || d.gsy < d.sy || d.gsz < d.sz)
    return set_thread_err(FFE_EINVAL, "global mesh smaller than the meshblock");
  if (d.precision < FFE_FP64 || d.precision > FFE_FP32CD)
    return set_thread_err(FFE_EINVAL, "bad precision %d", d.precision);
  if (d.setup < FFE_SETUP_NONE || d.setup > FFE_SETUP_LOOP) return set_thread_err(FFE_EINVAL, "bad setup %d", d.setup);
  if (d.path < FFE_PATH_AUTO || d.path > FFE_PATH_FUSED_EXACT) return set_thread_err(FFE_EINVAL, "bad path %d", d.path);
  if ((d.flags & ~(FFE_FLAG_ABSORB_CLAMP | FFE_FLAG_CLEAN_TINY)) || d.reserved)
    return set_thread_err(FFE_EINVAL, "unknown flags 0x%x", d.flags);
  for (int a = 0; a < 3; ++a)
    if (d.boundary[a] < 0 || d.boundary[a] > 2) return set_thread_err(FFE_EINVAL, "bad boundary %d", d.boundary[a]);
  // one absorbing axis makes all three absorbing (src/logistics/initialize.F90:144-148)
  if (d.boundary[0] == 2 || d.boundary[1] == 2 || d.boundary[2] == 2)
    d.boundary[0] = d.boundary[1] = d.boundary[2] = 2;
  if (d.boundary[0] == 2 && d.absorb_buff <= 0) return set_thread_err(FFE_EINVAL, "absorb_buff must be positive");
  if (!(d.cc > 0.0)) return set_thread_err(FFE_EINVAL, "c must be positive");
  if (d.setup == FFE_SETUP_PSR && !(d.params[0] > 0.0 && d.params[2] != 0.0))
    return set_thread_err(FFE_EINVAL, "psr setup needs psr_radius > 0 and psr_period != 0");
  if (d.setup == FFE_SETUP_UNIFORM && !(d.params[0] > 0.0 && d.params[1] > 0.0 && d.params[2] > 0.0))
    return set_thread_err(FFE_EINVAL, "uniform setup needs L0, r_L0, t0 > 0");
  if (d.setup == FFE_SETUP_LOOP && !(d.params[0] > 0.0))
    return set_thread_err(FFE_EINVAL, "loop setup needs L0 > 0");

  ffe_solver* h = new (std::nothrow) ffe_solver();
  if (!h) return set_thread_err(FFE_ENOMEM, "host allocation failed");
  h->d = d;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) {
    delete h;
    return set_thread_err(FFE_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  }
  const bool dbl = d.precision == FFE_FP64;
  h->es = dbl ? 8 : 4;
  const int ox = dbl ? Layout<double>::OX : Layout<float>::OX;
  const int pxa = dbl ? Layout<double>::PXA : Layout<float>::PXA;
  Geom& g = h->g;
  g.sx = d.sx; g.sy = d.sy; g.sz = d.sz;
  g.ox = ox;
  g.px = ((ox + d.sx + NG) + pxa - 1) / pxa * pxa;
  g.py = d.sy + 2 * NG;
  g.plane = (long long)g.px * g.py;
  g.nelem = g.plane * (d.sz + 2 * NG);
  Phys& p = h->p;
  p.x0 = d.x0; p.y0 = d.y0; p.z0 = d.z0;
  p.gsx = d.gsx; p.gsy = d.gsy; p.gsz = d.gsz;
  for (int a = 0; a < 3; ++a) p.bnd[a] = d.boundary[a];
  p.absorb_buff = d.absorb_buff;
  p.cc = d.cc;

  const size_t abytes = ((size_t)g.nelem * h->es + 255) / 256 * 256;
  size_t total = abytes * 22;
  if (d.setup == FFE_SETUP_PSR) {
    // staged BC: 6 x box; fused fix-up: two buffers of 6 x (box + 2 cells)
    h->box_bytes = 2 * (dbl ? psr_fix_elems<double>(h) * 8 : psr_fix_elems<float>(h) * 4);
    h->box_bytes = (h->box_bytes + 255) / 256 * 256;
    total += h->box_bytes;
  }
  const size_t pbytes = (waves_param_bytes() + 255) / 256 * 256;
  total += pbytes;
  total += 256;  // flag word
  if (d.stream) {
    h->st = (cudaStream_t)d.stream;
  } else {
    e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete h;
      return set_thread_err(FFE_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    h->own_stream = true;
  }
  e = cudaMalloc(&h->arena, total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (h->own_stream) cudaStreamDestroy(h->st);
    delete h;
    return set_thread_err(FFE_ENOMEM, "cudaMalloc(%zu bytes): %s", total, cudaGetErrorString(e));
  }
  h->arena_bytes = total;
  char* base = (char*)h->arena;
  for (int s = 0; s < 3; ++s)
    for (int c = 0; c < 6; ++c) h->set[s][c] = base + abytes * (s * 6 + c);
  for (int c = 0; c < 3; ++c) h->b0[c] = base + abytes * (18 + c);
  h->rho = base + abytes * 21;
  size_t off = abytes * 22;
  if (h->box_bytes) {
    h->box = base + off;
    off += h->box_bytes;
  }
  h->param = base + off;
  off += pbytes;
  h->dflag = (int*)(base + off);
  h->derr = h->dflag + 1;
  e = cudaMemsetAsync(h->arena, 0, total, h->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e != cudaSuccess) {
    cudaFree(h->arena);
    if (h->own_stream) cudaStreamDestroy(h->st);
    delete h;
    return set_thread_err(FFE_ECUDA, "arena clear: %s", cudaGetErrorString(e));
  }
  // TMA tensor maps of every field array for the fused kernels
  h->maps_ok = true;
  for (int s = 0; s < 3 && h->maps_ok; ++s)
    for (int c = 0; c < 6 && h->maps_ok; ++c)
      h->maps_ok = make_stage_maps(&h->tm_old[s][c], &h->tm_en[s][c], h->set[s][c], g, (int)h->es) == 0;
  if (!h->maps_ok && d.path >= FFE_PATH_FUSED) {
    cudaFree(h->arena);
    if (h->own_stream) cudaStreamDestroy(h->st);
    delete h;
    return set_thread_err(FFE_EUNSUPPORTED, "cannot encode TMA tensor maps for the fused path");
  }
  *out = h;
  return FFE_OK;
}

int ffe_destroy(ffe_t h) {
  if (!h) return FFE_OK;
  cudaSetDevice(h->device);
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->arena) cudaFree(h->arena);
  if (h->own_stream) cudaStreamDestroy(h->st);
  delete h;
  return FFE_OK;
}

int ffe_last_error(ffe_t h, char* buf, size_t len) {
  const std::string& s = h ? h->err : t_err;
  const int st = h ? h->err_status : t_status;
  if (buf && len) {
    size_t n = std::min(len - 1, s.size());
    memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return st;
}

int ffe_field_elems(ffe_t h, size_t* n) {
  if (!h || !n) return set_thread_err(FFE_EINVAL, "null argument");
  *n = (size_t)(h->g.sx + 2 * NG) * (h->g.sy + 2 * NG) * (h->g.sz + 2 * NG);
  return FFE_OK;
}

int ffe_device_bytes(ffe_t h, size_t* b) {
  if (!h || !b) return set_thread_err(FFE_EINVAL, "null argument");
  *b = h->arena_bytes;
  return FFE_OK;
}

int ffe_upload(ffe_t h, int32_t f, const void* host, size_t n) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  size_t need;
  ffe_field_elems(h, &need);
  if (!host || n != need) return fail(h, FFE_EINVAL, "upload: need %zu elements, got %zu", need, n);
  void* dst = field_ptr(h, f);
  if (!dst) return fail(h, FFE_EINVAL, "upload: bad field id %d", f);
  const size_t es = h->es;
  const size_t row = (size_t)(h->g.sx + 2 * NG) * es;
  FFE_CUDA(h, cudaMemcpy2DAsync((char*)dst + (h->g.ox - NG) * es, (size_t)h->g.px * es, host, row, row,
                                (size_t)(h->g.sy + 2 * NG) * (h->g.sz + 2 * NG), cudaMemcpyHostToDevice, h->st));
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  if (f >= FFE_B0X && f <= FFE_B0Z) {
    // B0 enters the curl only when non-zero somewhere (field_solver.F90:84-89)
    const unsigned char* b = (const unsigned char*)host;
    bool nz = false;
    for (size_t i = 0; i < n * es && !nz; ++i) nz = b[i] != 0;
    if (nz) h->has_b0 = true;
  }
  h->ghosts_synced = false;
  return FFE_OK;
}

int ffe_download(ffe_t h, int32_t f, void* host, size_t n) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  size_t need;
  ffe_field_elems(h, &need);
  if (!host || n != need) return fail(h, FFE_EINVAL, "download: need %zu elements, got %zu", need, n);
  void* src = field_ptr(h, f);
  if (!src) return fail(h, FFE_EINVAL, "download: bad field id %d", f);
  const size_t es = h->es;
  const size_t row = (size_t)(h->g.sx + 2 * NG) * es;
  FFE_CUDA(h, cudaMemcpy2DAsync(host, row, (const char*)src + (h->g.ox - NG) * es, (size_t)h->g.px * es, row,
                                (size_t)(h->g.sy + 2 * NG) * (h->g.sz + 2 * NG), cudaMemcpyDeviceToHost, h->st));
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  return FFE_OK;
}

int ffe_init_rk_step(ffe_t h) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  return DISPATCH_R(h, op_init_rk, h);
}
int ffe_compute_rho(ffe_t h) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  return DISPATCH(h, op_rho, h);
}
int ffe_rk3_push(ffe_t h) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  return DISPATCH(h, op_push, h);
}
int ffe_rk3_update(ffe_t h, double c1, double c2, double c3) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  h->ghosts_synced = false;
  return DISPATCH(h, op_update, h, c1, c2, c3);
}
int ffe_rk3_stage(ffe_t h, double c1, double c2, double c3) {
  int rc;
  if ((rc = ffe_compute_rho(h))) return rc;
  if ((rc = ffe_rk3_push(h))) return rc;
  return ffe_rk3_update(h, c1, c2, c3);
}
int ffe_clean_epar(ffe_t h) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  return DISPATCH(h, op_clean, h);
}
int ffe_exchange_fields(ffe_t h, int32_t b0) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  h->ghosts_synced = false;
  return DISPATCH_R(h, op_fill, h, h->cur, b0 != 0);
}
int ffe_user_initialize(ffe_t h) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  return DISPATCH_R(h, op_user_init, h);
}
int ffe_user_bc(ffe_t h, int32_t step) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  h->ghosts_synced = false;
  return DISPATCH_R(h, op_bc, h, step);
}
int ffe_mainloop_prologue(ffe_t h) {
  int rc;
  if ((rc = ffe_exchange_fields(h, 1))) return rc;
  return ffe_user_bc(h, 0);
}
int ffe_step(ffe_t h, int32_t nsteps, int32_t step0) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  if (nsteps < 0) return fail(h, FFE_EINVAL, "nsteps < 0");
  return DISPATCH(h, do_step, h, nsteps, step0);
}
int ffe_step_path(ffe_t h, int32_t* path) {
  if (!h || !path) return set_thread_err(FFE_EINVAL, "null argument");
  const int p = h->d.path;
  if (p == FFE_PATH_STAGED || (p == FFE_PATH_AUTO && !fused_possible(h))) *path = FFE_PATH_STAGED;
  else *path = p == FFE_PATH_FUSED_EXACT ? FFE_PATH_FUSED_EXACT : FFE_PATH_FUSED;
  return FFE_OK;
}
int ffe_step_launches(ffe_t h, int32_t* n) {
  int32_t path;
  int rc;
  if ((rc = ffe_step_path(h, &path))) return rc;
  if (path != FFE_PATH_STAGED) {
    // per stage: the fused kernel, plus the three box fix-up kernels of the pulsar BC
    *n = h->d.setup == FFE_SETUP_PSR ? 12 : h->d.setup == FFE_SETUP_UNIFORM ? 3 + 3 * uniform_bc_launches(h) : 3;
    return FFE_OK;
  }
  // per stage: rho, push, update, [bc], [fill], clean + copy, [fill]
  const bool periodic = h->p.bnd[0] == 1 || h->p.bnd[1] == 1 || h->p.bnd[2] == 1;
  int bc = 0;
  if (h->d.setup == FFE_SETUP_PSR) bc = 2;
  else if (h->d.setup == FFE_SETUP_UNIFORM) bc = 2;
  else if (h->d.setup == FFE_SETUP_LOOP) bc = 1;
  *n = 3 * (3 + bc + (periodic ? 2 : 0) + 2);
  return FFE_OK;
}

int ffe_check_finite(ffe_t h, int32_t* ok) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  if (!ok) return fail(h, FFE_EINVAL, "null argument");
  FFE_CUDA(h, cudaMemsetAsync(h->dflag, 0, sizeof(int), h->st));
  if (h->d.precision == FFE_FP64) launch_finite<double>(h->g, ceb_of<double>(h, h->cur), h->dflag, h->st);
  else launch_finite<float>(h->g, ceb_of<float>(h, h->cur), h->dflag, h->st);
  if ((rc = check_launch(h, "check_finite"))) return rc;
  int bad = 0;
  FFE_CUDA(h, cudaMemcpyAsync(&bad, h->dflag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  *ok = bad ? 0 : 1;
  if (bad) return fail(h, FFE_ENONFINITE, "non-finite E or B in the interior");
  return FFE_OK;
}

int ffe_init_waves(ffe_t h, const double bg[3], int32_t nmodes, const double* modes) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  if (!bg || nmodes < 0 || nmodes > 64 || (nmodes > 0 && !modes))
    return fail(h, FFE_EINVAL, "init_waves: need bg[3] and 0 <= nmodes <= 64");
  const size_t bytes = (size_t)h->g.nelem * h->es;
  for (int c = 0; c < 3; ++c) FFE_CUDA(h, cudaMemsetAsync(h->b0[c], 0, bytes, h->st));
  h->has_b0 = false;
  if (h->d.precision == FFE_FP64) rc = launch_waves<double>(h->g, h->p, bg, nmodes, modes, h->param, eb_of<double>(h, h->cur), h->st);
  else rc = launch_waves<float>(h->g, h->p, bg, nmodes, modes, h->param, eb_of<float>(h, h->cur), h->st);
  if (rc) return fail(h, FFE_ECUDA, "init_waves: parameter copy failed");
  h->ghosts_synced = false;
  return check_launch(h, "init_waves");
}

// A fused-stage block that gave up waiting for its TMA copies leaves a 1 in
// the handle's error word; report it (and clear it) once the stream is idle.
static int check_device_error(ffe_t h) {
  int e = 0;
  FFE_CUDA(h, cudaMemcpyAsync(&e, h->derr, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  if (e) {
    FFE_CUDA(h, cudaMemsetAsync(h->derr, 0, sizeof(int), h->st));
    return fail(h, FFE_ETIMEOUT, "a fused-stage block timed out waiting for its plane copies");
  }
  return FFE_OK;
}

int ffe_synchronize(ffe_t h) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  return check_device_error(h);
}

int ffe_synchronize_timeout(ffe_t h, int32_t timeout_ms) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(h->st);
    if (e == cudaSuccess) return check_device_error(h);
    if (e != cudaErrorNotReady) return fail(h, FFE_ECUDA, "cudaStreamQuery: %s", cudaGetErrorString(e));
    const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
    if (ms >= timeout_ms) return fail(h, FFE_ETIMEOUT, "stream not idle after %d ms", timeout_ms);
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
}

}  // extern "C"
