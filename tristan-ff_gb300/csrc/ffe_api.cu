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
#include <vector>
#include <algorithm>
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
  void* arena_raw = nullptr;  // allocation (stream-ordered)
  void* arena = nullptr;      // 256-byte aligned start inside it
  size_t arena_bytes = 0;
  void* set[3][6] = {};
  void* b0[3] = {};
  void* rho = nullptr;
  void* box = nullptr;
  size_t box_bytes = 0;
  void* param = nullptr;  // device copy of the wave-mode table
  void* stage = nullptr;  // contiguous staging array for host copies (allocated on first use)
  void* stage2 = nullptr;            // second staging array of the multi-array copies
  cudaStream_t cst = nullptr;        // copy stream of the multi-array copies
  cudaEvent_t cev[4] = {};           // their ordering events
  int* dflag = nullptr;   // finite-check word
  int* derr = nullptr;    // fused-kernel timeout word
  bool maps_ok = false;   // TMA tensor maps encoded
  CUtensorMap tm_old[3][6];  // per field array: box of tile + 2 halo (stage input)
  CUtensorMap tm_en[3][6];   // per field array: box of tile + 1 halo rows (step start)
  CUtensorMap tm_plain[3][6];     // FP32: stage-input boxes of the plain variant's taller tile
  CUtensorMap tm_plain_en[3][6];  // FP32: its step-start boxes
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
  a.inv_buff = R(1) / a.buff;
  a.clamp = (h->d.flags & FFE_FLAG_ABSORB_CLAMP) ? 1 : 0;
  a.true_y = (h->d.flags & FFE_FLAG_ABSORB_TRUE_Y) ? 1 : 0;
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

// x_done: the fused stage kernel has stored the x ghost columns
template <typename R>
int op_fill(ffe_t h, int s, bool with_b0, bool x_done = false) {
  R* b0[3] = {(R*)h->b0[0], (R*)h->b0[1], (R*)h->b0[2]};
  launch_fill<R>(h->g, h->p, eb_of<R>(h, s), b0, with_b0, h->st, x_done);
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
      const void* mp = h->es == 4 ? (const void*)h->tm_plain[ins[s]] : nullptr;
      const void* mpe = h->es == 4 ? (const void*)h->tm_plain_en[A] : nullptr;
      const R ct = clean_tiny<R>(h);
      int lr;
      if (exact)
        lr = launch_fused_stage_exact<R, C>(h->g, h->p, ab, R(h->d.cc), R(c[0]), R(c[1]), R(c[2]), incr, s + 1, mi,
                                            me, mp, mpe, ceb_of<R>(h, ins[s]), ceb_of<R>(h, A), b0, h->has_b0,
                                            eb_of<R>(h, outs[s]), ct, ubp, h->derr, h->st);
      else
        lr = launch_fused_stage<R, C>(h->g, h->p, ab, R(h->d.cc), R(c[0]), R(c[1]), R(c[2]), incr, s + 1, mi, me,
                                      mp, mpe, ceb_of<R>(h, ins[s]), ceb_of<R>(h, A), b0, h->has_b0, eb_of<R>(h, outs[s]),
                                      ct, ubp, h->derr, h->st);
      if (lr == -4) return fail(h, FFE_EINVAL, "fused stage: the arrays of a set are not equally spaced, or no tensor maps");
      if (lr) return fail(h, FFE_ECUDA, "fused stage: cannot raise the shared-memory limit");
      if ((rc = check_launch(h, "fused stage"))) return rc;
      // the periodic images of the output set (the single-grid stage kernel
      // writes interior cells only); no launch when no axis is periodic
      if ((rc = op_fill<R>(h, outs[s], false, true))) return rc;
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

// The staging array of host copies: (sx+4)(sy+4)(sz+4) values, allocated
// stream-ordered on the first upload or download and kept until destroy.
int ensure_stage(ffe_t h) {
  if (h->stage) return FFE_OK;
  const size_t n = (size_t)(h->g.sx + 2 * NG) * (h->g.sy + 2 * NG) * (h->g.sz + 2 * NG);
  cudaError_t e = cudaMallocAsync(&h->stage, n * h->es, h->st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    h->stage = nullptr;
    return fail(h, FFE_ENOMEM, "staging array (%zu bytes): %s", n * h->es, cudaGetErrorString(e));
  }
  return FFE_OK;
}

// The second staging array, the copy stream and the events of the
// multi-array copies (created on first use).
int ensure_pipeline(ffe_t h) {
  int rc;
  if ((rc = ensure_stage(h))) return rc;
  if (!h->stage2) {
    const size_t n = (size_t)(h->g.sx + 2 * NG) * (h->g.sy + 2 * NG) * (h->g.sz + 2 * NG);
    cudaError_t e = cudaMallocAsync(&h->stage2, n * h->es, h->st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      h->stage2 = nullptr;
      return fail(h, FFE_ENOMEM, "staging array (%zu bytes): %s", n * h->es, cudaGetErrorString(e));
    }
  }
  if (!h->cst) FFE_CUDA(h, cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking));
  for (int i = 0; i < 4; ++i)
    if (!h->cev[i]) FFE_CUDA(h, cudaEventCreateWithFlags(&h->cev[i], cudaEventDisableTiming));
  return FFE_OK;
}

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

}  // extern "C"

namespace {

// Check a descriptor and apply the reference's coupling of boundaries; 0 or
// the failing status (message in the thread's error slot).
int validate_desc(ffe_grid_desc& d) {
  if (d.sx < FFE_NGHOST || d.sy < FFE_NGHOST || d.sz < FFE_NGHOST)
    return set_thread_err(FFE_EINVAL, "ERROR: ghost zones overflow the domain size (s=%d,%d,%d < %d)", d.sx, d.sy,
                          d.sz, FFE_NGHOST);
  if (d.gsx < d.sx || d.gsy < d.sy || d.gsz < d.sz)
    return set_thread_err(FFE_EINVAL, "global mesh smaller than the meshblock");
  if (d.precision < FFE_FP64 || d.precision > FFE_FP32CD)
    return set_thread_err(FFE_EINVAL, "bad precision %d", d.precision);
  if (d.setup < FFE_SETUP_NONE || d.setup > FFE_SETUP_LOOP) return set_thread_err(FFE_EINVAL, "bad setup %d", d.setup);
  if (d.path < FFE_PATH_AUTO || d.path > FFE_PATH_FUSED_EXACT) return set_thread_err(FFE_EINVAL, "bad path %d", d.path);
  if ((d.flags & ~(FFE_FLAG_ABSORB_CLAMP | FFE_FLAG_CLEAN_TINY | FFE_FLAG_ABSORB_TRUE_Y |
                   FFE_FLAG_TEST_WITHHOLD_COPY)) ||
      d.reserved)
    return set_thread_err(FFE_EINVAL, "unknown flags 0x%x", d.flags);
  for (int a = 0; a < 3; ++a)
    if (d.boundary[a] < 0 || d.boundary[a] > 2) return set_thread_err(FFE_EINVAL, "bad boundary %d", d.boundary[a]);
  // the fused kernels hold in-plane offsets in 32 bits
  if ((long long)(d.sx + 2 * FFE_NGHOST + 64) * (d.sy + 2 * FFE_NGHOST) >= (1LL << 31))
    return set_thread_err(FFE_EINVAL, "a plane of more than 2^31 elements is not supported");
  // the per-cell kernels put z planes (ghosts included) on the grid's z
  // dimension and 8-row groups on its y dimension, each at most 65535 blocks
  if (d.sz + 2 * FFE_NGHOST > 65535 || (d.sy + 2 * FFE_NGHOST + 7) / 8 > 65535)
    return set_thread_err(FFE_EINVAL, "sz + 4 must be <= 65535 and sy + 4 <= 524280 (kernel grid limits)");
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
  return FFE_OK;
}

// Layout of a handle's arena: fills es, g, p and box_bytes from h->d and
// returns the bytes of the arena; *abytes = bytes of one field array,
// *pbytes = bytes of the wave-mode table.
size_t plan_arena(ffe_solver* h, size_t* abytes, size_t* pbytes) {
  const ffe_grid_desc& d = h->d;
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
  p.withhold_copy = (d.flags & FFE_FLAG_TEST_WITHHOLD_COPY) ? 1 : 0;
  p.cc = d.cc;
  *abytes = ((size_t)g.nelem * h->es + 255) / 256 * 256;
  size_t total = *abytes * 22;
  h->box_bytes = 0;
  if (d.setup == FFE_SETUP_PSR) {
    // staged BC: 6 x box; fused fix-up: two buffers of 6 x (box + 2 cells)
    h->box_bytes = 2 * (dbl ? psr_fix_elems<double>(h) * 8 : psr_fix_elems<float>(h) * 4);
    h->box_bytes = (h->box_bytes + 255) / 256 * 256;
    total += h->box_bytes;
  }
  *pbytes = (waves_param_bytes() + 255) / 256 * 256;
  total += *pbytes;
  total += 256;  // flag word
  return total;
}

}  // namespace

extern "C" {

int ffe_desc_device_bytes(const ffe_grid_desc* din, size_t* bytes) {
  if (!din || !bytes) return set_thread_err(FFE_EINVAL, "null argument");
  ffe_solver tmp;
  tmp.d = *din;
  int rc;
  if ((rc = validate_desc(tmp.d))) return rc;
  size_t ab, pb;
  *bytes = plan_arena(&tmp, &ab, &pb);
  return FFE_OK;
}

int ffe_create(ffe_t* out, const ffe_grid_desc* din) {
  if (!out || !din) return set_thread_err(FFE_EINVAL, "null argument");
  *out = nullptr;
  ffe_grid_desc d = *din;
  int rc;
  if ((rc = validate_desc(d))) return rc;
  ffe_solver* h = new (std::nothrow) ffe_solver();
  if (!h) return set_thread_err(FFE_ENOMEM, "host allocation failed");
  h->d = d;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) {
    delete h;
    return set_thread_err(FFE_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  }
  size_t abytes = 0, pbytes = 0;
  const size_t total = plan_arena(h, &abytes, &pbytes);
  const Geom& g = h->g;
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
  // Stream-ordered allocation: creating and destroying handles (a serving loop
  // does so while other handles compute) does not synchronise the device.
  e = cudaMallocAsync(&h->arena_raw, total + 256, h->st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (h->own_stream) cudaStreamDestroy(h->st);
    delete h;
    return set_thread_err(FFE_ENOMEM, "cudaMallocAsync(%zu bytes): %s", total, cudaGetErrorString(e));
  }
  h->arena = (void*)(((uintptr_t)h->arena_raw + 255) / 256 * 256);
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
    cudaFreeAsync(h->arena_raw, h->st);
    cudaStreamSynchronize(h->st);
    if (h->own_stream) cudaStreamDestroy(h->st);
    delete h;
    return set_thread_err(FFE_ECUDA, "arena clear: %s", cudaGetErrorString(e));
  }
  // TMA tensor maps of every field array for the fused kernels
  h->maps_ok = true;
  for (int s = 0; s < 3 && h->maps_ok; ++s)
    for (int c = 0; c < 6 && h->maps_ok; ++c)
      h->maps_ok = make_stage_maps(&h->tm_old[s][c], &h->tm_en[s][c], h->set[s][c], g, (int)h->es, FUSED_TY) == 0 &&
                   (h->es != 4 ||
                    make_stage_maps(&h->tm_plain[s][c], &h->tm_plain_en[s][c], h->set[s][c], g, (int)h->es,
                                    PLAIN_TY) == 0);
  if (!h->maps_ok && d.path >= FFE_PATH_FUSED) {
    cudaFreeAsync(h->arena_raw, h->st);
    cudaStreamSynchronize(h->st);
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
  if (h->cst) {
    cudaStreamSynchronize(h->cst);
    cudaStreamDestroy(h->cst);
  }
  for (int i = 0; i < 4; ++i)
    if (h->cev[i]) cudaEventDestroy(h->cev[i]);
  if (h->stage2) cudaFreeAsync(h->stage2, h->st);
  if (h->stage) cudaFreeAsync(h->stage, h->st);
  if (h->arena_raw) {
    cudaFreeAsync(h->arena_raw, h->st);
    cudaStreamSynchronize(h->st);
  }
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
  int rc2;
  if ((rc2 = ensure_stage(h))) return rc2;
  // one contiguous copy at the host link's full rate, then a repack into the padded rows
  FFE_CUDA(h, cudaMemcpyAsync(h->stage, host, need * h->es, cudaMemcpyHostToDevice, h->st));
  if (h->es == 8) launch_repack<double>(h->g, (const double*)h->stage, (double*)dst, true, h->st);
  else launch_repack<float>(h->g, (const float*)h->stage, (float*)dst, true, h->st);
  if ((rc2 = check_launch(h, "upload repack"))) return rc2;
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  if (f >= FFE_B0X && f <= FFE_B0Z) {
    // B0 enters the curl only when non-zero somewhere (field_solver.F90:84-89)
    const unsigned char* b = (const unsigned char*)host;
    bool nz = false;
    for (size_t i = 0; i < n * h->es && !nz; ++i) nz = b[i] != 0;
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
  int rc2;
  if ((rc2 = ensure_stage(h))) return rc2;
  if (h->es == 8) launch_repack<double>(h->g, (const double*)src, (double*)h->stage, false, h->st);
  else launch_repack<float>(h->g, (const float*)src, (float*)h->stage, false, h->st);
  if ((rc2 = check_launch(h, "download repack"))) return rc2;
  FFE_CUDA(h, cudaMemcpyAsync(host, h->stage, need * h->es, cudaMemcpyDeviceToHost, h->st));
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  return FFE_OK;
}

// Several arrays: two staging arrays alternate, the host copies run on the
// copy stream and the repacks on the handle's stream, so the copy of one array
// overlaps the repack of the previous one.
int ffe_upload_many(ffe_t h, int32_t n, const int32_t* fields, const void* const* host, size_t nelems) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  size_t need;
  ffe_field_elems(h, &need);
  if (n < 0 || (n > 0 && (!fields || !host)) || nelems != need)
    return fail(h, FFE_EINVAL, "upload_many: need %zu elements per array", need);
  for (int i = 0; i < n; ++i) {
    if (!host[i]) return fail(h, FFE_EINVAL, "upload_many: null host array %d", i);
    if (!field_ptr(h, fields[i])) return fail(h, FFE_EINVAL, "upload_many: bad field id %d", fields[i]);
    if (fields[i] >= FFE_B0X && fields[i] <= FFE_B0Z)  // B0 needs the host-side zero test
      return fail(h, FFE_EINVAL, "upload_many: upload B0 with ffe_upload");
  }
  if (n == 0) return FFE_OK;
  if ((rc = ensure_pipeline(h))) return rc;
  void* st[2] = {h->stage, h->stage2};
  // cev[0,1]: copy into stage b done (copy stream); cev[2,3]: repack out of stage b done (handle stream)
  FFE_CUDA(h, cudaEventRecord(h->cev[2], h->st));
  FFE_CUDA(h, cudaEventRecord(h->cev[3], h->st));
  for (int i = 0; i < n; ++i) {
    const int b = i & 1;
    FFE_CUDA(h, cudaStreamWaitEvent(h->cst, h->cev[2 + b], 0));
    FFE_CUDA(h, cudaMemcpyAsync(st[b], host[i], need * h->es, cudaMemcpyHostToDevice, h->cst));
    FFE_CUDA(h, cudaEventRecord(h->cev[b], h->cst));
    FFE_CUDA(h, cudaStreamWaitEvent(h->st, h->cev[b], 0));
    void* dst = field_ptr(h, fields[i]);
    if (h->es == 8) launch_repack<double>(h->g, (const double*)st[b], (double*)dst, true, h->st);
    else launch_repack<float>(h->g, (const float*)st[b], (float*)dst, true, h->st);
    if ((rc = check_launch(h, "upload repack"))) return rc;
    FFE_CUDA(h, cudaEventRecord(h->cev[2 + b], h->st));
  }
  FFE_CUDA(h, cudaStreamSynchronize(h->st));
  h->ghosts_synced = false;
  return FFE_OK;
}

int ffe_download_many(ffe_t h, int32_t n, const int32_t* fields, void* const* host, size_t nelems) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  size_t need;
  ffe_field_elems(h, &need);
  if (n < 0 || (n > 0 && (!fields || !host)) || nelems != need)
    return fail(h, FFE_EINVAL, "download_many: need %zu elements per array", need);
  for (int i = 0; i < n; ++i) {
    if (!host[i]) return fail(h, FFE_EINVAL, "download_many: null host array %d", i);
    if (!field_ptr(h, fields[i])) return fail(h, FFE_EINVAL, "download_many: bad field id %d", fields[i]);
  }
  if (n == 0) return FFE_OK;
  if ((rc = ensure_pipeline(h))) return rc;
  void* st[2] = {h->stage, h->stage2};
  // cev[0,1]: pack into stage b done (handle stream); cev[2,3]: copy out of stage b done (copy stream)
  FFE_CUDA(h, cudaEventRecord(h->cev[2], h->cst));
  FFE_CUDA(h, cudaEventRecord(h->cev[3], h->cst));
  for (int i = 0; i < n; ++i) {
    const int b = i & 1;
    FFE_CUDA(h, cudaStreamWaitEvent(h->st, h->cev[2 + b], 0));
    const void* src = field_ptr(h, fields[i]);
    if (h->es == 8) launch_repack<double>(h->g, (const double*)src, (double*)st[b], false, h->st);
    else launch_repack<float>(h->g, (const float*)src, (float*)st[b], false, h->st);
    if ((rc = check_launch(h, "download repack"))) return rc;
    FFE_CUDA(h, cudaEventRecord(h->cev[b], h->st));
    FFE_CUDA(h, cudaStreamWaitEvent(h->cst, h->cev[b], 0));
    FFE_CUDA(h, cudaMemcpyAsync(host[i], st[b], need * h->es, cudaMemcpyDeviceToHost, h->cst));
    FFE_CUDA(h, cudaEventRecord(h->cev[2 + b], h->cst));
  }
  FFE_CUDA(h, cudaStreamSynchronize(h->cst));
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
  const bool periodic = h->p.bnd[0] == 1 || h->p.bnd[1] == 1 || h->p.bnd[2] == 1;
  if (path != FFE_PATH_STAGED) {
    // per stage: the fused kernel, the ghost fill of a grid with a periodic
    // axis, the three box fix-up kernels of the pulsar BC, the ghost planes
    // of the twisted-footpoint BC
    const int per_stage = 1 + (periodic ? 1 : 0) + (h->d.setup == FFE_SETUP_PSR ? 3 : 0) +
                          (h->d.setup == FFE_SETUP_UNIFORM ? uniform_bc_launches(h) : 0);
    *n = 3 * per_stage;
    return FFE_OK;
  }
  // per stage: rho, push, update, [bc], [fill], clean + copy, [fill]
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

int ffe_output_dims(ffe_t h, int32_t istep, int32_t dims[3]) {
  if (!h || !dims) return set_thread_err(FFE_EINVAL, "null argument");
  if (istep < 1) return fail(h, FFE_EINVAL, "output istep must be >= 1");
  const NodeGrid n = node_grid(h->g, h->p, istep);
  dims[0] = n.nx;
  dims[1] = n.ny;
  dims[2] = n.nz;
  return FFE_OK;
}

int ffe_output(ffe_t h, int32_t istep, void* host_out, size_t elems) {
  int rc;
  if ((rc = check_handle(h))) return rc;
  if (istep < 1) return fail(h, FFE_EINVAL, "output istep must be >= 1");
  const NodeGrid n = node_grid(h->g, h->p, istep);
  const size_t nn = (size_t)n.nx * n.ny * n.nz;
  if (!host_out || elems != 12 * nn)
    return fail(h, FFE_EINVAL, "output: need 12 * %d * %d * %d = %zu elements, got %zu", n.nx, n.ny, n.nz, 12 * nn,
                elems);
  if (!nn) return FFE_OK;
  void* dbuf = nullptr;
  FFE_CUDA(h, cudaMallocAsync(&dbuf, 12 * nn * h->es, h->st));
  const bool v2 = h->d.setup == FFE_SETUP_UNIFORM;
  if (h->d.precision == FFE_FP64)
    launch_node_output<double>(h->g, h->p, n, v2, ceb_of<double>(h, h->cur), (double*)dbuf, h->st);
  else
    launch_node_output<float>(h->g, h->p, n, v2, ceb_of<float>(h, h->cur), (float*)dbuf, h->st);
  rc = check_launch(h, "node output");
  cudaError_t e = cudaSuccess;
  if (!rc) e = cudaMemcpyAsync(host_out, dbuf, 12 * nn * h->es, cudaMemcpyDeviceToHost, h->st);
  cudaFreeAsync(dbuf, h->st);
  cudaError_t e2 = cudaStreamSynchronize(h->st);
  if (rc) return rc;
  if (e != cudaSuccess || e2 != cudaSuccess)
    return fail(h, FFE_ECUDA, "output copy: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
  return FFE_OK;
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

// ===========================================================================
// Batches (ffe_batch_*): many meshblocks advanced together.
//
// Members are split into groups of up to BATCH_MAX.  Each SSP-RK3 stage of a
// group is one launch over the work items (member, tile, z-chunk) of all its
// members of one B0 / absorbing-layer variant (k_fused_batch_var, tile height
// 8), or of all its members (k_fused_batch, which switches per grid; tile
// height 16, or a member's variant changed); every member has an entry (BatchBox) in the
// launch's parameter table with its stage constants, its set pointers (the
// member's own set rotation) and this step's boundary constants.  Pulsar
// members add one batched fix-up (three launches) per stage, user_uniform
// members one batched ghost-plane launch.  The launches of a chunk of up to
// kChunk steps are captured into a CUDA graph; a later chunk of the same
// length updates the instantiated graph in place (same topology, new
// parameters) and replays it.
// ===========================================================================

struct ffe_batch {
  struct Group {
    int first = 0, n = 0;          // members [first, first + n)
    BatchItem* ditems = nullptr;   // stage work items (box = index in the group)
    int nitems = 0, cap = 0;
    FixItem* dghost = nullptr;     // user_uniform ghost-plane items (box = index in the group)
    int nghost = 0;
    // B0 / absorbing-layer variant of each member when the items were built
    // (bit 1 B0, bit 0 absorbing layer); the items are ordered by variant,
    // those of variant v at [vfirst[v], vfirst[v] + vcount[v])
    int mvar[BATCH_MAX] = {};
    int vfirst[4] = {}, vcount[4] = {};
  };
  struct G {
    int steps;
    cudaGraphExec_t exec;
  };
  int device = 0;
  int precision = FFE_FP32;
  std::vector<ffe_t> m;
  std::vector<Group> groups;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  cudaEvent_t ev = nullptr;      // ordering with member streams
  cudaEvent_t copied = nullptr;  // host staging of the fix-up table free again
  int ty = 8, kz = 0, persistent = 0;
  int blocks_per_sm = 0, sms = 0;
  int spec_bps[4] = {0, 0, 0, 0};  // blocks per SM of the one-variant kernels (tile 8), 0: none
  int* derr = nullptr;           // device timeout word
  CUtensorMap* dmaps = nullptr;  // device: [tile 8|16][member][set][12 maps]
  std::vector<int> kz_of;        // planes per block of each member
  FixItem* dfix = nullptr;       // pulsar fix-up items (box = pulsar index)
  int nfix = 0;
  std::vector<int> psr;          // members with the pulsar fix-up
  std::vector<unsigned char> tabs;  // host: BoxTable per (step, stage, group) of a chunk
  void* dfixtab = nullptr;       // device: FixParams [steps][3][pulsar members]
  void* hfixtab = nullptr;       // pinned staging of the fix-up table
  int fix_steps = 0;             // capacity of the fix-up tables in steps
  std::vector<G> graphs;         // instantiated graphs, by chunk length
};

namespace {

constexpr int kChunk = 256;  // steps per captured graph

int bfail(int st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  t_status = st;
  return st;
}

#define BCUDA(call)                                                                          \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return bfail(FFE_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

size_t fix_entry_bytes(int prec) {
  return prec == FFE_FP64 ? sizeof(FixParams<double>) : sizeof(FixParams<float>);
}

void drop_graphs(ffe_batch* b) {
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
  b->graphs.clear();
}

int tile_index(int ty) { return ty == 16 ? 1 : 0; }

int variant_of(const ffe_solver* h) { return (h->has_b0 ? 2 : 0) | (h->p.bnd[0] == 2 ? 1 : 0); }

// Work items of the current tiling per group, by variant and within a
// variant largest blocks first (the hardware and the persistent loop both
// take items in order).
int build_items(ffe_batch* b) {
  const int nm = (int)b->m.size();
  b->kz_of.assign(nm, 0);
  for (auto& gr : b->groups) {
    std::vector<std::pair<long long, BatchItem>> it;
    for (int l = 0; l < gr.n; ++l) {
      const int i = gr.first + l;
      gr.mvar[l] = variant_of(b->m[i]);
      const Geom& g = b->m[i]->g;
      const int kz = b->kz ? std::min(b->kz, g.sz) : fused_planes_per_block(g, b->ty);
      b->kz_of[i] = kz;
      const int tx = (g.sx + FUSED_TX - 1) / FUSED_TX, tyn = (g.sy + b->ty - 1) / b->ty, tz = (g.sz + kz - 1) / kz;
      for (int z = 0; z < tz; ++z)
        for (int y = 0; y < tyn; ++y)
          for (int x = 0; x < tx; ++x) {
            const long long w = (long long)std::min(FUSED_TX, g.sx - x * FUSED_TX) *
                                std::min(b->ty, g.sy - y * b->ty) * std::min(kz, g.sz - z * kz);
            it.push_back({w, BatchItem{l, x, y, z}});
          }
    }
    std::stable_sort(it.begin(), it.end(), [&](const auto& a, const auto& c) {
      const int va = gr.mvar[a.second.box], vc = gr.mvar[c.second.box];
      return va != vc ? va < vc : a.first > c.first;
    });
    std::vector<BatchItem> v(it.size());
    for (int q = 0; q < 4; ++q) gr.vfirst[q] = gr.vcount[q] = 0;
    for (size_t k = 0; k < it.size(); ++k) {
      v[k] = it[k].second;
      const int q = gr.mvar[v[k].box];
      if (gr.vcount[q]++ == 0) gr.vfirst[q] = (int)k;
    }
    if ((int)v.size() > gr.cap) {
      if (gr.ditems) cudaFree(gr.ditems);
      gr.ditems = nullptr;
      gr.cap = 0;
      BCUDA(cudaMalloc(&gr.ditems, v.size() * sizeof(BatchItem)));
      gr.cap = (int)v.size();
    }
    gr.nitems = (int)v.size();
    if (!v.empty())
      BCUDA(cudaMemcpyAsync(gr.ditems, v.data(), v.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, b->st));
  }
  BCUDA(cudaStreamSynchronize(b->st));
  return FFE_OK;
}

// Tile height 16 exists for FP32 storage only (its rings do not fit in FP64).
template <typename R, int C> int prepare_kernels(int ty) {
  if constexpr (sizeof(R) == 4)
    if (ty == 16) return fused_batch_prepare_t16<R, C>();
  return fused_batch_prepare_t8<R, C>();
}
// True when every entry of the launch table still has the variant its items
// were built with (a member's B0 may have been set since).
template <typename R> bool variants_current(const ffe_batch::Group& gr, const BoxTable<R>& T) {
  for (int l = 0; l < gr.n; ++l)
    if (((T.b[l].has_b0 ? 2 : 0) | (T.b[l].absorb ? 1 : 0)) != gr.mvar[l]) return false;
  return true;
}

// Stage launches of a group: with tile height 8, one launch per variant
// present, each of a specialised kernel (the single-grid body of that
// variant) over the items of its variant; with tile height 16, or when a
// member's variant changed since the items were built, one launch of the
// kernel that switches per grid.  Persistent launches size the grid by the
// chosen kernel's residency.
template <typename R, int C>
int launch_batch_kernel(const ffe_batch* b, const ffe_batch::Group& gr, bool stage1, const BoxTable<R>& T) {
  auto grid_of = [&](int n, int per_sm) { return b->persistent ? std::max(1, std::min(n, per_sm * b->sms)) : n; };
  auto generic = [&](const BatchItem* it, int n) -> int {
    if (n <= 0) return 0;
    if constexpr (sizeof(R) == 4)
      if (b->ty == 16) return launch_fused_batch_t16<R, C>(stage1, it, n, T, grid_of(n, b->blocks_per_sm), b->st);
    return launch_fused_batch_t8<R, C>(stage1, it, n, T, grid_of(n, b->blocks_per_sm), b->st);
  };
  if (b->ty != 8 || !variants_current(gr, T)) return generic(gr.ditems, gr.nitems);
  for (int v = 0; v < 4; ++v) {
    const int n = gr.vcount[v];
    if (n <= 0) continue;
    const BatchItem* it = gr.ditems + gr.vfirst[v];
    const int rc = b->spec_bps[v] > 0
                       ? launch_fused_batch_spec_t8<R, C>(stage1, v, it, n, T, grid_of(n, b->spec_bps[v]), b->st)
                       : generic(it, n);
    if (rc) return rc;
  }
  return 0;
}

template <typename R, int C> void prepare_spec(ffe_batch* b) {
  for (int v = 0; v < 4; ++v) b->spec_bps[v] = fused_batch_prepare_spec_t8<R, C>(v);
}

int prepare(ffe_batch* b) {
  int n = 0;
  if (b->precision == FFE_FP64) n = b->ty == 8 ? prepare_kernels<double, 0>(8) : 0;
  else if (b->precision == FFE_FP32C) n = prepare_kernels<float, 1>(b->ty);
  else n = prepare_kernels<float, 0>(b->ty);
  if (n <= 0) return bfail(FFE_ECUDA, "batched stage kernel: cannot raise the shared-memory limit");
  b->blocks_per_sm = n;
  if (b->precision == FFE_FP64) prepare_spec<double, 0>(b);
  else if (b->precision == FFE_FP32C) prepare_spec<float, 1>(b);
  else prepare_spec<float, 0>(b);
  return FFE_OK;
}

template <typename R> BoxTable<R>* host_table(ffe_batch* b, int n, int s, int gi) {
  const size_t k = ((size_t)n * 3 + s) * b->groups.size() + gi;
  return reinterpret_cast<BoxTable<R>*>(b->tabs.data()) + k;
}

// Fill the launch tables for steps [n0, n0 + cn) of this call.
template <typename R, int C>
void fill_tables(ffe_batch* b, const std::vector<int>& cur0, const int32_t* step0, int n0, int cn) {
  const int np = (int)b->psr.size(), nm = (int)b->m.size();
  b->tabs.assign((size_t)cn * 3 * b->groups.size() * sizeof(BoxTable<R>), 0);
  FixParams<R>* ftab = (FixParams<R>*)b->hfixtab;
  const int ti = tile_index(b->ty);
  for (int gi = 0; gi < (int)b->groups.size(); ++gi) {
    const auto& gr = b->groups[gi];
    for (int l = 0; l < gr.n; ++l) {
      const int i = gr.first + l;
      ffe_t h = b->m[i];
      const Absorb<R> ab = absorb_consts<R>(h);
      const R ct = clean_tiny<R>(h);
      const bool uni = h->d.setup == FFE_SETUP_UNIFORM;
      const int pi = (int)(std::find(b->psr.begin(), b->psr.end(), i) - b->psr.begin());
      for (int n = 0; n < cn; ++n) {
        const int ts = (step0 ? step0[i] : 0) + n0 + n;
        const int A = (cur0[i] + n0 + n) % 3, B = (A + 1) % 3, Cs = (A + 2) % 3;
        const int ins[3] = {A, B, Cs}, outs[3] = {B, Cs, B};
        UniformBC<R> ub{};
        if (uni) ub = uniform_consts<R>(h, ts);
        PsrBC<R> q{};
        if (pi < np) q = psr_consts<R>(h, ts);
        for (int s = 0; s < 3; ++s) {
          double c[3];
          stage_coeffs<R>(s, c);
          const bool incr = C && std::fabs(c[0] + c[1] - 1.0) < 1e-6;
          BatchBox<R>& e = host_table<R>(b, n, s, gi)->b[l];
          Params<R>& P = e.P;
          P.g = h->g;
          P.p = h->p;
          P.ab = ab;
          P.cc = R(h->d.cc);
          P.c1 = R(c[0]);
          P.c2 = R(c[1]);
          P.c3 = R(c[2]);
          P.ct = ct;
          P.incr = incr ? 1 : 0;
          P.kz = b->kz_of[i];
          for (int k = 0; k < 3; ++k) P.b0[k] = (const R*)h->b0[k];
          P.in0 = (const R*)h->set[ins[s]][0];
          P.en0 = (const R*)h->set[A][0];
          P.out0 = (R*)h->set[outs[s]][0];
          P.fs = (const R*)h->set[0][1] - (const R*)h->set[0][0];
          P.err = b->derr;
          P.ubc = uni ? 1 : 0;
          P.ub = ub;
          e.mi = b->dmaps + (((size_t)ti * nm + i) * 3 + ins[s]) * 12;
          e.me = b->dmaps + (((size_t)ti * nm + i) * 3 + A) * 12 + 6;
          e.has_b0 = h->has_b0 ? 1 : 0;
          e.absorb = h->p.bnd[0] == 2 ? 1 : 0;
          if (pi < np) {
            FixParams<R>& F = ftab[((size_t)n * 3 + s) * np + pi];
            memset(&F, 0, sizeof F);
            F.g = h->g;
            F.p = h->p;
            F.ab = ab;
            F.q = q;
            F.cc = P.cc;
            F.c1 = P.c1;
            F.c2 = P.c2;
            F.c3 = P.c3;
            F.ct = ct;
            F.incr = P.incr;
            int u[6];
            psr_fix_box(h->g, q.i_lo, q.i_hi, q.j_lo, q.j_hi, q.k_lo, q.k_hi, u);
            F.ui = u[0]; F.uj = u[1]; F.uk = u[2]; F.ux = u[3]; F.uy = u[4]; F.uz = u[5];
            for (int k = 0; k < 6; ++k) {
              F.in[k] = P.in0 + k * P.fs;
              F.en[k] = P.en0 + k * P.fs;
              F.out[k] = P.out0 + k * P.fs;
            }
            for (int k = 0; k < 3; ++k) F.b0[k] = P.b0[k];
            F.s1 = (R*)h->box;
            F.s2 = (R*)h->box + psr_fix_elems<R>(h);
            F.has_b0 = e.has_b0;
            F.absorb = e.absorb;
          }
        }
      }
    }
  }
}

// All launches of stage s of step n of the current chunk.
template <typename R, int C>
int launch_stage(ffe_batch* b, int n, int s) {
  const int np = (int)b->psr.size();
  for (int gi = 0; gi < (int)b->groups.size(); ++gi) {
    const auto& gr = b->groups[gi];
    const BoxTable<R>& T = *host_table<R>(b, n, s, gi);
    if (launch_batch_kernel<R, C>(b, gr, s == 0, T)) return bfail(FFE_ECUDA, "batched stage launch");
    if (gr.nghost) launch_uniform_ghosts_batch<R>(gr.dghost, gr.nghost, T, b->st);
  }
  if (b->nfix)
    launch_fix_batch<R, C>(s == 0, b->dfix, b->nfix,
                           (const FixParams<R>*)b->dfixtab + ((size_t)n * 3 + s) * np, b->st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bfail(FFE_ECUDA, "batched launch: %s", cudaGetErrorString(e));
  return FFE_OK;
}

// Capture the cn steps of the filled tables; instantiate, or update the
// cached graph of the same length in place.
template <typename R, int C>
int capture(ffe_batch* b, int cn, cudaGraphExec_t* out) {
  BCUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  int rc = FFE_OK;
  for (int n = 0; n < cn && rc == FFE_OK; ++n)
    for (int s = 0; s < 3 && rc == FFE_OK; ++s) rc = launch_stage<R, C>(b, n, s);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->st, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bfail(FFE_ECUDA, "graph capture: %s", cudaGetErrorString(e));
  for (auto& c : b->graphs)
    if (c.steps == cn) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(c.exec, g, &info) == cudaSuccess) {
        cudaGraphDestroy(g);
        *out = c.exec;
        return FFE_OK;
      }
      cudaGetLastError();
      cudaGraphExecDestroy(c.exec);
      c = b->graphs.back();
      b->graphs.pop_back();
      break;
    }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(FFE_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
  b->graphs.push_back({cn, *out});
  return FFE_OK;
}

int ensure_fix_tables(ffe_batch* b, int steps) {
  const int np = (int)b->psr.size();
  if (!np || steps <= b->fix_steps) return FFE_OK;
  const size_t fb = (size_t)steps * 3 * np * fix_entry_bytes(b->precision);
  BCUDA(cudaStreamSynchronize(b->st));
  drop_graphs(b);
  if (b->dfixtab) cudaFree(b->dfixtab);
  if (b->hfixtab) cudaFreeHost(b->hfixtab);
  b->dfixtab = b->hfixtab = nullptr;
  b->fix_steps = 0;
  BCUDA(cudaMalloc(&b->dfixtab, fb));
  BCUDA(cudaMallocHost(&b->hfixtab, fb));
  b->fix_steps = steps;
  return FFE_OK;
}

// Order the batch stream after each member's queued work; returns the
// members' current sets.
template <typename R>
int join_members(ffe_batch* b, std::vector<int>& cur0) {
  int rc;
  const int nm = (int)b->m.size();
  cur0.resize(nm);
  for (int i = 0; i < nm; ++i) {
    ffe_t h = b->m[i];
    if ((rc = sync_ghosts<R>(h))) return rc;
    BCUDA(cudaEventRecord(b->ev, h->st));
    BCUDA(cudaStreamWaitEvent(b->st, b->ev, 0));
    cur0[i] = h->cur;
  }
  return FFE_OK;
}

template <typename R, int C>
int batch_run(ffe_batch* b, int nsteps, const int32_t* step0) {
  int rc;
  std::vector<int> cur0;
  if ((rc = join_members<R>(b, cur0))) return rc;
  if ((rc = ensure_fix_tables(b, std::min(nsteps, kChunk)))) return rc;
  const int np = (int)b->psr.size();
  for (int n0 = 0; n0 < nsteps; n0 += kChunk) {
    const int cn = std::min(kChunk, nsteps - n0);
    BCUDA(cudaEventSynchronize(b->copied));  // the previous chunk's fix-up table has left the staging buffer
    fill_tables<R, C>(b, cur0, step0, n0, cn);
    if (np) {
      BCUDA(cudaMemcpyAsync(b->dfixtab, b->hfixtab, (size_t)cn * 3 * np * sizeof(FixParams<R>),
                            cudaMemcpyHostToDevice, b->st));
      BCUDA(cudaEventRecord(b->copied, b->st));
    }
    cudaGraphExec_t ex = nullptr;
    if ((rc = capture<R, C>(b, cn, &ex))) return rc;
    BCUDA(cudaGraphLaunch(ex, b->st));
  }
  BCUDA(cudaEventRecord(b->ev, b->st));
  for (int i = 0; i < (int)b->m.size(); ++i) {
    ffe_t h = b->m[i];
    h->cur = (cur0[i] + nsteps) % 3;
    BCUDA(cudaStreamWaitEvent(h->st, b->ev, 0));
  }
  return FFE_OK;
}

// Time the stage launches of all groups for the current tiling, in the form
// of stage 2 with the stage input equal to the step start (both the current
// set); the output is the set that stage 2 of the next step overwrites.
template <typename R, int C>
int time_stage(ffe_batch* b, int reps, double* ms) {
  int rc;
  std::vector<int> cur0;
  if ((rc = join_members<R>(b, cur0))) return rc;
  if ((rc = ensure_fix_tables(b, 1))) return rc;
  BCUDA(cudaEventSynchronize(b->copied));
  fill_tables<R, C>(b, cur0, nullptr, 0, 1);
  for (int gi = 0; gi < (int)b->groups.size(); ++gi) {
    BoxTable<R>* T = host_table<R>(b, 0, 1, gi);
    for (int l = 0; l < b->groups[gi].n; ++l) {
      BatchBox<R>& e = T->b[l];
      const int A = cur0[b->groups[gi].first + l];
      e.P.in0 = (const R*)b->m[b->groups[gi].first + l]->set[A][0];
      e.mi = e.me - 6;
    }
  }
  cudaEvent_t t0, t1;
  BCUDA(cudaEventCreate(&t0));
  BCUDA(cudaEventCreate(&t1));
  float best = 1e30f;
  bool bad = false;
  for (int r = -1; r < reps && !bad; ++r) {  // r = -1: warm-up
    cudaEventRecord(t0, b->st);
    for (int gi = 0; gi < (int)b->groups.size(); ++gi) {
      const auto& gr = b->groups[gi];
      bad |= launch_batch_kernel<R, C>(b, gr, false, *host_table<R>(b, 0, 1, gi)) != 0;
    }
    cudaEventRecord(t1, b->st);
    bad |= cudaEventSynchronize(t1) != cudaSuccess || cudaGetLastError() != cudaSuccess;
    float t = 0;
    cudaEventElapsedTime(&t, t0, t1);
    if (r >= 0) best = std::min(best, t);
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (bad) return bfail(FFE_ECUDA, "autotune launch failed");
  *ms = best;
  int err = 0;
  BCUDA(cudaMemcpy(&err, b->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return bfail(FFE_ETIMEOUT, "a batched stage block timed out waiting for its plane copies");
  return FFE_OK;
}

#define BDISPATCH(b, FN, ...)                                \
  ((b)->precision == FFE_FP64    ? FN<double, 0>(__VA_ARGS__) \
   : (b)->precision == FFE_FP32C ? FN<float, 1>(__VA_ARGS__)  \
                                 : FN<float, 0>(__VA_ARGS__))

int set_tiling(ffe_batch* b, int ty, int kz, int persistent) {
  if (ty != 8 && ty != 16) return bfail(FFE_EINVAL, "tile height must be 8 or 16");
  if (ty == 16 && b->precision == FFE_FP64) return bfail(FFE_EUNSUPPORTED, "tile height 16 needs FP32 storage");
  if (kz < 0) return bfail(FFE_EINVAL, "planes per block must be >= 0");
  BCUDA(cudaStreamSynchronize(b->st));
  drop_graphs(b);
  b->ty = ty;
  b->kz = kz;
  b->persistent = persistent ? 1 : 0;
  int rc;
  if ((rc = prepare(b))) return rc;
  return build_items(b);
}

void free_batch(ffe_batch* b) {
  if (b->st) cudaStreamSynchronize(b->st);
  drop_graphs(b);
  for (auto& gr : b->groups) {
    if (gr.ditems) cudaFree(gr.ditems);
    if (gr.dghost) cudaFree(gr.dghost);
  }
  if (b->dfix) cudaFree(b->dfix);
  if (b->dfixtab) cudaFree(b->dfixtab);
  if (b->hfixtab) cudaFreeHost(b->hfixtab);
  if (b->dmaps) cudaFree(b->dmaps);
  if (b->derr) cudaFree(b->derr);
  if (b->ev) cudaEventDestroy(b->ev);
  if (b->copied) cudaEventDestroy(b->copied);
  if (b->own_stream && b->st) cudaStreamDestroy(b->st);
  delete b;
}

int check_batch(ffe_batch_t b) {
  if (!b) return bfail(FFE_EINVAL, "null batch");
  BCUDA(cudaSetDevice(b->device));
  return FFE_OK;
}

}  // namespace

extern "C" {

int ffe_batch_create(ffe_batch_t* out, const ffe_t* members, int32_t n, void* stream) {
  if (!out || !members || n <= 0) return bfail(FFE_EINVAL, "ffe_batch_create: need n > 0 members");
  *out = nullptr;
  int dev = 0;
  BCUDA(cudaGetDevice(&dev));
  const int prec = members[0] ? members[0]->d.precision : -1;
  for (int i = 0; i < n; ++i) {
    ffe_t h = members[i];
    if (!h) return bfail(FFE_EINVAL, "member %d is null", i);
    for (int j = 0; j < i; ++j)
      if (members[j] == h) return bfail(FFE_EINVAL, "member %d appears twice", i);
    if (h->device != dev) return bfail(FFE_EINVAL, "member %d lives on device %d, not %d", i, h->device, dev);
    if (h->d.precision != prec) return bfail(FFE_EINVAL, "members must share one precision");
    if (prec == FFE_FP32CD) return bfail(FFE_EUNSUPPORTED, "batches run FP64, FP32 or FP32C");
    if (h->d.path == FFE_PATH_STAGED || h->d.path == FFE_PATH_FUSED_EXACT || !fused_possible(h))
      return bfail(FFE_EUNSUPPORTED, "member %d cannot take the fused path (setup %d, path %d)", i, h->d.setup,
                   h->d.path);
  }
  ffe_batch* b = new (std::nothrow) ffe_batch();
  if (!b) return bfail(FFE_ENOMEM, "host allocation failed");
  b->device = dev;
  b->precision = prec;
  b->m.assign(members, members + n);
  for (int f = 0; f < n; f += BATCH_MAX) {
    ffe_batch::Group gr;
    gr.first = f;
    gr.n = std::min(BATCH_MAX, n - f);
    b->groups.push_back(gr);
  }
  int rc = FFE_OK;
  auto cu = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && rc == FFE_OK) rc = bfail(FFE_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    return rc == FFE_OK;
  };
  if (stream) {
    b->st = (cudaStream_t)stream;
  } else if (cu(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking), "cudaStreamCreate")) {
    b->own_stream = true;
  }
  cudaDeviceProp prop;
  if (rc == FFE_OK && cu(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties"))
    b->sms = prop.multiProcessorCount;
  if (rc == FFE_OK) cu(cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming), "cudaEventCreate");
  if (rc == FFE_OK) cu(cudaEventCreateWithFlags(&b->copied, cudaEventDisableTiming), "cudaEventCreate");
  if (rc == FFE_OK && cu(cudaMalloc(&b->derr, 256), "cudaMalloc")) cu(cudaMemset(b->derr, 0, 256), "cudaMemset");
  // tensor maps of every member's sets for both tile heights
  if (rc == FFE_OK) {
    std::vector<CUtensorMap> maps((size_t)2 * n * 3 * 12);
    for (int t = 0; t < 2 && rc == FFE_OK; ++t)
      for (int i = 0; i < n && rc == FFE_OK; ++i)
        for (int s = 0; s < 3 && rc == FFE_OK; ++s)
          for (int c = 0; c < 6 && rc == FFE_OK; ++c) {
            CUtensorMap* e = &maps[(((size_t)t * n + i) * 3 + s) * 12];
            ffe_t h = members[i];
            if (make_stage_maps(&e[c], &e[6 + c], h->set[s][c], h->g, (int)h->es, t ? 16 : 8))
              rc = bfail(FFE_EUNSUPPORTED, "cannot encode TMA tensor maps for member %d", i);
          }
    if (rc == FFE_OK && cu(cudaMalloc(&b->dmaps, maps.size() * sizeof(CUtensorMap)), "cudaMalloc"))
      cu(cudaMemcpy(b->dmaps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  // pulsar fix-up items (all members) and user_uniform ghost-plane items (per group)
  if (rc == FFE_OK) {
    std::vector<FixItem> fx;
    for (auto& gr : b->groups) {
      std::vector<FixItem> gh;
      for (int l = 0; l < gr.n; ++l) {
        ffe_t h = members[gr.first + l];
        if (h->d.setup == FFE_SETUP_PSR) {
          const PsrBC<float> q = psr_consts<float>(h, 0);  // the box does not depend on the step
          if (q.bx > 0 && q.by > 0 && q.bz > 0) {
            const int pi = (int)b->psr.size();
            b->psr.push_back(gr.first + l);
            int u[6];
            psr_fix_box(h->g, q.i_lo, q.i_hi, q.j_lo, q.j_hi, q.k_lo, q.k_hi, u);
            for (int z = 0; z < u[5]; ++z)
              for (int y = 0; y < (u[4] + 7) / 8; ++y)
                for (int x = 0; x < (u[3] + 31) / 32; ++x) fx.push_back(FixItem{pi, x, y, z});
          }
        }
        if (h->d.setup == FFE_SETUP_UNIFORM) {
          // ghost planes with z_glob <= 0 or >= gsz (interior planes take the BC inside the stage kernel)
          const int sz = h->g.sz, z0 = h->p.z0, gsz = h->p.gsz;
          for (int k = -NG; k < sz + NG; ++k) {
            if (k >= 0 && k < sz) continue;
            if (!(k + z0 <= 0 || k + z0 >= gsz)) continue;
            for (int y = 0; y < (h->g.sy + 2 * NG + 7) / 8; ++y)
              for (int x = 0; x < (h->g.sx + 2 * NG + 31) / 32; ++x) gh.push_back(FixItem{l, x, y, k});
          }
        }
      }
      gr.nghost = (int)gh.size();
      if (rc == FFE_OK && !gh.empty() && cu(cudaMalloc(&gr.dghost, gh.size() * sizeof(FixItem)), "cudaMalloc"))
        cu(cudaMemcpy(gr.dghost, gh.data(), gh.size() * sizeof(FixItem), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    b->nfix = (int)fx.size();
    if (rc == FFE_OK && !fx.empty() && cu(cudaMalloc(&b->dfix, fx.size() * sizeof(FixItem)), "cudaMalloc"))
      cu(cudaMemcpy(b->dfix, fx.data(), fx.size() * sizeof(FixItem), cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  if (rc == FFE_OK) cu(cudaEventRecord(b->copied, b->st), "cudaEventRecord");
  if (rc == FFE_OK) rc = set_tiling(b, 8, 0, 0);
  if (rc != FFE_OK) {
    free_batch(b);
    return rc;
  }
  *out = b;
  return FFE_OK;
}

int ffe_batch_destroy(ffe_batch_t b) {
  if (!b) return FFE_OK;
  cudaSetDevice(b->device);
  free_batch(b);
  return FFE_OK;
}

int ffe_batch_step(ffe_batch_t b, int32_t nsteps, const int32_t* step0) {
  int rc;
  if ((rc = check_batch(b))) return rc;
  if (nsteps < 0) return bfail(FFE_EINVAL, "nsteps < 0");
  if (nsteps == 0) return FFE_OK;
  return BDISPATCH(b, batch_run, b, nsteps, step0);
}

int ffe_batch_set_tiling(ffe_batch_t b, int32_t tile_y, int32_t planes, int32_t persistent) {
  int rc;
  if ((rc = check_batch(b))) return rc;
  return set_tiling(b, tile_y, planes, persistent);
}

int ffe_batch_get_tiling(ffe_batch_t b, int32_t* tile_y, int32_t* planes, int32_t* persistent) {
  if (!b || !tile_y || !planes || !persistent) return bfail(FFE_EINVAL, "null argument");
  *tile_y = b->ty;
  *planes = b->kz;
  *persistent = b->persistent;
  return FFE_OK;
}

int ffe_batch_autotune(ffe_batch_t b, int32_t reps, double* best_ms) {
  int rc;
  if ((rc = check_batch(b))) return rc;
  if (reps < 1) return bfail(FFE_EINVAL, "reps must be >= 1");
  const int tys[2] = {8, 16}, kzs[5] = {0, 8, 16, 32, 64};
  double best = 1e300;
  int bt = 8, bk = 0, bp = 0;
  for (int t : tys) {
    if (t == 16 && b->precision == FFE_FP64) continue;
    for (int k : kzs)
      for (int p = 0; p < 2; ++p) {
        if ((rc = set_tiling(b, t, k, p))) return rc;
        double ms = 0;
        if ((rc = BDISPATCH(b, time_stage, b, reps, &ms))) return rc;
        if (ms < best) {
          best = ms;
          bt = t;
          bk = k;
          bp = p;
        }
      }
  }
  if ((rc = set_tiling(b, bt, bk, bp))) return rc;
  if (best_ms) *best_ms = best;
  return FFE_OK;
}

int ffe_batch_launches(ffe_batch_t b, int32_t* per_step) {
  if (!b || !per_step) return bfail(FFE_EINVAL, "null argument");
  int ng = 0, ns = 0;
  for (auto& gr : b->groups) {
    ng += gr.nghost ? 1 : 0;
    int nv = 0;  // stage launches of the group: one per variant present at tile height 8
    for (int v = 0; v < 4; ++v) nv += gr.vcount[v] > 0 ? 1 : 0;
    ns += b->ty == 8 && nv > 0 ? nv : 1;
  }
  *per_step = 3 * (ns + ng + (b->nfix ? 3 : 0));
  return FFE_OK;
}

int ffe_batch_synchronize(ffe_batch_t b) {
  int rc;
  if ((rc = check_batch(b))) return rc;
  BCUDA(cudaStreamSynchronize(b->st));
  int e = 0;
  BCUDA(cudaMemcpyAsync(&e, b->derr, sizeof(int), cudaMemcpyDeviceToHost, b->st));
  BCUDA(cudaStreamSynchronize(b->st));
  if (e) {
    BCUDA(cudaMemsetAsync(b->derr, 0, sizeof(int), b->st));
    return bfail(FFE_ETIMEOUT, "a batched stage block timed out waiting for its plane copies");
  }
  return FFE_OK;
}

}  // extern "C"
