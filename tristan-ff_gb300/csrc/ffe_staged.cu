// ffe_staged.cu — one kernel per reference procedure, reference order.
//
// These kernels reproduce the reference's procedures one to one: computeRho,
// rk3Push, rk3Update (+ absorbing shell), cleanEpar (out of place through dE),
// the ghost fill that replaces exchangeFields, and the shipped user boundary
// conditions and initial fields.  This translation unit is compiled with
// -fmad=false: no multiply-add is contracted, so with correctly rounded
// division and square root the results equal the CPU restatement bit for bit
// (transcendentals aside: tanh, exp of the user boundary conditions).
#include "ffe_kernels.h"
#include "ffe_physics.cuh"
#include "ffe_psr.cuh"

namespace ffe {

namespace {

// Accessor over global arrays around linear index s.
template <typename R>
struct GAcc {
  const R* f[9];
  const R* rhoa;
  long long s, dj, dk;
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    return f[c][s + di + djj * dj + dkk * dk];
  }
  __device__ __forceinline__ R rho(int di, int djj, int dkk) const { return rhoa[s + di + djj * dj + dkk * dk]; }
};

inline dim3 grid_for(int nx, int ny, int nz, dim3 b) {
  return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y, nz);
}

// ---- computeRho over [-1, s+1]^3 (field_solver.F90:54-62) -----------------
template <typename R>
__global__ void k_rho(Geom g, const R* __restrict__ ex, const R* __restrict__ ey, const R* __restrict__ ez,
                      R* __restrict__ rho) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
  const int k = blockIdx.z - 1;
  if (i > g.sx + 1 || j > g.sy + 1) return;
  const long long s = g.idx(i, j, k);
  rho[s] = ((ex[s] - ex[s - 1]) + (ey[s] - ey[s - g.px])) + (ez[s] - ez[s - g.plane]);
}

// ---- rk3Push over the interior (field_solver.F90:78-165) ------------------
template <typename R, int C, bool B0>
__global__ void k_push(Geom g, R cc, CEB<R> eb, CEB<R> b0, const R* __restrict__ rho, EB<R> d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  GAcc<R> a;
  for (int c = 0; c < 6; ++c) a.f[c] = eb.c[c];
  for (int c = 0; c < 3; ++c) a.f[6 + c] = b0.c[c];
  a.rhoa = rho;
  a.s = g.idx(i, j, k);
  a.dj = g.px;
  a.dk = g.plane;
  R out[6];
  push_cell<R, C, B0>(a, cc, out);
  for (int c = 0; c < 6; ++c) d.c[c][a.s] = out[c];
}

// ---- rk3Update over the interior (field_solver.F90:180-268) ---------------
template <typename R, int C, bool ABS>
__global__ void k_update(Geom g, Phys p, Absorb<R> ab, R c1, R c2, R c3, int incr, EB<R> f, CEB<R> fn, CEB<R> df) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  const long long s = g.idx(i, j, k);
  R v[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) v[c] = combine<R, C>(c1, c2, c3, fn.c[c][s], f.c[c][s], df.c[c][s], incr != 0);
  if (ABS) absorb_cell<R>(ab, i + p.x0, shell_jg(ab, i, j, p.y0), k + p.z0, v);
#pragma unroll
  for (int c = 0; c < 6; ++c) f.c[c][s] = v[c];
}

// ---- cleanEpar into dE, then dE -> E over the interior (:284-334) ---------
template <typename R, int C>
__global__ void k_clean(Geom g, CEB<R> eb, R* __restrict__ dex, R* __restrict__ dey, R* __restrict__ dez, R ct) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  GAcc<R> a;
  for (int c = 0; c < 6; ++c) a.f[c] = eb.c[c];
  a.s = g.idx(i, j, k);
  a.dj = g.px;
  a.dk = g.plane;
  R e[3];
  clean_cell<R, C>(a, e, ct);
  dex[a.s] = e[0];
  dey[a.s] = e[1];
  dez[a.s] = e[2];
}

template <typename R>
__global__ void k_copy_e(Geom g, const R* __restrict__ dex, const R* __restrict__ dey, const R* __restrict__ dez,
                         R* __restrict__ ex, R* __restrict__ ey, R* __restrict__ ez) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  const long long s = g.idx(i, j, k);
  ex[s] = dex[s];
  ey[s] = dey[s];
  ez[s] = dez[s];
}

// ---- ghost fill: the single-meshblock form of exchangeFields --------------
// A ghost is written iff every axis on which it lies outside is periodic; it
// takes the value of the interior cell it wraps to on those axes.  Every
// source is an interior cell, so the order of the writes does not matter.
// Work items, one block each: the rows of the z-slabs (planes k < 0 and
// k >= sz, every row j of the padded plane), the rows of the y-slabs (rows
// j < 0 and j >= sy of every interior plane), each copied as a whole row by
// the block's threads (coalesced), then blocks of x-slab rows: one thread per
// interior row (j, k) writes its 2 x NG ghost cells (two 16-byte pieces at
// the row's ends).  32-bit index arithmetic, no divisions by runtime values
// beyond one per block.
template <typename R>
__global__ void k_fill(Geom g, int per_x, int per_y, int per_z, int nf, EB<R> f6, R* b0x, R* b0y, R* b0z,
                       int zrows, int yrows, int xslabs) {
  R* f[9] = {f6.c[0], f6.c[1], f6.c[2], f6.c[3], f6.c[4], f6.c[5], b0x, b0y, b0z};
  const int nxg = g.sx + 2 * NG, nyg = g.sy + 2 * NG;
  const int b = blockIdx.x;
  if (b < zrows + yrows) {
    int j, k;
    if (b < zrows) {  // z-slab row: plane kk of the 2 NG ghost planes, row j of the padded plane
      const int kk = b / nyg;
      j = b - kk * nyg - NG;
      k = kk < NG ? kk - NG : g.sz + (kk - NG);
    } else {  // y-slab row: ghost row jj of interior plane k
      const int e = b - zrows, jj = e % (2 * NG);
      k = e / (2 * NG);
      j = jj < NG ? jj - NG : g.sy + (jj - NG);
    }
    int sj = j, sk = k;
    if (j < 0 || j >= g.sy) { if (!per_y) return; sj = j < 0 ? j + g.sy : j - g.sy; }
    if (k < 0 || k >= g.sz) { if (!per_z) return; sk = k < 0 ? k + g.sz : k - g.sz; }
    const long long dst = g.idx(-NG, j, k), src = g.idx(-NG, sj, sk);
    for (int t = threadIdx.x; t < nxg; t += blockDim.x) {
      const int i = t - NG;
      int si = i;
      if (i < 0 || i >= g.sx) { if (!per_x) continue; si = i < 0 ? i + g.sx : i - g.sx; }
      const long long d = dst + t, s = src + (si + NG);
      R v[9];  // every load before any store: the loads stay in flight together
#pragma unroll
      for (int c = 0; c < 9; ++c)
        if (c < nf) v[c] = f[c][s];
#pragma unroll
      for (int c = 0; c < 9; ++c)
        if (c < nf) f[c][d] = v[c];
    }
    return;
  }
  if (!per_x || !xslabs) return;
  // x-slab rows
  const int r = (b - zrows - yrows) * blockDim.x + threadIdx.x;
  if (r >= g.sy * g.sz) return;
  const int k = r / g.sy, j = r - k * g.sy;
  const long long row = g.idx(0, j, k);
  R lo[9][NG], hi[9][NG];  // every load before any store
#pragma unroll
  for (int c = 0; c < 9; ++c)
    if (c < nf) {
      const R* q = f[c] + row;
#pragma unroll
      for (int a = 0; a < NG; ++a) {
        lo[c][a] = q[g.sx - NG + a];  // for ghost i = a - NG (<- i + sx)
        hi[c][a] = q[a];              // for ghost i = sx + a (<- i)
      }
    }
#pragma unroll
  for (int c = 0; c < 9; ++c)
    if (c < nf) {
      R* q = f[c] + row;
#pragma unroll
      for (int a = 0; a < NG; ++a) {
        q[a - NG] = lo[c][a];
        q[g.sx + a] = hi[c][a];
      }
    }
}

// ---- user_psr boundary condition (user/user_psr.F90:72-332) ---------------
// Pass 1: new values of all six components for the cells of the bounding box
// that lie inside r < 2R, written to a compact box buffer (6 * box cells).
template <typename R>
__global__ void k_psr_bc(Geom g, Phys p, PsrBC<R> q, CEB<R> f, R* __restrict__ box) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  const int bj = blockIdx.y * blockDim.y + threadIdx.y;
  const int bk = blockIdx.z;
  if (bi >= q.bx || bj >= q.by) return;
  const int i = q.i_lo + bi, j = q.j_lo + bj, k = q.k_lo + bk;
  if (!psr_inside(q, p, i, j, k)) return;
  GAcc<R> a;
  for (int c = 0; c < 6; ++c) a.f[c] = f.c[c];
  a.s = g.idx(i, j, k);
  a.dj = g.px;
  a.dk = g.plane;
  R o[6];
  psr_cell(q, p, a, i, j, k, o);
  const long long nbox = (long long)q.bx * q.by * q.bz;
  const long long ob = bi + (long long)q.bx * (bj + (long long)q.by * bk);
#pragma unroll
  for (int c = 0; c < 6; ++c) box[c * nbox + ob] = o[c];
}

// Pass 2: copy the box values back for cells inside r < 2R (:305-325).
template <typename R>
__global__ void k_psr_copy(Geom g, Phys p, PsrBC<R> q, EB<R> f, const R* __restrict__ box) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  const int bj = blockIdx.y * blockDim.y + threadIdx.y;
  const int bk = blockIdx.z;
  if (bi >= q.bx || bj >= q.by) return;
  const int i = q.i_lo + bi, j = q.j_lo + bj, k = q.k_lo + bk;
  if (!psr_inside(q, p, i, j, k)) return;
  const long long s = g.idx(i, j, k);
  const long long nbox = (long long)q.bx * q.by * q.bz;
  const long long o = bi + (long long)q.bx * (bj + (long long)q.by * bk);
#pragma unroll
  for (int c = 0; c < 6; ++c) f.c[c][s] = box[c * nbox + o];
}

// ---- user_uniform boundary condition (user/user_uniform.F90:91-145) -------
// Planes with z_glob <= 0 and z_glob >= gsz, all i, j including ghosts.
template <typename R>
__global__ void k_uniform_bc(Geom g, Phys p, UniformBC<R> u, EB<R> f, int k_first, int nk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x - NG;
  const int j = blockIdx.y * blockDim.y + threadIdx.y - NG;
  const int k = k_first + (int)blockIdx.z;
  if (i >= g.sx + NG || j >= g.sy + NG || (int)blockIdx.z >= nk) return;
  const long long s = g.idx(i, j, k);
  uniform_bc_apply(u, p, i, j, k, f.c[0][s], f.c[1][s], f.c[5][s]);
}

// ---- user_loop boundary condition (user/user_loop.F90:115-163) ------------
template <typename R>
__global__ void k_loop_bc(Geom g, Phys p, EB<R> f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x - NG;
  const int j = blockIdx.y * blockDim.y + threadIdx.y - NG;
  const int kk = blockIdx.z;  // 0..2*NG-1: ghost planes below, then above
  if (i >= g.sx + NG || j >= g.sy + NG) return;
  const int k = kk < NG ? kk - NG : g.sz + (kk - NG);
  const R zg = R(k + p.z0);
  const long long s = g.idx(i, j, k);
  int src = -1;
  if (zg < R(0)) src = 0;
  if (zg >= R(p.gsz)) src = g.sz - 1;
  if (src < 0) return;
  const long long t = g.idx(i, j, src);
  f.c[0][s] = f.c[0][t];
  f.c[1][s] = f.c[1][t];
  f.c[5][s] = f.c[5][t];
}

// ---- userInitialize ---------------------------------------------------------
template <typename R>
__global__ void k_psr_init(Geom g, Phys p, PsrBC<R> q, EB<R> f) {  // user_psr.F90:47-67
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  const long long s = g.idx(i, j, k);
  const R ig = R(i + p.x0), jg = R(j + p.y0), kg = R(k + p.z0), h = R(0.5);
  R b0, b1, b2;
  psr_dipole(q, ig, jg + h, kg + h, b0, b1, b2);
  f.c[3][s] = b0;
  psr_dipole(q, ig + h, jg, kg + h, b0, b1, b2);
  f.c[4][s] = b1;
  psr_dipole(q, ig + h, jg + h, kg, b0, b1, b2);
  f.c[5][s] = b2;
}

template <typename R>
__global__ void k_uniform_init(Geom g, Phys p, UniformBC<R> u, R* bz, R* b0z) {  // user_uniform.F90:55-68
  const int i = blockIdx.x * blockDim.x + threadIdx.x - NG;
  const int j = blockIdx.y * blockDim.y + threadIdx.y - NG;
  const int k = (int)blockIdx.z - NG;
  if (i >= g.sx + NG || j >= g.sy + NG) return;
  const R xg = R(i + p.x0), yg = R(j + p.y0), h = R(0.5);
  const R rx = (xg + h) - u.xc, ry = (yg + h) - u.yc;
  const R rr = sqrt((rx * rx + ry * ry) + tiny<R>());
  const long long s = g.idx(i, j, k);
  const R v = u.bnorm / (R(1.0) + (rr / u.r0));
  bz[s] = v;
  b0z[s] = v;
}

template <typename R>
struct LoopInit { R xc, yc1, yc2, zc, bnorm; };

template <typename R>
__global__ void k_loop_init(Geom g, Phys p, LoopInit<R> L, EB<R> f, EB<R> f0) {  // user_loop.F90:58-92
  const int i = blockIdx.x * blockDim.x + threadIdx.x - NG;
  const int j = blockIdx.y * blockDim.y + threadIdx.y - NG;
  const int k = (int)blockIdx.z - NG;
  if (i >= g.sx + NG || j >= g.sy + NG) return;
  const R xg = R(i + p.x0), yg = R(j + p.y0), zg = R(k + p.z0), h = R(0.5);
  const long long s = g.idx(i, j, k);
  R rx, ry1, ry2, rz, rr1, rr2, v;
  rx = xg - L.xc; ry1 = (yg + h) - L.yc1; ry2 = (yg + h) - L.yc2; rz = (zg + h) - L.zc;
  rr1 = sqrt((rx * rx + ry1 * ry1) + rz * rz);
  rr2 = sqrt((rx * rx + ry2 * ry2) + rz * rz);
  v = L.bnorm * (rx / ((rr1 * rr1) * rr1) - rx / ((rr2 * rr2) * rr2));
  f.c[3][s] = v; f0.c[0][s] = v;
  rx = (xg + h) - L.xc; ry1 = yg - L.yc1; ry2 = yg - L.yc2; rz = (zg + h) - L.zc;
  rr1 = sqrt((rx * rx + ry1 * ry1) + rz * rz);
  rr2 = sqrt((rx * rx + ry2 * ry2) + rz * rz);
  v = L.bnorm * (ry1 / ((rr1 * rr1) * rr1) - ry2 / ((rr2 * rr2) * rr2));
  f.c[4][s] = v; f0.c[1][s] = v;
  rx = (xg + h) - L.xc; ry1 = (yg + h) - L.yc1; ry2 = (yg + h) - L.yc2; rz = zg - L.zc;
  rr1 = sqrt((rx * rx + ry1 * ry1) + rz * rz);
  rr2 = sqrt((rx * rx + ry2 * ry2) + rz * rz);
  v = L.bnorm * (rz / ((rr1 * rr1) * rr1) - rz / ((rr2 * rr2) * rr2));
  f.c[5][s] = v; f0.c[2][s] = v;
}

// ---- synthetic plane-wave workloads (not a reference setup) ---------------
// Each mode m: phase(x) = K.x + phi; dB(x) = -a sin(phase) u; dE(x) = -n x dB(x),
// with u the unit polarisation (host-computed from the discrete wavenumbers so
// that the discrete divergence of B vanishes) and n the propagation direction.
// Evaluated in double at every staggered point of every cell (ghosts included)
// and rounded once to R.
struct Mode { double K[3], phi, a, u[3], n[3]; };
constexpr int MAX_MODES = 64;
struct Modes { int n; double bg[3]; Mode m[MAX_MODES]; };

template <typename R>
__global__ void k_waves(Geom g, Phys p, const Modes* __restrict__ M, EB<R> f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x - NG;
  const int j = blockIdx.y * blockDim.y + threadIdx.y - NG;
  const int k = (int)blockIdx.z - NG;
  if (i >= g.sx + NG || j >= g.sy + NG) return;
  const double X = i + p.x0, Y = j + p.y0, Z = k + p.z0;
  // staggered positions: Ex Ey Ez Bx By Bz
  const double ox[6] = {0.5, 0, 0, 0, 0.5, 0.5}, oy[6] = {0, 0.5, 0, 0.5, 0, 0.5}, oz[6] = {0, 0, 0.5, 0.5, 0.5, 0};
  double v[6] = {0, 0, 0, M->bg[0], M->bg[1], M->bg[2]};
  for (int m = 0; m < M->n; ++m) {
    const Mode& q = M->m[m];
    for (int c = 0; c < 6; ++c) {
      const double s = sin(q.K[0] * (X + ox[c]) + q.K[1] * (Y + oy[c]) + q.K[2] * (Z + oz[c]) + q.phi);
      const double db[3] = {-q.a * s * q.u[0], -q.a * s * q.u[1], -q.a * s * q.u[2]};
      if (c < 3) {  // -n x dB, component c
        const double cr[3] = {q.n[1] * db[2] - q.n[2] * db[1], q.n[2] * db[0] - q.n[0] * db[2],
                              q.n[0] * db[1] - q.n[1] * db[0]};
        v[c] -= cr[c];
      } else {
        v[c] += db[c - 3];
      }
    }
  }
  const long long s = g.idx(i, j, k);
#pragma unroll
  for (int c = 0; c < 6; ++c) f.c[c][s] = (R)v[c];
}

// ---- finite check over the interior of E and B ------------------------------
template <typename R>
__global__ void k_finite(Geom g, CEB<R> f, int* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.sx || j >= g.sy) return;
  const long long s = g.idx(i, j, k);
  bool ok = true;
#pragma unroll
  for (int c = 0; c < 6; ++c) ok = ok && isfinite(f.c[c][s]);
  if (!ok) atomicOr(bad, 1);
}

const dim3 B2(32, 8, 1);

}  // namespace

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <typename R>
void launch_rho(const Geom& g, const R* ex, const R* ey, const R* ez, R* rho, cudaStream_t st) {
  k_rho<R><<<grid_for(g.sx + 3, g.sy + 3, g.sz + 3, B2), B2, 0, st>>>(g, ex, ey, ez, rho);
}

template <typename R, int C>
void launch_push(const Geom& g, R cc, const CEB<R>& eb, const CEB<R>& b0, bool has_b0, const R* rho, const EB<R>& d,
                 cudaStream_t st) {
  const dim3 gr = grid_for(g.sx, g.sy, g.sz, B2);
  if (has_b0) k_push<R, C, true><<<gr, B2, 0, st>>>(g, cc, eb, b0, rho, d);
  else k_push<R, C, false><<<gr, B2, 0, st>>>(g, cc, eb, b0, rho, d);
}

template <typename R, int C>
void launch_update(const Geom& g, const Phys& p, const Absorb<R>& ab, R c1, R c2, R c3, bool incr, const EB<R>& f,
                   const CEB<R>& fn, const CEB<R>& df, cudaStream_t st) {
  const dim3 gr = grid_for(g.sx, g.sy, g.sz, B2);
  if (p.bnd[0] == 2) k_update<R, C, true><<<gr, B2, 0, st>>>(g, p, ab, c1, c2, c3, incr, f, fn, df);
  else k_update<R, C, false><<<gr, B2, 0, st>>>(g, p, ab, c1, c2, c3, incr, f, fn, df);
}

template <typename R, int C>
void launch_clean(const Geom& g, const EB<R>& eb, const EB<R>& d, R ct, cudaStream_t st) {
  const dim3 gr = grid_for(g.sx, g.sy, g.sz, B2);
  CEB<R> c;
  for (int i = 0; i < 6; ++i) c.c[i] = eb.c[i];
  k_clean<R, C><<<gr, B2, 0, st>>>(g, c, d.c[0], d.c[1], d.c[2], ct);
  k_copy_e<R><<<gr, B2, 0, st>>>(g, d.c[0], d.c[1], d.c[2], eb.c[0], eb.c[1], eb.c[2]);
}

// x_done: the x ghost columns of the interior rows are already filled (the
// fused stage kernels store them), unless sx < 2 NG (two images per cell)
template <typename R>
void launch_fill(const Geom& g, const Phys& p, const EB<R>& f, R* const b0[3], bool with_b0, cudaStream_t st,
                 bool x_done) {
  const bool px = p.bnd[0] == 1, py = p.bnd[1] == 1, pz = p.bnd[2] == 1;
  const bool xs = px && !(x_done && g.sx >= 2 * NG);
  if (!xs && !py && !pz) return;  // nothing to wrap
  const int zrows = pz ? 2 * NG * (g.sy + 2 * NG) : 0;
  const int yrows = py ? 2 * NG * g.sz : 0;
  const int bs = 128;
  const int xblocks = xs ? (g.sy * g.sz + bs - 1) / bs : 0;
  k_fill<R><<<(unsigned)(zrows + yrows + xblocks), bs, 0, st>>>(g, px, py, pz, with_b0 ? 9 : 6, f, b0[0], b0[1],
                                                                  b0[2], zrows, yrows, xs ? 1 : 0);
}

template <typename R>
void launch_psr_bc(const Geom& g, const Phys& p, const PsrBC<R>& q, const EB<R>& f, R* box, cudaStream_t st) {
  if (q.bx <= 0 || q.by <= 0 || q.bz <= 0) return;
  const dim3 gr = grid_for(q.bx, q.by, q.bz, B2);
  CEB<R> c;
  for (int i = 0; i < 6; ++i) c.c[i] = f.c[i];
  k_psr_bc<R><<<gr, B2, 0, st>>>(g, p, q, c, box);
  k_psr_copy<R><<<gr, B2, 0, st>>>(g, p, q, f, box);
}

template <typename R>
void launch_uniform_bc(const Geom& g, const Phys& p, const UniformBC<R>& u, const EB<R>& f, bool ghosts_only,
                       cudaStream_t st) {
  // planes k with k + z0 <= 0 or k + z0 >= gsz, k in [-2, sz+1]; the fused
  // path applies the BC to the interior plane itself and asks for ghosts only
  const int klo = -NG, khi = g.sz + NG - 1;
  int a_hi = std::min(khi, -p.z0);              // z_glob <= 0
  int b_lo = std::max(klo, p.gsz - p.z0);       // z_glob >= gsz
  if (ghosts_only) {
    a_hi = std::min(a_hi, -1);
    b_lo = std::max(b_lo, g.sz);
  }
  const dim3 b(32, 8, 1);
  if (a_hi >= klo) {
    const int nk = a_hi - klo + 1;
    k_uniform_bc<R><<<grid_for(g.sx + 2 * NG, g.sy + 2 * NG, nk, b), b, 0, st>>>(g, p, u, f, klo, nk);
  }
  if (b_lo <= khi) {
    const int nk = khi - b_lo + 1;
    k_uniform_bc<R><<<grid_for(g.sx + 2 * NG, g.sy + 2 * NG, nk, b), b, 0, st>>>(g, p, u, f, b_lo, nk);
  }
}

template <typename R>
void launch_loop_bc(const Geom& g, const Phys& p, const EB<R>& f, cudaStream_t st) {
  k_loop_bc<R><<<grid_for(g.sx + 2 * NG, g.sy + 2 * NG, 2 * NG, B2), B2, 0, st>>>(g, p, f);
}

template <typename R>
void launch_psr_init(const Geom& g, const Phys& p, const PsrBC<R>& q, const EB<R>& f, cudaStream_t st) {
  k_psr_init<R><<<grid_for(g.sx, g.sy, g.sz, B2), B2, 0, st>>>(g, p, q, f);
}

template <typename R>
void launch_uniform_init(const Geom& g, const Phys& p, const UniformBC<R>& u, R* bz, R* b0z, cudaStream_t st) {
  k_uniform_init<R><<<grid_for(g.sx + 2 * NG, g.sy + 2 * NG, g.sz + 2 * NG, B2), B2, 0, st>>>(g, p, u, bz, b0z);
}

template <typename R>
void launch_loop_init(const Geom& g, const Phys& p, const double prm[8], const EB<R>& f, const EB<R>& f0,
                      cudaStream_t st) {
  // user_loop.F90:27-41, in precision R
  const R L0 = R(prm[0]), a0 = R(prm[1]), h0 = R(prm[2]);
  LoopInit<R> L;
  L.xc = R(0.5) * R(p.gsx);
  L.yc1 = R(0.5) * R(p.gsy) - a0 * L0;
  L.yc2 = R(0.5) * R(p.gsy) + a0 * L0;
  L.zc = -h0 * L0;
  L.bnorm = (R(1000.0) * (h0 * h0)) * (L0 * L0);
  k_loop_init<R><<<grid_for(g.sx + 2 * NG, g.sy + 2 * NG, g.sz + 2 * NG, B2), B2, 0, st>>>(g, p, L, f, f0);
}

// Reference layout (rows of sx+4 elements, contiguous) <-> padded rows of px.
template <typename R>
__global__ void k_repack(Geom g, const R* __restrict__ src, R* __restrict__ dst, long long n, int to_padded) {
  const long long w = g.sx + 2 * NG;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long r = e / w, i = e - r * w;
    const long long q = r * g.px + (g.ox - NG) + i;
    if (to_padded) dst[q] = src[e];
    else dst[e] = src[q];
  }
}

template <typename R>
void launch_repack(const Geom& g, const R* src, R* dst, bool to_padded, cudaStream_t st) {
  const long long n = (long long)(g.sx + 2 * NG) * (g.sy + 2 * NG) * (g.sz + 2 * NG);
  const int bs = 256;
  const long long blocks = std::min<long long>((n + bs - 1) / bs, 152LL * 64);
  k_repack<R><<<(unsigned)blocks, bs, 0, st>>>(g, src, dst, n, to_padded ? 1 : 0);
}
template void launch_repack<float>(const Geom&, const float*, float*, bool, cudaStream_t);
template void launch_repack<double>(const Geom&, const double*, double*, bool, cudaStream_t);

template <typename R>
void launch_finite(const Geom& g, const CEB<R>& f, int* bad, cudaStream_t st) {
  k_finite<R><<<grid_for(g.sx, g.sy, g.sz, B2), B2, 0, st>>>(g, f, bad);
}

size_t waves_param_bytes() { return sizeof(Modes); }

// modes: 11 doubles per mode (K[3], phi, a, u[3], n[3]); bg: uniform background B.
template <typename R>
int launch_waves(const Geom& g, const Phys& p, const double bg[3], int n, const double* modes, void* dparam,
                 const EB<R>& f, cudaStream_t st) {
  if (n < 0 || n > MAX_MODES) return -1;
  Modes M;
  M.n = n;
  for (int c = 0; c < 3; ++c) M.bg[c] = bg[c];
  for (int m = 0; m < n; ++m) {
    const double* q = modes + 11 * m;
    Mode& o = M.m[m];
    for (int c = 0; c < 3; ++c) { o.K[c] = q[c]; o.u[c] = q[5 + c]; o.n[c] = q[8 + c]; }
    o.phi = q[3];
    o.a = q[4];
  }
  cudaError_t e = cudaMemcpyAsync(dparam, &M, sizeof M, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return -3;
  e = cudaStreamSynchronize(st);  // M lives on this stack frame
  if (e != cudaSuccess) return -3;
  k_waves<R><<<grid_for(g.sx + 2 * NG, g.sy + 2 * NG, g.sz + 2 * NG, B2), B2, 0, st>>>(g, p, (const Modes*)dparam, f);
  return 0;
}
template int launch_waves<float>(const Geom&, const Phys&, const double[3], int, const double*, void*, const EB<float>&,
                                 cudaStream_t);
template int launch_waves<double>(const Geom&, const Phys&, const double[3], int, const double*, void*,
                                  const EB<double>&, cudaStream_t);

// explicit instantiations
#define FFE_INST_R(R)                                                                                          \
  template void launch_rho<R>(const Geom&, const R*, const R*, const R*, R*, cudaStream_t);                      \
  template void launch_fill<R>(const Geom&, const Phys&, const EB<R>&, R* const[3], bool, cudaStream_t, bool);         \
  template void launch_psr_bc<R>(const Geom&, const Phys&, const PsrBC<R>&, const EB<R>&, R*, cudaStream_t);     \
  template void launch_uniform_bc<R>(const Geom&, const Phys&, const UniformBC<R>&, const EB<R>&, bool,          \
                                     cudaStream_t);                                                             \
  template void launch_loop_bc<R>(const Geom&, const Phys&, const EB<R>&, cudaStream_t);                         \
  template void launch_psr_init<R>(const Geom&, const Phys&, const PsrBC<R>&, const EB<R>&, cudaStream_t);       \
  template void launch_uniform_init<R>(const Geom&, const Phys&, const UniformBC<R>&, R*, R*, cudaStream_t);     \
  template void launch_loop_init<R>(const Geom&, const Phys&, const double[8], const EB<R>&, const EB<R>&,       \
                                    cudaStream_t);                                                             \
  template void launch_finite<R>(const Geom&, const CEB<R>&, int*, cudaStream_t);
#define FFE_INST_RC(R, C)                                                                                     \
  template void launch_push<R, C>(const Geom&, R, const CEB<R>&, const CEB<R>&, bool, const R*, const EB<R>&,  \
                                  cudaStream_t);                                                              \
  template void launch_update<R, C>(const Geom&, const Phys&, const Absorb<R>&, R, R, R, bool, const EB<R>&,   \
                                    const CEB<R>&, const CEB<R>&, cudaStream_t);                              \
  template void launch_clean<R, C>(const Geom&, const EB<R>&, const EB<R>&, R, cudaStream_t);

FFE_INST_R(float)
FFE_INST_R(double)
FFE_INST_RC(float, 0)
FFE_INST_RC(float, 1)
FFE_INST_RC(float, 2)
FFE_INST_RC(double, 0)

}  // namespace ffe
