// ffe_output.cu — the field datasets of writeOutput on the device.
//
// src/io/write_output.F90:336-413 writes twelve node-centred datasets per
// output step: ex ey ez (interpFromEdges at offset 0), bx by bz
// (interpFromFaces at offset 0; src/tools/helpers.F90:93-257), the setup's
// userOutput variables var1..var3 and the node coordinates xx yy zz, at every
// output_istep-th node of the meshblock (:270-294).  One thread per output
// node computes all twelve values and stores them into twelve compact arrays
// (x fastest, as the reference's sm_arr(0:n_i, 0:n_j, 0:n_k)).
//
// Compiled with -fmad=false, so the values equal the CPU restatement's bit
// for bit.
#include "ffe_kernels.h"
#include "ffe_physics.cuh"

namespace ffe {

namespace {

template <typename R>
struct NodeAcc {  // f(c)(i + di, j + dj, k + dk) around linear index s
  const R* f[6];
  long long s, dj, dk;
  __device__ __forceinline__ R operator()(int c, int di, int djj, int dkk) const {
    return f[c][s + di + djj * dj + dkk * dk];
  }
};

// The reference's trilinear blend of the eight corner averages.
template <typename R>
__device__ __forceinline__ R blend(R c000, R c100, R c010, R c110, R c001, R c101, R c011, R c111, R dx, R dy,
                                   R dz) {
  const R one = R(1);
  const R c00 = c000 * (one - dx) + c100 * dx;
  const R c10 = c010 * (one - dx) + c110 * dx;
  const R c0 = c00 * (one - dy) + c10 * dy;
  const R c01 = c001 * (one - dx) + c101 * dx;
  const R c11 = c011 * (one - dx) + c111 * dx;
  const R c1 = c01 * (one - dy) + c11 * dy;
  return c0 * (one - dz) + c1 * dz;
}

// interpFromEdges (helpers.F90:93-160), components EX, EY, EZ of `a`.
template <typename R, class A>
__device__ __forceinline__ void from_edges(const A& a, R dx, R dy, R dz, R o[3]) {
  const R h = R(0.5);
  o[0] = blend(h * (a(EX, 0, 0, 0) + a(EX, -1, 0, 0)), h * (a(EX, 0, 0, 0) + a(EX, 1, 0, 0)),
               h * (a(EX, 0, 1, 0) + a(EX, -1, 1, 0)), h * (a(EX, 0, 1, 0) + a(EX, 1, 1, 0)),
               h * (a(EX, 0, 0, 1) + a(EX, -1, 0, 1)), h * (a(EX, 0, 0, 1) + a(EX, 1, 0, 1)),
               h * (a(EX, 0, 1, 1) + a(EX, -1, 1, 1)), h * (a(EX, 0, 1, 1) + a(EX, 1, 1, 1)), dx, dy, dz);
  o[1] = blend(h * (a(EY, 0, 0, 0) + a(EY, 0, -1, 0)), h * (a(EY, 1, 0, 0) + a(EY, 1, -1, 0)),
               h * (a(EY, 0, 0, 0) + a(EY, 0, 1, 0)), h * (a(EY, 1, 0, 0) + a(EY, 1, 1, 0)),
               h * (a(EY, 0, 0, 1) + a(EY, 0, -1, 1)), h * (a(EY, 1, 0, 1) + a(EY, 1, -1, 1)),
               h * (a(EY, 0, 0, 1) + a(EY, 0, 1, 1)), h * (a(EY, 1, 0, 1) + a(EY, 1, 1, 1)), dx, dy, dz);
  o[2] = blend(h * (a(EZ, 0, 0, 0) + a(EZ, 0, 0, -1)), h * (a(EZ, 1, 0, 0) + a(EZ, 1, 0, -1)),
               h * (a(EZ, 0, 1, 0) + a(EZ, 0, 1, -1)), h * (a(EZ, 1, 1, 0) + a(EZ, 1, 1, -1)),
               h * (a(EZ, 0, 0, 0) + a(EZ, 0, 0, 1)), h * (a(EZ, 1, 0, 0) + a(EZ, 1, 0, 1)),
               h * (a(EZ, 0, 1, 0) + a(EZ, 0, 1, 1)), h * (a(EZ, 1, 1, 0) + a(EZ, 1, 1, 1)), dx, dy, dz);
}

// interpFromFaces (helpers.F90:162-257), components BX, BY, BZ of `a`.
template <typename R, class A>
__device__ __forceinline__ void from_faces(const A& a, R dx, R dy, R dz, R o[3]) {
  const R q = R(0.25);
  o[0] = blend(q * (((a(BX, 0, 0, 0) + a(BX, 0, -1, 0)) + a(BX, 0, 0, -1)) + a(BX, 0, -1, -1)),
               q * (((a(BX, 1, 0, 0) + a(BX, 1, -1, 0)) + a(BX, 1, 0, -1)) + a(BX, 1, -1, -1)),
               q * (((a(BX, 0, 0, 0) + a(BX, 0, 1, 0)) + a(BX, 0, 0, -1)) + a(BX, 0, 1, -1)),
               q * (((a(BX, 1, 0, 0) + a(BX, 1, 0, -1)) + a(BX, 1, 1, -1)) + a(BX, 1, 1, 0)),
               q * (((a(BX, 0, 0, 0) + a(BX, 0, 0, 1)) + a(BX, 0, -1, 0)) + a(BX, 0, -1, 1)),
               q * (((a(BX, 1, 0, 0) + a(BX, 1, 0, 1)) + a(BX, 1, -1, 0)) + a(BX, 1, -1, 1)),
               q * (((a(BX, 0, 0, 0) + a(BX, 0, 1, 0)) + a(BX, 0, 1, 1)) + a(BX, 0, 0, 1)),
               q * (((a(BX, 1, 0, 0) + a(BX, 1, 1, 0)) + a(BX, 1, 1, 1)) + a(BX, 1, 0, 1)), dx, dy, dz);
  o[1] = blend(q * (((a(BY, -1, 0, -1) + a(BY, -1, 0, 0)) + a(BY, 0, 0, -1)) + a(BY, 0, 0, 0)),
               q * (((a(BY, 0, 0, -1) + a(BY, 0, 0, 0)) + a(BY, 1, 0, -1)) + a(BY, 1, 0, 0)),
               q * (((a(BY, -1, 1, -1) + a(BY, -1, 1, 0)) + a(BY, 0, 1, -1)) + a(BY, 0, 1, 0)),
               q * (((a(BY, 0, 1, -1) + a(BY, 0, 1, 0)) + a(BY, 1, 1, -1)) + a(BY, 1, 1, 0)),
               q * (((a(BY, -1, 0, 0) + a(BY, -1, 0, 1)) + a(BY, 0, 0, 0)) + a(BY, 0, 0, 1)),
               q * (((a(BY, 0, 0, 0) + a(BY, 0, 0, 1)) + a(BY, 1, 0, 0)) + a(BY, 1, 0, 1)),
               q * (((a(BY, -1, 1, 0) + a(BY, -1, 1, 1)) + a(BY, 0, 1, 0)) + a(BY, 0, 1, 1)),
               q * (((a(BY, 0, 1, 0) + a(BY, 0, 1, 1)) + a(BY, 1, 1, 0)) + a(BY, 1, 1, 1)), dx, dy, dz);
  o[2] = blend(q * (((a(BZ, -1, -1, 0) + a(BZ, -1, 0, 0)) + a(BZ, 0, -1, 0)) + a(BZ, 0, 0, 0)),
               q * (((a(BZ, 0, -1, 0) + a(BZ, 0, 0, 0)) + a(BZ, 1, -1, 0)) + a(BZ, 1, 0, 0)),
               q * (((a(BZ, -1, 0, 0) + a(BZ, -1, 1, 0)) + a(BZ, 0, 0, 0)) + a(BZ, 0, 1, 0)),
               q * (((a(BZ, 0, 0, 0) + a(BZ, 0, 1, 0)) + a(BZ, 1, 0, 0)) + a(BZ, 1, 1, 0)),
               q * (((a(BZ, -1, -1, 1) + a(BZ, -1, 0, 1)) + a(BZ, 0, -1, 1)) + a(BZ, 0, 0, 1)),
               q * (((a(BZ, 0, -1, 1) + a(BZ, 0, 0, 1)) + a(BZ, 1, -1, 1)) + a(BZ, 1, 0, 1)),
               q * (((a(BZ, -1, 0, 1) + a(BZ, -1, 1, 1)) + a(BZ, 0, 0, 1)) + a(BZ, 0, 1, 1)),
               q * (((a(BZ, 0, 0, 1) + a(BZ, 0, 1, 1)) + a(BZ, 1, 0, 1)) + a(BZ, 1, 1, 1)), dx, dy, dz);
}

template <typename R>
__global__ void k_node_output(Geom g, Phys p, NodeGrid n, int var2_uniform, CEB<R> f, R* __restrict__ out) {
  const int i1 = blockIdx.x * blockDim.x + threadIdx.x, j1 = blockIdx.y * blockDim.y + threadIdx.y;
  const int k1 = blockIdx.z;
  if (i1 >= n.nx || j1 >= n.ny) return;
  const int i = n.i0 + i1 * n.istep, j = n.j0 + j1 * n.istep, k = n.k0 + k1 * n.istep;
  NodeAcc<R> a;
  for (int c = 0; c < 6; ++c) a.f[c] = f.c[c];
  a.s = g.idx(i, j, k);
  a.dj = g.px;
  a.dk = g.plane;
  R e[3], b[3];
  from_edges(a, R(0), R(0), R(0), e);
  from_faces(a, R(0), R(0), R(0), b);
  // var1: rho at the node's cell (user files' userOutput, var 1)
  const R rho = ((a(EX, 0, 0, 0) - a(EX, -1, 0, 0)) + (a(EY, 0, 0, 0) - a(EY, 0, -1, 0))) +
                (a(EZ, 0, 0, 0) - a(EZ, 0, 0, -1));
  // var2: user_uniform's |E x B|_perp / (r_perp |B|^2) at the raw cell values
  // (user/user_uniform.F90:159-170); zero for the other setups
  R v2 = R(0);
  if (var2_uniform) {
    const R ex = a(EX, 0, 0, 0), ey = a(EY, 0, 0, 0), ez = a(EZ, 0, 0, 0);
    const R bx = a(BX, 0, 0, 0), by = a(BY, 0, 0, 0), bz = a(BZ, 0, 0, 0);
    const R t1 = -bz * ex + bx * ez, t2 = bz * ey - by * ez;
    v2 = sqrt(t1 * t1 + t2 * t2);
    const R d1 = R(float(p.x0 + i)) - R(0.5) * R(p.gsx);
    const R d2 = R(float(p.y0 + j)) - R(0.5) * R(p.gsy);
    v2 = v2 / sqrt((d1 * d1 + d2 * d2) + tiny<R>());
    v2 = v2 / ((bx * bx + by * by) + bz * bz);
  }
  const R vals[12] = {e[0], e[1], e[2], b[0], b[1], b[2], rho, v2, R(0),
                      R(float(p.x0 + i)), R(float(p.y0 + j)), R(float(p.z0 + k))};
  const long long nn = (long long)n.nx * n.ny * n.nz;
  const long long o = i1 + (long long)n.nx * (j1 + (long long)n.ny * k1);
#pragma unroll
  for (int v = 0; v < 12; ++v) out[v * nn + o] = vals[v];
}

}  // namespace

// Output nodes of a meshblock (write_output.F90:270-294): i = i0 + i1*istep,
// i0 = ceil(x0/istep)*istep - x0, up to (ceil((x0+sx)/istep) - 1)*istep - x0.
NodeGrid node_grid(const Geom& g, const Phys& p, int istep) {
  NodeGrid n;
  n.istep = istep;
  auto axis = [&](int x0, int s, int& first, int& count) {
    const int a = (x0 + istep - 1) / istep, b = (x0 + s + istep - 1) / istep;
    first = a * istep - x0;
    const int last = (b - 1) * istep - x0;
    count = last >= first ? (last - first) / istep + 1 : 0;
  };
  axis(p.x0, g.sx, n.i0, n.nx);
  axis(p.y0, g.sy, n.j0, n.ny);
  axis(p.z0, g.sz, n.k0, n.nz);
  return n;
}

template <typename R>
void launch_node_output(const Geom& g, const Phys& p, const NodeGrid& n, bool var2_uniform, const CEB<R>& f, R* out,
                        cudaStream_t st) {
  if (n.nx <= 0 || n.ny <= 0 || n.nz <= 0) return;
  const dim3 b(32, 8, 1), gr((n.nx + 31) / 32, (n.ny + 7) / 8, n.nz);
  k_node_output<R><<<gr, b, 0, st>>>(g, p, n, var2_uniform ? 1 : 0, f, out);
}

template void launch_node_output<float>(const Geom&, const Phys&, const NodeGrid&, bool, const CEB<float>&, float*,
                                        cudaStream_t);
template void launch_node_output<double>(const Geom&, const Phys&, const NodeGrid&, bool, const CEB<double>&,
                                         double*, cudaStream_t);

}  // namespace ffe
