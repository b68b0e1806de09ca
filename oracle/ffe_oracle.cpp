// ffe_oracle.cpp — TEST INFRASTRUCTURE ONLY: the CPU oracle.
//
// A restatement, in C++, of tristan-ff's force-free field update so that the
// GPU library can be checked against it.  Only the tests, the smoke check and
// the CPU-baseline leg of the benchmark load this file's library; the product
// path never does.
//
// PARITY UNPINNED.  The reference ships no tests, golden vectors or fixtures,
// and it cannot be built in this image (Fortran + MPI + HDF5 + Intel ifport,
// none present), so no output of the reference itself exists to pin this
// restatement to.  It is pinned instead by (1) an independent numpy
// restatement of the same procedures that must agree bit for bit
// (oracle/ffe_numpy.py), and (2) analytic known-answer tests (tests/).
//
// What is restated (file:line in the reference project):
//   computeRho          src/algorithms/field_solver.F90:44-63
//   rk3Push             src/algorithms/field_solver.F90:65-166
//   rk3Update + absorb  src/algorithms/field_solver.F90:168-271  (incl. jg = i + y0, :211)
//   cleanEpar           src/algorithms/field_solver.F90:273-335  (out of place, no TINY)
//   initRKstep          src/algorithms/field_solver.F90:15-33    (QNAN writes 0.0, src/defs.F90:8)
//   exchangeFields      src/logistics/exchange_fields.F90:45-188 + src/tools/helpers.F90:22-46
//   mainloop sequence   src/tristanmainloop.F90:41-84
//   user_psr            user/user_psr.F90:20-69 (init), :72-332 (BC), :345-383 (dipole, shape)
//   user_uniform        user/user_uniform.F90:27-69 (init), :77-147 (BC)
//   user_loop           user/user_loop.F90:27-93 (init), :101-164 (BC)
//   TINY = 1e-7         src/defs.F90:4 (a default-real literal)
//
// Arithmetic rules: every Fortran expression keeps its left-to-right
// association ((a+b)+c, (a*b)/c), x**2 -> x*x, x**3 -> (x*x)*x, and the file
// is compiled with -ffp-contract=off so that no multiply-add is fused.  The
// precision of "real" is a template parameter: double (a -fdefault-real-8
// build) or float (the shipped build).  FP32C is this library's own
// compensated variant, defined identically on the GPU.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <memory>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum {
  F_EX, F_EY, F_EZ, F_BX, F_BY, F_BZ, F_B0X, F_B0Y, F_B0Z,
  F_DEX, F_DEY, F_DEZ, F_DBX, F_DBY, F_DBZ,
  F_ENX, F_ENY, F_ENZ, F_BNX, F_BNY, F_BNZ, F_RHO, F_N
};

constexpr int NG = 2;  // NGHOST, src/CMakeLists.txt:18

struct Desc {
  int sx, sy, sz, x0, y0, z0, gsx, gsy, gsz;
  int bnd[3];
  int absorb_buff;
  int precision;  // 0 fp64, 1 fp32, 2 fp32c
  int setup;      // 0 none, 1 psr, 2 uniform, 3 loop
  int flags;      // this library's opt-ins: 1 clamp the absorbing depth to 1, 2 TINY in
                  // the cleaning denominators, 4 the absorbing shell's true y coordinate
  double cc;
  double params[8];
};

struct OracleBase {
  Desc d;
  int loop_order = 1;  // 0: reference order (k innermost), 1: x innermost
  int nthreads = 1;
  virtual ~OracleBase() {}
  virtual void* field(int f) = 0;
  virtual size_t elem_size() const = 0;
  virtual void init_rk_step() = 0;
  virtual void compute_rho() = 0;
  virtual void push() = 0;
  virtual void update(double c1, double c2, double c3) = 0;
  virtual void clean() = 0;
  virtual void exchange(int b0) = 0;
  virtual void user_init() = 0;
  virtual void user_bc(int step) = 0;
  virtual void init_waves(const double bg[3], int n, const double* modes) = 0;
  void rk3_stage(double c1, double c2, double c3) {
    compute_rho();
    push();
    update(c1, c2, c3);
  }
  void prologue() {  // src/tristanmainloop.F90:41-42
    exchange(1);
    user_bc(0);
  }
  virtual void step(int nsteps, int step0) = 0;
};

// COMP: 0 the reference's arithmetic; 1 increment-form RK combination;
// 2 that plus double B^2 denominators (this library's FP32C / FP32CD).
template <typename R, int COMP>
struct Oracle : OracleBase {
  long nx, ny, nz, nxy, ntot;
  std::vector<R> a[F_N];
  // per-setup constants, evaluated in precision R as the user files do
  R psr_radius, psr_angle, psr_period, psr_omega, psr_scale, xc_g, yc_g, zc_g;
  R u_L0, u_r0, u_t0, u_beta, u_xc, u_yc, u_bnorm;
  R CC, CCINV;

  explicit Oracle(const Desc& dd) {
    d = dd;
    nx = d.sx + 2 * NG;
    ny = d.sy + 2 * NG;
    nz = d.sz + 2 * NG;
    nxy = nx * ny;
    ntot = nxy * nz;
    for (int f = 0; f < F_N; ++f) a[f].assign(ntot, R(0));
    CC = R(d.cc);
    CCINV = R(1.0) / CC;  // src/logistics/initialize.F90:190
    if (d.flags & 2) ct = TINYR();
    setup_constants();
  }

  void* field(int f) override { return a[f].data(); }
  size_t elem_size() const override { return sizeof(R); }

  inline long I(int i, int j, int k) const {
    return (long)(i + NG) + nx * ((long)(j + NG) + ny * (long)(k + NG));
  }

  // Synthetic plane-wave fields (the benchmark workloads; not a reference
  // procedure): B = bg + sum_m dB_m, E = sum_m -n_m x dB_m with
  // dB_m = -a_m sin(K_m.x + phi_m) u_m at every staggered point, ghosts
  // included, 11 doubles per mode as for ffe_init_waves.  The sine of the
  // separable phase is the imaginary part of a product of per-axis complex
  // exponentials, so a point costs two multiply-adds per mode; only used to
  // set up timing samples, where its last-bit rounding is immaterial.
  void init_waves(const double bg[3], int n, const double* modes) override {
    const double ox[6] = {0.5, 0, 0, 0, 0.5, 0.5}, oy[6] = {0, 0.5, 0, 0.5, 0, 0.5}, oz[6] = {0, 0, 0.5, 0.5, 0.5, 0};
    for (int c = 0; c < 6; ++c) {
      std::vector<double> coef(n), xr((size_t)n * nx), xi((size_t)n * nx);
      for (int m = 0; m < n; ++m) {
        const double* q = modes + 11 * m;  // K[3], phi, a, u[3], n[3]
        const double u[3] = {q[5], q[6], q[7]}, nn[3] = {q[8], q[9], q[10]};
        const double nxu[3] = {nn[1] * u[2] - nn[2] * u[1], nn[2] * u[0] - nn[0] * u[2], nn[0] * u[1] - nn[1] * u[0]};
        // B: + (-a s u_c);  E: - (n x dB)_c = + a s (n x u)_c
        coef[m] = c >= 3 ? -q[4] * u[c - 3] : q[4] * nxu[c];
        for (long i = 0; i < nx; ++i) {
          const double ph = q[0] * ((double)(i - NG + d.x0) + ox[c]);
          xr[(size_t)m * nx + i] = std::cos(ph);
          xi[(size_t)m * nx + i] = std::sin(ph);
        }
      }
      R* f = a[F_EX + c].data();
      const double base = c >= 3 ? bg[c - 3] : 0.0;
#pragma omp parallel for num_threads(nthreads) schedule(static)
      for (long k = 0; k < nz; ++k) {
        std::vector<double> v(nx);
        for (long j = 0; j < ny; ++j) {
          for (long i = 0; i < nx; ++i) v[i] = base;
          for (int m = 0; m < n; ++m) {
            const double* q = modes + 11 * m;
            const double ph = q[1] * ((double)(j - NG + d.y0) + oy[c]) + q[2] * ((double)(k - NG + d.z0) + oz[c]) + q[3];
            const double wr = std::cos(ph), wi = std::sin(ph), cm = coef[m];
            const double* er = &xr[(size_t)m * nx];
            const double* ei = &xi[(size_t)m * nx];
            for (long i = 0; i < nx; ++i) v[i] += cm * (er[i] * wi + ei[i] * wr);
          }
          R* row = f + nx * (j + ny * k);
          for (long i = 0; i < nx; ++i) row[i] = (R)v[i];
        }
      }
    }
    for (int c = F_B0X; c <= F_B0Z; ++c) std::fill(a[c].begin(), a[c].end(), R(0));
  }

  // Loop over [i1,i2]x[j1,j2]x[k1,k2] in the configured order; body(i,j,k).
  template <typename F>
  void loop3(int i1, int i2, int j1, int j2, int k1, int k2, F&& body) {
    if (loop_order == 0) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
      for (int i = i1; i <= i2; ++i)
        for (int j = j1; j <= j2; ++j)
          for (int k = k1; k <= k2; ++k) body(i, j, k);
    } else {
#pragma omp parallel for num_threads(nthreads) schedule(static)
      for (int k = k1; k <= k2; ++k)
        for (int j = j1; j <= j2; ++j)
          for (int i = i1; i <= i2; ++i) body(i, j, k);
    }
  }

  static R TINYR() { return sizeof(R) == 4 ? R(1e-7f) : R(1e-7); }

  void setup_constants() {
    const R PI_PSR = R(3.14159265f);  // user/user_psr.F90:11, a default-real parameter
    // when real is double the literal 3.14159265 is read as double
    const R pi_psr = sizeof(R) == 8 ? R(3.14159265) : PI_PSR;
    psr_radius = R(d.params[0]);
    psr_angle = R(d.params[1]);
    psr_angle = psr_angle * pi_psr / R(180.0);               // user_psr.F90:30
    psr_period = R(d.params[2]);
    psr_omega = R(2.0) * pi_psr / (psr_period != R(0) ? psr_period : R(1));  // :32
    psr_scale = R(d.params[3] == 0.0 ? 1.0 : d.params[3]);
    xc_g = R(0.5) * R(d.gsx);  // :34-36
    yc_g = R(0.5) * R(d.gsy);
    zc_g = R(0.5) * R(d.gsz);
    if (d.setup == 2) {        // user_uniform.F90:29-40
      u_L0 = R(d.params[0]);
      u_r0 = R(d.params[1]);
      u_t0 = R(d.params[2]);
      u_beta = R(d.params[3]);
      u_xc = R(0.5) * R(d.gsx);
      u_yc = R(0.5) * R(d.gsy);
      u_r0 = u_r0 * u_L0;
      u_bnorm = R(1.0);
    }
  }

  // ---- initRKstep: src/algorithms/field_solver.F90:15-33 ---------------
  void init_rk_step() override {
    for (int c = 0; c < 3; ++c) {
      a[F_ENX + c] = a[F_EX + c];
      a[F_BNX + c] = a[F_BX + c];
    }
    // QNAN = TRANSFER((/Z'00000000',Z'7FF80000'/), 1.0_4) keeps the first
    // four bytes, i.e. 0.0 on little-endian hosts (src/defs.F90:8).
    for (int f = F_DEX; f <= F_DBZ; ++f) std::fill(a[f].begin(), a[f].end(), R(0));
    std::fill(a[F_RHO].begin(), a[F_RHO].end(), R(0));
  }

  // ---- computeRho: field_solver.F90:44-63 -------------------------------
  void compute_rho() override {
    const R* ex = a[F_EX].data();
    const R* ey = a[F_EY].data();
    const R* ez = a[F_EZ].data();
    R* rho = a[F_RHO].data();
    const long di = 1, dj = nx, dk = nxy;
    loop3(-1, d.sx + 1, -1, d.sy + 1, -1, d.sz + 1, [&](int i, int j, int k) {
      long s = I(i, j, k);
      rho[s] = ((ex[s] - ex[s - di]) + (ey[s] - ey[s - dj])) + (ez[s] - ez[s - dk]);
    });
  }

  // J denominators: plain (reference) or double (FP32C).
  static inline R jterm(R cc, R bmag, R intbx, R intby, R intbz, R num) {
    if (COMP == 2) {
      double bd = ((double)intbx * (double)intbx + (double)intby * (double)intby) +
                  (double)intbz * (double)intbz;
      return (R)((double)cc / (bd + (double)1e-7f) * (double)num);
    } else {
      return cc / (bmag + TINYR()) * num;
    }
  }

  // ---- rk3Push: field_solver.F90:65-166 ---------------------------------
  void push() override {
    const R *ex = a[F_EX].data(), *ey = a[F_EY].data(), *ez = a[F_EZ].data();
    const R *bx = a[F_BX].data(), *by = a[F_BY].data(), *bz = a[F_BZ].data();
    const R *b0x = a[F_B0X].data(), *b0y = a[F_B0Y].data(), *b0z = a[F_B0Z].data();
    const R* rho = a[F_RHO].data();
    R *dex = a[F_DEX].data(), *dey = a[F_DEY].data(), *dez = a[F_DEZ].data();
    R *dbx = a[F_DBX].data(), *dby = a[F_DBY].data(), *dbz = a[F_DBZ].data();
    const long di = 1, dj = nx, dk = nxy;
    const R cc = CC;
    loop3(0, d.sx - 1, 0, d.sy - 1, 0, d.sz - 1, [&](int i, int j, int k) {
      const long s = I(i, j, k);
      dbx[s] = cc * ((ey[s + dk] - ey[s]) - (ez[s + dj] - ez[s]));
      dby[s] = cc * ((ez[s + di] - ez[s]) - (ex[s + dk] - ex[s]));
      dbz[s] = cc * ((ex[s + dj] - ex[s]) - (ey[s + di] - ey[s]));
      dex[s] = -(cc * (((by[s] - by[s - dk]) - (bz[s] - bz[s - dj])) -
                       ((b0y[s] - b0y[s - dk]) - (b0z[s] - b0z[s - dj]))));
      dey[s] = -(cc * (((bz[s] - bz[s - di]) - (bx[s] - bx[s - dk])) -
                       ((b0z[s] - b0z[s - di]) - (b0x[s] - b0x[s - dk]))));
      dez[s] = -(cc * (((bx[s] - bx[s - dj]) - (by[s] - by[s - di])) -
                       ((b0x[s] - b0x[s - dj]) - (b0y[s] - b0y[s - di]))));
      R intrho, intex, intey, intez, intbx, intby, intbz, bmag, emag, corr;
      // X current (:91-111)
      intrho = R(0.5) * (rho[s + di] + rho[s]);
      intex = ex[s];
      intey = R(0.25) * (((ey[s] + ey[s + di]) + ey[s - dj]) + ey[s + di - dj]);
      intez = R(0.25) * (((ez[s] + ez[s + di]) + ez[s - dk]) + ez[s + di - dk]);
      intbx = R(0.125) * (((((((bx[s] + bx[s - dj]) + bx[s + di - dj]) + bx[s + di]) + bx[s - dk]) +
                             bx[s - dj - dk]) + bx[s + di - dj - dk]) + bx[s + di - dk]);
      intby = R(0.5) * (by[s] + by[s - dk]);
      intbz = R(0.5) * (bz[s] + bz[s - dj]);
      bmag = (intbx * intbx + intby * intby) + intbz * intbz;
      emag = (intex * intex + intey * intey) + intez * intez;
      if (emag > bmag) {
        corr = std::sqrt(bmag / emag);
        intey = intey * corr;
        intez = intez * corr;
      }
      const R jx = jterm(cc, bmag, intbx, intby, intbz, intrho * (intey * intbz - intby * intez));
      // Y current (:114-134)
      intrho = R(0.5) * (rho[s + dj] + rho[s]);
      intex = R(0.25) * (((ex[s] + ex[s - di]) + ex[s + dj]) + ex[s - di + dj]);
      intey = ey[s];
      intez = R(0.25) * (((ez[s] + ez[s + dj]) + ez[s - dk]) + ez[s + dj - dk]);
      intbx = R(0.5) * (bx[s] + bx[s - dk]);
      intby = R(0.125) * (((((((by[s] + by[s - di]) + by[s - di + dj]) + by[s + dj]) + by[s - dk]) +
                             by[s - di - dk]) + by[s - di + dj - dk]) + by[s + dj - dk]);
      intbz = R(0.5) * (bz[s] + bz[s - di]);
      bmag = (intbx * intbx + intby * intby) + intbz * intbz;
      emag = (intex * intex + intey * intey) + intez * intez;
      if (emag > bmag) {
        corr = std::sqrt(bmag / emag);
        intex = intex * corr;
        intez = intez * corr;
      }
      const R jy = jterm(cc, bmag, intbx, intby, intbz, intrho * (intez * intbx - intex * intbz));
      // Z current (:137-157)
      intrho = R(0.5) * (rho[s] + rho[s + dk]);
      intex = R(0.25) * (((ex[s] + ex[s - di]) + ex[s + dk]) + ex[s - di + dk]);
      intey = R(0.25) * (((ey[s] + ey[s - dj]) + ey[s + dk]) + ey[s - dj + dk]);
      intez = ez[s];
      intbx = R(0.5) * (bx[s] + bx[s - dj]);
      intby = R(0.5) * (by[s] + by[s - di]);
      intbz = R(0.125) * (((((((bz[s] + bz[s - di]) + bz[s - di - dj]) + bz[s - dj]) + bz[s + dk]) +
                             bz[s - di + dk]) + bz[s - di - dj + dk]) + bz[s - dj + dk]);
      bmag = (intbx * intbx + intby * intby) + intbz * intbz;
      emag = (intex * intex + intey * intey) + intez * intez;
      if (emag > bmag) {
        corr = std::sqrt(bmag / emag);
        intex = intex * corr;
        intey = intey * corr;
      }
      const R jz = jterm(cc, bmag, intbx, intby, intbz, intrho * (intex * intby - intbx * intey));
      dex[s] = dex[s] - jx;
      dey[s] = dey[s] - jy;
      dez[s] = dez[s] - jz;
    });
  }

  // RK combination: reference form (c1*fn + c2*f) + c3*df, or the FP32C
  // increment form fn + (c2*(f - fn) + c3*df) when c1 + c2 == 1.
  static inline R combine(R c1, R c2, R c3, R fn, R f, R df, bool incr) {
    if (COMP && incr) return fn + (c2 * (f - fn) + c3 * df);
    return (c1 * fn + c2 * f) + c3 * df;
  }

  // ---- rk3Update: field_solver.F90:168-271 ------------------------------
  void update(double c1d, double c2d, double c3d) override {
    const R c1 = R(c1d), c2 = R(c2d), c3 = R(c3d);
    // c1 + c2 = 1 for SSP-RK3; the float-rounded 1/3 + 2/3 misses by 3e-8
    const bool incr = COMP && std::fabs(c1d + c2d - 1.0) < 1e-6;
    R* f[6];
    const R* fn[6];
    const R* df[6];
    for (int c = 0; c < 3; ++c) {
      f[c] = a[F_EX + c].data();
      f[3 + c] = a[F_BX + c].data();
      fn[c] = a[F_ENX + c].data();
      fn[3 + c] = a[F_BNX + c].data();
      df[c] = a[F_DEX + c].data();
      df[3 + c] = a[F_DBX + c].data();
    }
    if (d.bnd[0] != 2) {
      loop3(0, d.sx - 1, 0, d.sy - 1, 0, d.sz - 1, [&](int i, int j, int k) {
        const long s = I(i, j, k);
        for (int c = 0; c < 6; ++c) f[c][s] = combine(c1, c2, c3, fn[c][s], f[c][s], df[c][s], incr);
      });
      return;
    }
    // absorbing boundaries (:198-268)
    const R xc = R(0.5) * R(d.gsx), yc = R(0.5) * R(d.gsy), zc = R(0.5) * R(d.gsz);
    const R rmax = std::min(std::min(xc, yc), zc);
    const R rabsorb = rmax - R(d.absorb_buff);
    const R buff = R(d.absorb_buff);
    loop3(0, d.sx - 1, 0, d.sy - 1, 0, d.sz - 1, [&](int i, int j, int k) {
      const long s = I(i, j, k);
      const R ig = R(i + d.x0);
      // the reference uses i here (field_solver.F90:211); flag 4 = this library's opt-in true y
      const R jg = R(((d.flags & 4) ? j : i) + d.y0);
      const R kg = R(k + d.z0);
      for (int c = 0; c < 6; ++c) f[c][s] = combine(c1, c2, c3, fn[c][s], f[c][s], df[c][s], incr);
      R r = std::sqrt(((ig - xc) * (ig - xc) + (jg - yc) * (jg - yc)) + (kg - zc) * (kg - zc));
      if (r > rabsorb - R(1.0)) {
        // offsets of the six staggered points: Ex, Ey, Ez, Bx, By, Bz
        const R ox[6] = {R(0.5), R(0), R(0), R(0), R(0.5), R(0.5)};
        const R oy[6] = {R(0), R(0.5), R(0), R(0.5), R(0), R(0.5)};
        const R oz[6] = {R(0), R(0), R(0.5), R(0.5), R(0.5), R(0)};
        for (int c = 0; c < 6; ++c) {
          const R dx = ox[c] != R(0) ? (ig + ox[c]) - xc : ig - xc;
          const R dy = oy[c] != R(0) ? (jg + oy[c]) - yc : jg - yc;
          const R dz = oz[c] != R(0) ? (kg + oz[c]) - zc : kg - zc;
          r = std::sqrt((dx * dx + dy * dy) + dz * dz);
          R delta_r = (r - rabsorb) / buff;
          if ((d.flags & 1) && delta_r > R(1.0)) delta_r = R(1.0);
          if (delta_r > R(0.0)) f[c][s] = (R(1.0) - (delta_r * delta_r) * delta_r) * f[c][s];
        }
      }
    });
  }

  // ---- cleanEpar: field_solver.F90:273-335 ------------------------------
  // ct = 0 as in the reference, or TINY under this library's opt-in flag 2
  R ct = R(0);
  inline R clean_term(R epar, R bi, R bmag, R intbx, R intby, R intbz) const {
    if (COMP == 2) {
      double bd = ((double)intbx * (double)intbx + (double)intby * (double)intby) +
                  (double)intbz * (double)intbz;
      return (R)((double)(epar * bi) / (bd + (double)ct));
    }
    return epar * bi / (bmag + ct);
  }

  void clean() override {
    const R *ex = a[F_EX].data(), *ey = a[F_EY].data(), *ez = a[F_EZ].data();
    const R *bx = a[F_BX].data(), *by = a[F_BY].data(), *bz = a[F_BZ].data();
    R *dex = a[F_DEX].data(), *dey = a[F_DEY].data(), *dez = a[F_DEZ].data();
    const long di = 1, dj = nx, dk = nxy;
    loop3(0, d.sx - 1, 0, d.sy - 1, 0, d.sz - 1, [&](int i, int j, int k) {
      const long s = I(i, j, k);
      R intex, intey, intez, intbx, intby, intbz, bmag, epar;
      intex = ex[s];
      intey = R(0.25) * (((ey[s] + ey[s + di]) + ey[s - dj]) + ey[s + di - dj]);
      intez = R(0.25) * (((ez[s] + ez[s + di]) + ez[s - dk]) + ez[s + di - dk]);
      intbx = R(0.125) * (((((((bx[s] + bx[s - dj]) + bx[s + di - dj]) + bx[s + di]) + bx[s - dk]) +
                             bx[s - dj - dk]) + bx[s + di - dj - dk]) + bx[s + di - dk]);
      intby = R(0.5) * (by[s] + by[s - dk]);
      intbz = R(0.5) * (bz[s] + bz[s - dj]);
      bmag = (intbx * intbx + intby * intby) + intbz * intbz;
      epar = (intex * intbx + intey * intby) + intez * intbz;
      dex[s] = ex[s] - clean_term(epar, intbx, bmag, intbx, intby, intbz);

      intex = R(0.25) * (((ex[s] + ex[s - di]) + ex[s + dj]) + ex[s - di + dj]);
      intey = ey[s];
      intez = R(0.25) * (((ez[s] + ez[s + dj]) + ez[s - dk]) + ez[s + dj - dk]);
      intbx = R(0.5) * (bx[s] + bx[s - dk]);
      intby = R(0.125) * (((((((by[s] + by[s - di]) + by[s - di + dj]) + by[s + dj]) + by[s - dk]) +
                             by[s - di - dk]) + by[s - di + dj - dk]) + by[s + dj - dk]);
      intbz = R(0.5) * (bz[s] + bz[s - di]);
      bmag = (intbx * intbx + intby * intby) + intbz * intbz;
      epar = (intex * intbx + intey * intby) + intez * intbz;
      dey[s] = ey[s] - clean_term(epar, intby, bmag, intbx, intby, intbz);

      intex = R(0.25) * (((ex[s] + ex[s - di]) + ex[s + dk]) + ex[s - di + dk]);
      intey = R(0.25) * (((ey[s] + ey[s - dj]) + ey[s + dk]) + ey[s - dj + dk]);
      intez = ez[s];
      intbx = R(0.5) * (bx[s] + bx[s - dj]);
      intby = R(0.5) * (by[s] + by[s - di]);
      intbz = R(0.125) * (((((((bz[s] + bz[s - di]) + bz[s - di - dj]) + bz[s - dj]) + bz[s + dk]) +
                             bz[s - di + dk]) + bz[s - di - dj + dk]) + bz[s - dj + dk]);
      bmag = (intbx * intbx + intby * intby) + intbz * intbz;
      epar = (intex * intbx + intey * intby) + intez * intbz;
      dez[s] = ez[s] - clean_term(epar, intbz, bmag, intbx, intby, intbz);
    });
    // ex(i1:i2, j1:j2, k1:k2) = dex(...)  (:332-334)
    R *wx = a[F_EX].data(), *wy = a[F_EY].data(), *wz = a[F_EZ].data();
    loop3(0, d.sx - 1, 0, d.sy - 1, 0, d.sz - 1, [&](int i, int j, int k) {
      const long s = I(i, j, k);
      wx[s] = dex[s];
      wy[s] = dey[s];
      wz[s] = dez[s];
    });
  }

  // ---- exchangeFields on one meshblock: exchange_fields.F90:45-188 ------
  // A ghost cell is written iff every axis on which it lies outside the
  // interior is periodic (a neighbour exists, helpers.F90:22-46); its value
  // is that of the wrapped interior cell.  Other ghosts keep their values.
  void exchange(int b0) override {
    const int s3[3] = {d.sx, d.sy, d.sz};
    const int nf = b0 ? 9 : 6;
    for (int k = -NG; k < d.sz + NG; ++k)
      for (int j = -NG; j < d.sy + NG; ++j)
        for (int i = -NG; i < d.sx + NG; ++i) {
          int c[3] = {i, j, k};
          bool ghost = false, ok = true;
          for (int ax = 0; ax < 3; ++ax) {
            if (c[ax] < 0 || c[ax] >= s3[ax]) {
              ghost = true;
              if (d.bnd[ax] != 1) ok = false;
              c[ax] = c[ax] < 0 ? c[ax] + s3[ax] : c[ax] - s3[ax];
            }
          }
          if (!ghost || !ok) continue;
          const long dst = I(i, j, k), src = I(c[0], c[1], c[2]);
          for (int f = 0; f < nf; ++f) a[f][dst] = a[f][src];
        }
  }

  // ---- user_psr: dipole and shape (user_psr.F90:345-383) ----------------
  inline void dipole(const R mu[3], R x_g, R y_g, R z_g, R& obx, R& oby, R& obz) const {
    R nxv = x_g - xc_g, nyv = y_g - yc_g, nzv = z_g - zc_g;
    R rr = R(1.0) / std::sqrt((nxv * nxv + nyv * nyv) + nzv * nzv);
    nxv = nxv * rr;
    nyv = nyv * rr;
    nzv = nzv * rr;
    rr = (rr * rr) * rr;
    const R mu_dot_n = (mu[0] * nxv + mu[1] * nyv) + mu[2] * nzv;
    obx = (R(3.0) * nxv * mu_dot_n - mu[0]) * rr;
    oby = (R(3.0) * nyv * mu_dot_n - mu[1]) * rr;
    obz = (R(3.0) * nzv * mu_dot_n - mu[2]) * rr;
  }
  // mux = psr_radius**3 * sin(psr_angle) * cos(phase + offset), phase = omega*step
  void dipole_moment(int step, R mu[3]) const {
    const R phase = psr_omega * R(step);
    const R r3 = ((psr_radius * psr_radius) * psr_radius) * psr_scale;
    mu[0] = r3 * std::sin(psr_angle) * std::cos(phase);
    mu[1] = r3 * std::sin(psr_angle) * std::sin(phase);
    mu[2] = r3 * std::cos(psr_angle);
  }
  static inline R shape(R rad, R rad0) { return R(0.5) * (R(1.0) - std::tanh((rad - rad0) / R(1.0))); }

  void user_init() override {
    for (int f = 0; f < 9; ++f) std::fill(a[f].begin(), a[f].end(), R(0));
    if (d.setup == 1) {  // user_psr.F90:39-69
      R mu[3];
      dipole_moment(0, mu);
      R b0, b1, b2;
      for (int k = 0; k < d.sz; ++k)
        for (int j = 0; j < d.sy; ++j)
          for (int i = 0; i < d.sx; ++i) {
            const long s = I(i, j, k);
            const R ig = R(i + d.x0), jg = R(j + d.y0), kg = R(k + d.z0);
            dipole(mu, ig, jg + R(0.5), kg + R(0.5), b0, b1, b2);
            a[F_BX][s] = b0;
            dipole(mu, ig + R(0.5), jg, kg + R(0.5), b0, b1, b2);
            a[F_BY][s] = b1;
            dipole(mu, ig + R(0.5), jg + R(0.5), kg, b0, b1, b2);
            a[F_BZ][s] = b2;
          }
    } else if (d.setup == 2) {  // user_uniform.F90:43-69
      const R tiny = TINYR();
      for (int k = -NG; k < d.sz + NG; ++k)
        for (int j = -NG; j < d.sy + NG; ++j)
          for (int i = -NG; i < d.sx + NG; ++i) {
            const R xg = R(i + d.x0), yg = R(j + d.y0);
            const R rx = (xg + R(0.5)) - u_xc, ry = (yg + R(0.5)) - u_yc;
            const R rr = std::sqrt((rx * rx + ry * ry) + tiny);
            a[F_BZ][I(i, j, k)] = u_bnorm / (R(1.0) + (rr / u_r0));
          }
      for (int c = 0; c < 3; ++c) a[F_B0X + c] = a[F_BX + c];
    } else if (d.setup == 3) {  // user_loop.F90:27-93
      const R L0 = R(d.params[0]), a0 = R(d.params[1]), h0 = R(d.params[2]);
      const R xc = R(0.5) * R(d.gsx);
      const R yc1 = R(0.5) * R(d.gsy) - a0 * L0;
      const R yc2 = R(0.5) * R(d.gsy) + a0 * L0;
      const R zc = -h0 * L0;
      const R bnorm = ((R(1000.0) * (h0 * h0)) * (L0 * L0));
      for (int k = -NG; k < d.sz + NG; ++k)
        for (int j = -NG; j < d.sy + NG; ++j)
          for (int i = -NG; i < d.sx + NG; ++i) {
            const long s = I(i, j, k);
            const R xg = R(i + d.x0), yg = R(j + d.y0), zg = R(k + d.z0);
            R rx, ry1, ry2, rz, rr1, rr2;
            rx = xg - xc; ry1 = (yg + R(0.5)) - yc1; ry2 = (yg + R(0.5)) - yc2; rz = (zg + R(0.5)) - zc;
            rr1 = std::sqrt((rx * rx + ry1 * ry1) + rz * rz);
            rr2 = std::sqrt((rx * rx + ry2 * ry2) + rz * rz);
            a[F_BX][s] = bnorm * (rx / ((rr1 * rr1) * rr1) - rx / ((rr2 * rr2) * rr2));
            rx = (xg + R(0.5)) - xc; ry1 = yg - yc1; ry2 = yg - yc2; rz = (zg + R(0.5)) - zc;
            rr1 = std::sqrt((rx * rx + ry1 * ry1) + rz * rz);
            rr2 = std::sqrt((rx * rx + ry2 * ry2) + rz * rz);
            a[F_BY][s] = bnorm * (ry1 / ((rr1 * rr1) * rr1) - ry2 / ((rr2 * rr2) * rr2));
            rx = (xg + R(0.5)) - xc; ry1 = (yg + R(0.5)) - yc1; ry2 = (yg + R(0.5)) - yc2; rz = zg - zc;
            rr1 = std::sqrt((rx * rx + ry1 * ry1) + rz * rz);
            rr2 = std::sqrt((rx * rx + ry2 * ry2) + rz * rz);
            a[F_BZ][s] = bnorm * (rz / ((rr1 * rr1) * rr1) - rz / ((rr2 * rr2) * rr2));
          }
      for (int c = 0; c < 3; ++c) a[F_B0X + c] = a[F_BX + c];
    }
  }

  void user_bc(int step) override {
    if (d.setup == 1) bc_psr(step);
    else if (d.setup == 2) bc_uniform(step);
    else if (d.setup == 3) bc_loop();
  }

  // ---- user_psr BC: user_psr.F90:72-332 ---------------------------------
  void bc_psr(int step) {
    const R sr2 = (psr_radius * R(2)) * (psr_radius * R(2));
    // does the meshblock touch the sphere of radius 2R?  (:93-96)
    const R xq = std::max(R(d.x0 - NG), std::min(R(d.x0 + d.sx - 1 + NG), xc_g));
    const R yq = std::max(R(d.y0 - NG), std::min(R(d.y0 + d.sy - 1 + NG), yc_g));
    const R zq = std::max(R(d.z0 - NG), std::min(R(d.z0 + d.sz - 1 + NG), zc_g));
    if (!(((xq - xc_g) * (xq - xc_g) + (yq - yc_g) * (yq - yc_g)) + (zq - zc_g) * (zq - zc_g) < sr2)) return;
    R mu[3];
    dipole_moment(step, mu);
    const R shift_B = R(4.0), shift_E = R(0.0);
    const R scaleEpar = R(0.5), scaleEperp = R(0.25), scaleBperp = R(0.5), scaleBpar = R(0.25);
    const R *ex = a[F_EX].data(), *ey = a[F_EY].data(), *ez = a[F_EZ].data();
    const R *bx = a[F_BX].data(), *by = a[F_BY].data(), *bz = a[F_BZ].data();
    const long di = 1, dj = nx, dk = nxy;
    std::vector<R> nw[6];
    for (int c = 0; c < 6; ++c) nw[c].assign(ntot, R(0));
    auto inside = [&](int i, int j, int k) {
      const R ig = R(i + d.x0), jg = R(j + d.y0), kg = R(k + d.z0);
      return ((ig - xc_g) * (ig - xc_g) + (jg - yc_g) * (jg - yc_g)) + (kg - zc_g) * (kg - zc_g) < sr2;
    };
    loop3(0, d.sx - 1, 0, d.sy - 1, 0, d.sz - 1, [&](int i, int j, int k) {
      if (!inside(i, j, k)) return;
      const long s = I(i, j, k);
      const R ig = R(i + d.x0), jg = R(j + d.y0), kg = R(k + d.z0);
      R rx, ry, rz, rr_sqr, bdx, bdy, bdz, bint, bdip, sc, sh, v;
      // B_x (:157-174)
      rx = ig - xc_g; ry = (jg + R(0.5)) - yc_g; rz = (kg + R(0.5)) - zc_g;
      rr_sqr = (rx * rx + ry * ry) + rz * rz;
      bint = (bx[s] * rx + R(0.25) * (((by[s] + by[s + dj]) + by[s - di]) + by[s - di + dj]) * ry) +
             R(0.25) * (((bz[s] + bz[s + dk]) + bz[s - di]) + bz[s - di + dk]) * rz;
      dipole(mu, rx + xc_g, ry + yc_g, rz + zc_g, bdx, bdy, bdz);
      bdip = (bdx * rx + bdy * ry) + bdz * rz;
      sc = R(1.0) / scaleBperp;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_B) * sc);
      v = (bint - bdip) * (rx / rr_sqr) * (R(1.0) - sh);
      sc = R(1.0) / scaleBpar;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_B) * sc);
      nw[3][s] = (v + bdx) + ((bx[s] - bint * rx / rr_sqr) - (bdx - bdip * rx / rr_sqr)) * (R(1.0) - sh);
      // B_y (:177-194)
      rx = (ig + R(0.5)) - xc_g; ry = jg - yc_g; rz = (kg + R(0.5)) - zc_g;
      rr_sqr = (rx * rx + ry * ry) + rz * rz;
      bint = (R(0.25) * (((bx[s] + bx[s + di]) + bx[s - dj]) + bx[s + di - dj]) * rx + by[s] * ry) +
             R(0.25) * (((bz[s] + bz[s + dk]) + bz[s - dj]) + bz[s - dj + dk]) * rz;
      dipole(mu, rx + xc_g, ry + yc_g, rz + zc_g, bdx, bdy, bdz);
      bdip = (bdx * rx + bdy * ry) + bdz * rz;
      sc = R(1.0) / scaleBperp;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_B) * sc);
      v = (bint - bdip) * (ry / rr_sqr) * (R(1.0) - sh);
      sc = R(1.0) / scaleBpar;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_B) * sc);
      nw[4][s] = (v + bdy) + ((by[s] - bint * ry / rr_sqr) - (bdy - bdip * ry / rr_sqr)) * (R(1.0) - sh);
      // B_z (:197-214)
      rx = (ig + R(0.5)) - xc_g; ry = (jg + R(0.5)) - yc_g; rz = kg - zc_g;
      rr_sqr = (rx * rx + ry * ry) + rz * rz;
      bint = (R(0.25) * (((bx[s] + bx[s + di]) + bx[s - dk]) + bx[s + di - dk]) * rx +
              R(0.25) * (((by[s] + by[s + dj]) + by[s - dk]) + by[s + dj - dk]) * ry) +
             bz[s] * rz;
      dipole(mu, rx + xc_g, ry + yc_g, rz + zc_g, bdx, bdy, bdz);
      bdip = (bdx * rx + bdy * ry) + bdz * rz;
      sc = R(1.0) / scaleBperp;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_B) * sc);
      v = (bint - bdip) * (rz / rr_sqr) * (R(1.0) - sh);
      sc = R(1.0) / scaleBpar;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_B) * sc);
      nw[5][s] = (v + bdz) + ((bz[s] - bint * rz / rr_sqr) - (bdz - bdip * rz / rr_sqr)) * (R(1.0) - sh);

      R eint, edip, vx, vy, vz, exd, eyd, ezd;
      // E_x (:219-243)
      rx = (ig + R(0.5)) - xc_g; ry = jg - yc_g; rz = kg - zc_g;
      rr_sqr = (rx * rx + ry * ry) + rz * rz;
      eint = (ex[s] * rx + R(0.25) * (((ey[s] + ey[s + di]) + ey[s - dj]) + ey[s + di - dj]) * ry) +
             R(0.25) * (((ez[s] + ez[s + di]) + ez[s - dk]) + ez[s + di - dk]) * rz;
      dipole(mu, rx + xc_g, ry + yc_g, rz + zc_g, bdx, bdy, bdz);
      vx = -(psr_omega * ry); vy = psr_omega * rx; vz = R(0.0);
      exd = -(vy * bdz - vz * bdy) * CCINV;
      eyd = (vx * bdz - vz * bdx) * CCINV;
      ezd = -(vx * bdy - vy * bdx) * CCINV;
      edip = (exd * rx + eyd * ry) + ezd * rz;
      sc = R(1.0) / scaleEpar;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_E) * sc);
      v = exd + ((ex[s] - eint * rx / rr_sqr) - (exd - edip * rx / rr_sqr)) * (R(1.0) - sh);
      sc = R(1.0) / scaleEperp;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_E) * sc);
      nw[0][s] = v + (eint - edip) * (rx / rr_sqr) * (R(1.0) - sh);
      // E_y (:246-270)
      rx = ig - xc_g; ry = (jg + R(0.5)) - yc_g; rz = kg - zc_g;
      rr_sqr = (rx * rx + ry * ry) + rz * rz;
      eint = (R(0.25) * (((ex[s] + ex[s + dj]) + ex[s - di]) + ex[s - di + dj]) * rx + ey[s] * ry) +
             R(0.25) * (((ez[s] + ez[s + dj]) + ez[s - dk]) + ez[s + dj - dk]) * rz;
      dipole(mu, rx + xc_g, ry + yc_g, rz + zc_g, bdx, bdy, bdz);
      vx = -(psr_omega * ry); vy = psr_omega * rx; vz = R(0.0);
      exd = -(vy * bdz - vz * bdy) * CCINV;
      eyd = (vx * bdz - vz * bdx) * CCINV;
      ezd = -(vx * bdy - vy * bdx) * CCINV;
      edip = (exd * rx + eyd * ry) + ezd * rz;
      sc = R(1.0) / scaleEpar;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_E) * sc);
      v = eyd + ((ey[s] - eint * ry / rr_sqr) - (eyd - edip * ry / rr_sqr)) * (R(1.0) - sh);
      sc = R(1.0) / scaleEperp;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_E) * sc);
      nw[1][s] = v + (eint - edip) * (ry / rr_sqr) * (R(1.0) - sh);
      // E_z (:273-297)
      rx = ig - xc_g; ry = jg - yc_g; rz = (kg + R(0.5)) - zc_g;
      rr_sqr = (rx * rx + ry * ry) + rz * rz;
      eint = (R(0.25) * (((ex[s] + ex[s + dk]) + ex[s - di]) + ex[s - di + dk]) * rx +
              R(0.25) * (((ey[s] + ey[s - dj]) + ey[s + dk]) + ey[s - dj + dk]) * ry) +
             ez[s] * rz;
      dipole(mu, rx + xc_g, ry + yc_g, rz + zc_g, bdx, bdy, bdz);
      vx = -(psr_omega * ry); vy = psr_omega * rx; vz = R(0.0);
      exd = -(vy * bdz - vz * bdy) * CCINV;
      eyd = (vx * bdz - vz * bdx) * CCINV;
      ezd = -(vx * bdy - vy * bdx) * CCINV;
      edip = (exd * rx + eyd * ry) + ezd * rz;
      sc = R(1.0) / scaleEpar;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_E) * sc);
      v = ezd + ((ez[s] - eint * rz / rr_sqr) - (ezd - edip * rz / rr_sqr)) * (R(1.0) - sh);
      sc = R(1.0) / scaleEperp;
      sh = shape(std::sqrt(rr_sqr) * sc, (psr_radius - shift_E) * sc);
      nw[2][s] = v + (eint - edip) * (rz / rr_sqr) * (R(1.0) - sh);
    });
    // copy back (:305-325)
    loop3(0, d.sx - 1, 0, d.sy - 1, 0, d.sz - 1, [&](int i, int j, int k) {
      if (!inside(i, j, k)) return;
      const long s = I(i, j, k);
      for (int c = 0; c < 6; ++c) a[F_EX + c][s] = nw[c][s];
    });
  }

  // ---- user_uniform BC: user_uniform.F90:77-147 -------------------------
  void bc_uniform(int step) {
    const R time = R(step);
    const R tiny = TINYR();
    const R th = std::tanh(time / u_t0);
    for (int k = -NG; k < d.sz + NG; ++k)
      for (int j = -NG; j < d.sy + NG; ++j)
        for (int i = -NG; i < d.sx + NG; ++i) {
          const long s = I(i, j, k);
          const R xg = R(i + d.x0), yg = R(j + d.y0), zg = R(k + d.z0);
          R rx, ry, rr, omega, ee0;
          if (zg <= R(0)) {
            rx = (xg + R(0.5)) - u_xc; ry = yg - u_yc;
            rr = std::sqrt((rx * rx + ry * ry) + tiny);
            omega = std::exp(-rr / u_r0) * u_beta * CC / u_r0;
            ee0 = -omega * u_bnorm * th;
            a[F_EX][s] = rx * ee0;
            rx = xg - u_xc; ry = (yg + R(0.5)) - u_yc;
            rr = std::sqrt((rx * rx + ry * ry) + tiny);
            omega = std::exp(-rr / u_r0) * u_beta * CC / u_r0;
            ee0 = -omega * u_bnorm * th;
            a[F_EY][s] = ry * ee0;
            rx = (xg + R(0.5)) - u_xc; ry = (yg + R(0.5)) - u_yc;
            rr = std::sqrt((rx * rx + ry * ry) + tiny);
            a[F_BZ][s] = u_bnorm / (R(1.0) + (rr / u_r0));
          }
          if (zg >= R(d.gsz)) {
            rx = (xg + R(0.5)) - u_xc; ry = (yg + R(0.5)) - u_yc;
            rr = std::sqrt((rx * rx + ry * ry) + tiny);
            a[F_BZ][s] = u_bnorm / (R(1.0) + (rr / u_r0));
            a[F_EX][s] = R(0.0);
            a[F_EY][s] = R(0.0);
          }
        }
  }

  // ---- user_loop BC: user_loop.F90:101-164 ------------------------------
  void bc_loop() {
    for (int k = -NG; k < d.sz + NG; ++k)
      for (int j = -NG; j < d.sy + NG; ++j)
        for (int i = -NG; i < d.sx + NG; ++i) {
          const long s = I(i, j, k);
          const R zg = R(k + d.z0);
          if (zg < R(0)) {
            a[F_EX][s] = a[F_EX][I(i, j, 0)];
            a[F_EY][s] = a[F_EY][I(i, j, 0)];
            a[F_BZ][s] = a[F_BZ][I(i, j, 0)];
          }
          if (zg >= R(d.gsz)) {
            a[F_EX][s] = a[F_EX][I(i, j, d.sz - 1)];
            a[F_EY][s] = a[F_EY][I(i, j, d.sz - 1)];
            a[F_BZ][s] = a[F_BZ][I(i, j, d.sz - 1)];
          }
        }
  }

  // ---- mainloop body: src/tristanmainloop.F90:50-84 ---------------------
  void step(int nsteps, int step0) override {
    const double c[3][3] = {{1.0, 0.0, 1.0},
                            {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0},
                            {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
    for (int n = 0; n < nsteps; ++n) {
      const int ts = step0 + n;
      init_rk_step();
      for (int st = 0; st < 3; ++st) {
        // the coefficients are default-real constants: rounded to R first
        rk3_stage((double)R(c[st][0]), (double)R(c[st][1]), (double)R(c[st][2]));
        user_bc(ts);
        exchange(0);
        clean();
        exchange(0);
      }
    }
  }
};

thread_local char g_err[256];

}  // namespace

extern "C" {

typedef struct {
  int32_t sx, sy, sz, x0, y0, z0, gsx, gsy, gsz;
  int32_t boundary[3];
  int32_t absorb_buff, precision, setup, path, flags, reserved;
  double cc;
  double params[8];
  void* stream;
} ora_desc;  // same layout as ffe_grid_desc in include/ffe.h

void* ora_create(const ora_desc* in) {
  Desc d;
  d.sx = in->sx; d.sy = in->sy; d.sz = in->sz;
  d.x0 = in->x0; d.y0 = in->y0; d.z0 = in->z0;
  d.gsx = in->gsx; d.gsy = in->gsy; d.gsz = in->gsz;
  for (int i = 0; i < 3; ++i) d.bnd[i] = in->boundary[i];
  if (d.bnd[0] == 2 || d.bnd[1] == 2 || d.bnd[2] == 2) d.bnd[0] = d.bnd[1] = d.bnd[2] = 2;
  d.absorb_buff = in->absorb_buff;
  d.precision = in->precision;
  d.setup = in->setup;
  d.flags = in->flags;
  d.cc = in->cc;
  for (int i = 0; i < 8; ++i) d.params[i] = in->params[i];
  if (d.sx < NG || d.sy < NG || d.sz < NG) {
    snprintf(g_err, sizeof g_err, "ghost zones overflow the domain size");
    return nullptr;
  }
  OracleBase* o = nullptr;
  if (d.precision == 0) o = new Oracle<double, 0>(d);
  else if (d.precision == 1) o = new Oracle<float, 0>(d);
  else if (d.precision == 2) o = new Oracle<float, 1>(d);
  else if (d.precision == 3) o = new Oracle<float, 2>(d);
  else snprintf(g_err, sizeof g_err, "bad precision %d", d.precision);
  return o;
}
void ora_destroy(void* h) { delete (OracleBase*)h; }
const char* ora_error(void) { return g_err; }
void ora_set_threads(void* h, int n, int loop_order) {
  auto* o = (OracleBase*)h;
  o->nthreads = n > 0 ? n : 1;
  o->loop_order = loop_order;
}
size_t ora_elem_size(void* h) { return ((OracleBase*)h)->elem_size(); }
size_t ora_field_elems(void* h) {
  auto* o = (OracleBase*)h;
  return (size_t)(o->d.sx + 2 * NG) * (o->d.sy + 2 * NG) * (o->d.sz + 2 * NG);
}
void ora_set_field(void* h, int f, const void* src) {
  auto* o = (OracleBase*)h;
  memcpy(o->field(f), src, ora_field_elems(h) * o->elem_size());
}
void ora_get_field(void* h, int f, void* dst) {
  auto* o = (OracleBase*)h;
  memcpy(dst, o->field(f), ora_field_elems(h) * o->elem_size());
}
void ora_init_rk_step(void* h) { ((OracleBase*)h)->init_rk_step(); }
void ora_compute_rho(void* h) { ((OracleBase*)h)->compute_rho(); }
void ora_push(void* h) { ((OracleBase*)h)->push(); }
void ora_update(void* h, double c1, double c2, double c3) { ((OracleBase*)h)->update(c1, c2, c3); }
void ora_rk3_stage(void* h, double c1, double c2, double c3) { ((OracleBase*)h)->rk3_stage(c1, c2, c3); }
void ora_clean(void* h) { ((OracleBase*)h)->clean(); }
void ora_exchange(void* h, int b0) { ((OracleBase*)h)->exchange(b0); }
void ora_user_init(void* h) { ((OracleBase*)h)->user_init(); }
void ora_user_bc(void* h, int step) { ((OracleBase*)h)->user_bc(step); }
void ora_prologue(void* h) { ((OracleBase*)h)->prologue(); }
void ora_step(void* h, int nsteps, int step0) { ((OracleBase*)h)->step(nsteps, step0); }
void ora_init_waves(void* h, const double* bg, int n, const double* modes) {
  ((OracleBase*)h)->init_waves(bg, n, modes);
}

}  // extern "C"
