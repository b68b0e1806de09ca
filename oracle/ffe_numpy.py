"""TEST INFRASTRUCTURE ONLY — an independent numpy restatement of the solver.

This second transcription of tristan-ff's field solver exists to check the C++
oracle (oracle/ffe_oracle.cpp): the two are written separately (array slices
here, per-cell loops there) and must agree bit for bit on the same inputs in
float32 and float64.  Parity with the reference itself is UNPINNED: the
reference ships no tests or golden data and cannot be built in this image.

Arrays are indexed A[k+2, j+2, i+2] (z, y, x), which is the memory order of
the reference's column-major (x fastest) allocation with NGHOST = 2
(src/logistics/initialize.F90:192-199).  numpy evaluates each binary
operation separately, so no multiply-add is fused; the association of every
sum follows the Fortran source left to right.

Restated procedures (reference file:line):
  computeRho   src/algorithms/field_solver.F90:44-63
  rk3Push      src/algorithms/field_solver.F90:65-166
  rk3Update    src/algorithms/field_solver.F90:168-271
  cleanEpar    src/algorithms/field_solver.F90:273-335
  exchange     src/logistics/exchange_fields.F90:45-188
  mainloop     src/tristanmainloop.F90:41-84
"""
import numpy as np

NG = 2
FIELDS = ("ex", "ey", "ez", "bx", "by", "bz", "b0x", "b0y", "b0z")


class NumpySolver:
    def __init__(self, sx, sy, sz, dtype, cc=0.45, boundary=(1, 1, 1), absorb_buff=20,
                 gsize=None, offset=(0, 0, 0)):
        self.s = (sx, sy, sz)
        self.dt = np.dtype(dtype)
        self.R = self.dt.type
        self.cc = self.R(cc)
        self.bnd = tuple(boundary)
        if 2 in self.bnd:
            self.bnd = (2, 2, 2)
        self.absorb_buff = absorb_buff
        self.gs = gsize or (sx, sy, sz)
        self.off = offset
        shp = (sz + 2 * NG, sy + 2 * NG, sx + 2 * NG)
        self.f = {n: np.zeros(shp, self.dt) for n in FIELDS}
        self.tiny = self.R(np.float32(1e-7)) if self.dt == np.float32 else self.R(1e-7)

    # view of array A over cells i in [i1,i2], j in [j1,j2], k in [k1,k2], shifted by (di,dj,dk)
    def v(self, A, di=0, dj=0, dk=0, lo=0, hi=None):
        sx, sy, sz = self.s
        hi = hi if hi is not None else 0
        return A[NG + lo + dk: NG + sz + hi + dk,
                 NG + lo + dj: NG + sy + hi + dj,
                 NG + lo + di: NG + sx + hi + di]

    def compute_rho(self):
        ex, ey, ez = self.f["ex"], self.f["ey"], self.f["ez"]
        rho = np.zeros_like(ex)
        w = dict(lo=-1, hi=2)  # cells -1 .. s+1
        self.v(rho, **w)[...] = ((self.v(ex, **w) - self.v(ex, -1, **w)) +
                                 (self.v(ey, **w) - self.v(ey, 0, -1, **w))) + \
                                (self.v(ez, **w) - self.v(ez, 0, 0, -1, **w))
        self.rho = rho

    def _avg4(self, A, d1, d2):
        v = self.v
        return self.R(0.25) * (((v(A) + v(A, *d1)) + v(A, *d2)) +
                               v(A, *[a + b for a, b in zip(d1, d2)]))

    def push(self):
        R, v, f, cc = self.R, self.v, self.f, self.cc
        ex, ey, ez, bx, by, bz = (f[n] for n in FIELDS[:6])
        b0x, b0y, b0z = f["b0x"], f["b0y"], f["b0z"]
        rho = self.rho
        X, Y, Z = (1, 0, 0), (0, 1, 0), (0, 0, 1)
        mX, mY, mZ = (-1, 0, 0), (0, -1, 0), (0, 0, -1)
        dbx = cc * ((v(ey, *Z) - v(ey)) - (v(ez, *Y) - v(ez)))
        dby = cc * ((v(ez, *X) - v(ez)) - (v(ex, *Z) - v(ex)))
        dbz = cc * ((v(ex, *Y) - v(ex)) - (v(ey, *X) - v(ey)))
        dex = -(cc * (((v(by) - v(by, *mZ)) - (v(bz) - v(bz, *mY))) -
                      ((v(b0y) - v(b0y, *mZ)) - (v(b0z) - v(b0z, *mY)))))
        dey = -(cc * (((v(bz) - v(bz, *mX)) - (v(bx) - v(bx, *mZ))) -
                      ((v(b0z) - v(b0z, *mX)) - (v(b0x) - v(b0x, *mZ)))))
        dez = -(cc * (((v(bx) - v(bx, *mY)) - (v(by) - v(by, *mX))) -
                      ((v(b0x) - v(b0x, *mY)) - (v(b0y) - v(b0y, *mX)))))

        def avg8(A, order):
            acc = v(A, *order[0])
            for o in order[1:]:
                acc = acc + v(A, *o)
            return R(0.125) * acc

        def current(intrho, intex, intey, intez, intbx, intby, intbz, comp):
            bmag = (intbx * intbx + intby * intby) + intbz * intbz
            emag = (intex * intex + intey * intey) + intez * intez
            lim = emag > bmag
            with np.errstate(divide="ignore", invalid="ignore"):
                corr = np.sqrt(bmag / emag)
            if comp == 0:
                intey = np.where(lim, intey * corr, intey)
                intez = np.where(lim, intez * corr, intez)
                num = intrho * (intey * intbz - intby * intez)
            elif comp == 1:
                intex = np.where(lim, intex * corr, intex)
                intez = np.where(lim, intez * corr, intez)
                num = intrho * (intez * intbx - intex * intbz)
            else:
                intex = np.where(lim, intex * corr, intex)
                intey = np.where(lim, intey * corr, intey)
                num = intrho * (intex * intby - intbx * intey)
            return cc / (bmag + self.tiny) * num

        jx = current(R(0.5) * (v(rho, *X) + v(rho)), v(ex),
                     self._avg4(ey, X, mY), self._avg4(ez, X, mZ),
                     avg8(bx, [(0, 0, 0), (0, -1, 0), (1, -1, 0), (1, 0, 0),
                               (0, 0, -1), (0, -1, -1), (1, -1, -1), (1, 0, -1)]),
                     R(0.5) * (v(by) + v(by, *mZ)), R(0.5) * (v(bz) + v(bz, *mY)), 0)
        jy = current(R(0.5) * (v(rho, *Y) + v(rho)),
                     self._avg4(ex, mX, Y), v(ey), self._avg4(ez, Y, mZ),
                     R(0.5) * (v(bx) + v(bx, *mZ)),
                     avg8(by, [(0, 0, 0), (-1, 0, 0), (-1, 1, 0), (0, 1, 0),
                               (0, 0, -1), (-1, 0, -1), (-1, 1, -1), (0, 1, -1)]),
                     R(0.5) * (v(bz) + v(bz, *mX)), 1)
        jz = current(R(0.5) * (v(rho) + v(rho, *Z)),
                     self._avg4(ex, mX, Z), self._avg4(ey, mY, Z), v(ez),
                     R(0.5) * (v(bx) + v(bx, *mY)), R(0.5) * (v(by) + v(by, *mX)),
                     avg8(bz, [(0, 0, 0), (-1, 0, 0), (-1, -1, 0), (0, -1, 0),
                               (0, 0, 1), (-1, 0, 1), (-1, -1, 1), (0, -1, 1)]), 2)
        self.d = {"ex": dex - jx, "ey": dey - jy, "ez": dez - jz,
                  "bx": dbx, "by": dby, "bz": dbz}

    def update(self, c1, c2, c3):
        R, v, f = self.R, self.v, self.f
        c1, c2, c3 = R(c1), R(c2), R(c3)
        for n in FIELDS[:6]:
            v(f[n])[...] = (c1 * v(self.fn[n]) + c2 * v(f[n])) + c3 * self.d[n]
        if self.bnd[0] != 2:
            return
        sx, sy, sz = self.s
        xc, yc, zc = (R(0.5) * R(g) for g in self.gs)
        rmax = min(min(xc, yc), zc)
        rabsorb = rmax - R(self.absorb_buff)
        buff = R(self.absorb_buff)
        k, j, i = np.meshgrid(np.arange(sz), np.arange(sy), np.arange(sx), indexing="ij")
        ig = (i + self.off[0]).astype(self.dt)
        jg = (i + self.off[1]).astype(self.dt)   # field_solver.F90:211 uses i for jg
        kg = (k + self.off[2]).astype(self.dt)
        r = np.sqrt(((ig - xc) * (ig - xc) + (jg - yc) * (jg - yc)) + (kg - zc) * (kg - zc))
        shell = r > rabsorb - R(1.0)
        h = R(0.5)
        offs = {"ex": (h, 0, 0), "ey": (0, h, 0), "ez": (0, 0, h),
                "bx": (0, h, h), "by": (h, 0, h), "bz": (h, h, 0)}
        for n, (ox, oy, oz) in offs.items():
            dx = (ig + ox) - xc if ox else ig - xc
            dy = (jg + oy) - yc if oy else jg - yc
            dz = (kg + oz) - zc if oz else kg - zc
            rr = np.sqrt((dx * dx + dy * dy) + dz * dz)
            dr = (rr - rabsorb) / buff
            damp = shell & (dr > R(0.0))
            cur = v(f[n])
            cur[...] = np.where(damp, (R(1.0) - (dr * dr) * dr) * cur, cur)

    def clean(self):
        R, v, f = self.R, self.v, self.f
        ex, ey, ez, bx, by, bz = (f[n] for n in FIELDS[:6])
        X, Y, Z = (1, 0, 0), (0, 1, 0), (0, 0, 1)
        mX, mY, mZ = (-1, 0, 0), (0, -1, 0), (0, 0, -1)

        def avg8(A, order):
            acc = v(A, *order[0])
            for o in order[1:]:
                acc = acc + v(A, *o)
            return R(0.125) * acc

        def proj(intex, intey, intez, intbx, intby, intbz, bi):
            bmag = (intbx * intbx + intby * intby) + intbz * intbz
            epar = (intex * intbx + intey * intby) + intez * intbz
            with np.errstate(divide="ignore", invalid="ignore"):
                return epar * bi / bmag

        bxa = avg8(bx, [(0, 0, 0), (0, -1, 0), (1, -1, 0), (1, 0, 0),
                        (0, 0, -1), (0, -1, -1), (1, -1, -1), (1, 0, -1)])
        nex = v(ex) - proj(v(ex), self._avg4(ey, X, mY), self._avg4(ez, X, mZ), bxa,
                           R(0.5) * (v(by) + v(by, *mZ)), R(0.5) * (v(bz) + v(bz, *mY)), bxa)
        bya = avg8(by, [(0, 0, 0), (-1, 0, 0), (-1, 1, 0), (0, 1, 0),
                        (0, 0, -1), (-1, 0, -1), (-1, 1, -1), (0, 1, -1)])
        ney = v(ey) - proj(self._avg4(ex, mX, Y), v(ey), self._avg4(ez, Y, mZ),
                           R(0.5) * (v(bx) + v(bx, *mZ)), bya, R(0.5) * (v(bz) + v(bz, *mX)), bya)
        bza = avg8(bz, [(0, 0, 0), (-1, 0, 0), (-1, -1, 0), (0, -1, 0),
                        (0, 0, 1), (-1, 0, 1), (-1, -1, 1), (0, -1, 1)])
        nez = v(ez) - proj(self._avg4(ex, mX, Z), self._avg4(ey, mY, Z), v(ez),
                           R(0.5) * (v(bx) + v(bx, *mY)), R(0.5) * (v(by) + v(by, *mX)), bza, bza)
        v(ex)[...] = nex
        v(ey)[...] = ney
        v(ez)[...] = nez

    def exchange(self, b0=False):
        """A ghost is written iff every axis on which it lies outside the
        interior is periodic; it takes the value of the wrapped interior cell."""
        sx, sy, sz = self.s
        axes = []
        for n, b in ((sz, self.bnd[2]), (sy, self.bnd[1]), (sx, self.bnd[0])):
            idx = np.arange(-NG, n + NG)
            out = (idx < 0) | (idx >= n)
            src = np.where(idx < 0, idx + n, np.where(idx >= n, idx - n, idx)) + NG
            axes.append((src, out, b == 1))
        (zs, zo, zp), (ys, yo, yp), (xs, xo, xp) = axes
        Zo, Yo, Xo = zo[:, None, None], yo[None, :, None], xo[None, None, :]
        ghost = Zo | Yo | Xo
        blocked = (Zo & (not zp)) | (Yo & (not yp)) | (Xo & (not xp))
        fill = ghost & ~blocked
        for a in (FIELDS if b0 else FIELDS[:6]):
            A = self.f[a]
            W = A[np.ix_(zs, ys, xs)]
            A[fill] = W[fill]

    def init_rk_step(self):
        self.fn = {n: self.f[n].copy() for n in FIELDS[:6]}

    def rk3_stage(self, c1, c2, c3):
        self.compute_rho()
        self.push()
        self.update(c1, c2, c3)

    def step(self, nsteps=1):
        R = self.R
        coeffs = ((1.0, 0.0, 1.0), (R(3.0) / R(4.0), R(1.0) / R(4.0), R(1.0) / R(4.0)),
                  (R(1.0) / R(3.0), R(2.0) / R(3.0), R(2.0) / R(3.0)))
        for _ in range(nsteps):
            self.init_rk_step()
            for c in coeffs:
                self.rk3_stage(*c)
                self.exchange()
                self.clean()
                self.exchange()
