"""TEST INFRASTRUCTURE ONLY — numpy restatement of writeOutput's field datasets.

Follows src/io/write_output.F90:270-294 (output nodes of a meshblock for
output_istep) and :336-413 (the twelve datasets), src/tools/helpers.F90:93-257
(interpFromEdges / interpFromFaces, evaluated at offset 0 as the writer calls
them), and the userOutput hooks (user/user_psr.F90:387-398,
user/user_uniform.F90:151-173, user/user_loop.F90:168-179).  var1 is rho of
the given E at the node's cell (the reference writes its rho work array).
Fields are ghosted arrays indexed A[k+2, j+2, i+2]; every operation is one
numpy operation in the array's dtype, associated as in the Fortran source.
"""
import numpy as np

NG = 2
VARS = ("ex", "ey", "ez", "bx", "by", "bz", "var1", "var2", "var3", "xx", "yy", "zz")


def node_axis(x0, s, istep):
    """First node and node count along one axis (write_output.F90:272-293)."""
    a = -(-x0 // istep)
    b = -(-(x0 + s) // istep)
    first = a * istep - x0
    last = (b - 1) * istep - x0
    return first, ((last - first) // istep + 1) if last >= first else 0


def _blend(c000, c100, c010, c110, c001, c101, c011, c111, d):
    one = d.dtype.type(1)
    dx = dy = dz = d
    c00 = c000 * (one - dx) + c100 * dx
    c10 = c010 * (one - dx) + c110 * dx
    c0 = c00 * (one - dy) + c10 * dy
    c01 = c001 * (one - dx) + c101 * dx
    c11 = c011 * (one - dx) + c111 * dx
    c1 = c01 * (one - dy) + c11 * dy
    return c0 * (one - dz) + c1 * dz


def node_output(f, size, istep, offset=(0, 0, 0), gsize=None, uniform=False):
    """The twelve datasets, each (nz, ny, nx), for ghosted fields f (dict)."""
    sx, sy, sz = size
    x0, y0, z0 = offset
    gsx, gsy, gsz = gsize or size
    R = f["ex"].dtype.type
    i0, nx = node_axis(x0, sx, istep)
    j0, ny = node_axis(y0, sy, istep)
    k0, nz = node_axis(z0, sz, istep)
    ii = i0 + istep * np.arange(nx)
    jj = j0 + istep * np.arange(ny)
    kk = k0 + istep * np.arange(nz)

    def at(A, di, dj, dk):
        return A[np.ix_(kk + NG + dk, jj + NG + dj, ii + NG + di)]

    h, q, z = R(0.5), R(0.25), np.asarray(R(0))
    ex, ey, ez, bx, by, bz = (f[n] for n in ("ex", "ey", "ez", "bx", "by", "bz"))
    out = {}
    # interpFromEdges (helpers.F90:115-159)
    X = lambda di, dj, dk: at(ex, di, dj, dk)
    out["ex"] = _blend(h * (X(0, 0, 0) + X(-1, 0, 0)), h * (X(0, 0, 0) + X(1, 0, 0)),
                       h * (X(0, 1, 0) + X(-1, 1, 0)), h * (X(0, 1, 0) + X(1, 1, 0)),
                       h * (X(0, 0, 1) + X(-1, 0, 1)), h * (X(0, 0, 1) + X(1, 0, 1)),
                       h * (X(0, 1, 1) + X(-1, 1, 1)), h * (X(0, 1, 1) + X(1, 1, 1)), z)
    Y = lambda di, dj, dk: at(ey, di, dj, dk)
    out["ey"] = _blend(h * (Y(0, 0, 0) + Y(0, -1, 0)), h * (Y(1, 0, 0) + Y(1, -1, 0)),
                       h * (Y(0, 0, 0) + Y(0, 1, 0)), h * (Y(1, 0, 0) + Y(1, 1, 0)),
                       h * (Y(0, 0, 1) + Y(0, -1, 1)), h * (Y(1, 0, 1) + Y(1, -1, 1)),
                       h * (Y(0, 0, 1) + Y(0, 1, 1)), h * (Y(1, 0, 1) + Y(1, 1, 1)), z)
    Z = lambda di, dj, dk: at(ez, di, dj, dk)
    out["ez"] = _blend(h * (Z(0, 0, 0) + Z(0, 0, -1)), h * (Z(1, 0, 0) + Z(1, 0, -1)),
                       h * (Z(0, 1, 0) + Z(0, 1, -1)), h * (Z(1, 1, 0) + Z(1, 1, -1)),
                       h * (Z(0, 0, 0) + Z(0, 0, 1)), h * (Z(1, 0, 0) + Z(1, 0, 1)),
                       h * (Z(0, 1, 0) + Z(0, 1, 1)), h * (Z(1, 1, 0) + Z(1, 1, 1)), z)
    # interpFromFaces (helpers.F90:184-256)
    A = lambda di, dj, dk: at(bx, di, dj, dk)
    out["bx"] = _blend(q * (((A(0, 0, 0) + A(0, -1, 0)) + A(0, 0, -1)) + A(0, -1, -1)),
                       q * (((A(1, 0, 0) + A(1, -1, 0)) + A(1, 0, -1)) + A(1, -1, -1)),
                       q * (((A(0, 0, 0) + A(0, 1, 0)) + A(0, 0, -1)) + A(0, 1, -1)),
                       q * (((A(1, 0, 0) + A(1, 0, -1)) + A(1, 1, -1)) + A(1, 1, 0)),
                       q * (((A(0, 0, 0) + A(0, 0, 1)) + A(0, -1, 0)) + A(0, -1, 1)),
                       q * (((A(1, 0, 0) + A(1, 0, 1)) + A(1, -1, 0)) + A(1, -1, 1)),
                       q * (((A(0, 0, 0) + A(0, 1, 0)) + A(0, 1, 1)) + A(0, 0, 1)),
                       q * (((A(1, 0, 0) + A(1, 1, 0)) + A(1, 1, 1)) + A(1, 0, 1)), z)
    B = lambda di, dj, dk: at(by, di, dj, dk)
    out["by"] = _blend(q * (((B(-1, 0, -1) + B(-1, 0, 0)) + B(0, 0, -1)) + B(0, 0, 0)),
                       q * (((B(0, 0, -1) + B(0, 0, 0)) + B(1, 0, -1)) + B(1, 0, 0)),
                       q * (((B(-1, 1, -1) + B(-1, 1, 0)) + B(0, 1, -1)) + B(0, 1, 0)),
                       q * (((B(0, 1, -1) + B(0, 1, 0)) + B(1, 1, -1)) + B(1, 1, 0)),
                       q * (((B(-1, 0, 0) + B(-1, 0, 1)) + B(0, 0, 0)) + B(0, 0, 1)),
                       q * (((B(0, 0, 0) + B(0, 0, 1)) + B(1, 0, 0)) + B(1, 0, 1)),
                       q * (((B(-1, 1, 0) + B(-1, 1, 1)) + B(0, 1, 0)) + B(0, 1, 1)),
                       q * (((B(0, 1, 0) + B(0, 1, 1)) + B(1, 1, 0)) + B(1, 1, 1)), z)
    C = lambda di, dj, dk: at(bz, di, dj, dk)
    out["bz"] = _blend(q * (((C(-1, -1, 0) + C(-1, 0, 0)) + C(0, -1, 0)) + C(0, 0, 0)),
                       q * (((C(0, -1, 0) + C(0, 0, 0)) + C(1, -1, 0)) + C(1, 0, 0)),
                       q * (((C(-1, 0, 0) + C(-1, 1, 0)) + C(0, 0, 0)) + C(0, 1, 0)),
                       q * (((C(0, 0, 0) + C(0, 1, 0)) + C(1, 0, 0)) + C(1, 1, 0)),
                       q * (((C(-1, -1, 1) + C(-1, 0, 1)) + C(0, -1, 1)) + C(0, 0, 1)),
                       q * (((C(0, -1, 1) + C(0, 0, 1)) + C(1, -1, 1)) + C(1, 0, 1)),
                       q * (((C(-1, 0, 1) + C(-1, 1, 1)) + C(0, 0, 1)) + C(0, 1, 1)),
                       q * (((C(0, 0, 1) + C(0, 1, 1)) + C(1, 0, 1)) + C(1, 1, 1)), z)
    # userOutput var1 = rho (field_solver.F90:54-62 at the node's cell)
    out["var1"] = ((X(0, 0, 0) - X(-1, 0, 0)) + (Y(0, 0, 0) - Y(0, -1, 0))) + (Z(0, 0, 0) - Z(0, 0, -1))
    shp = (nz, ny, nx)
    if uniform:  # user_uniform.F90:159-170 at the raw cell values
        e_x, e_y, e_z = X(0, 0, 0), Y(0, 0, 0), Z(0, 0, 0)
        b_x, b_y, b_z = A(0, 0, 0), B(0, 0, 0), C(0, 0, 0)
        t1 = -b_z * e_x + b_x * e_z
        t2 = b_z * e_y - b_y * e_z
        v = np.sqrt(t1 * t1 + t2 * t2)
        xs = np.asarray((x0 + ii).astype(np.float32), R)[None, None, :]
        ys = np.asarray((y0 + jj).astype(np.float32), R)[None, :, None]
        d1 = xs - h * R(gsx)
        d2 = ys - h * R(gsy)
        tiny = R(np.float32(1e-7)) if R is np.float32 else R(1e-7)
        v = v / np.sqrt((d1 * d1 + d2 * d2) + tiny)
        out["var2"] = v / ((b_x * b_x + b_y * b_y) + b_z * b_z)
    else:
        out["var2"] = np.zeros(shp, R)
    out["var3"] = np.zeros(shp, R)
    out["xx"] = np.broadcast_to(np.asarray((x0 + ii).astype(np.float32), R)[None, None, :], shp).copy()
    out["yy"] = np.broadcast_to(np.asarray((y0 + jj).astype(np.float32), R)[None, :, None], shp).copy()
    out["zz"] = np.broadcast_to(np.asarray((z0 + kk).astype(np.float32), R)[:, None, None], shp).copy()
    return out
