"""Synthetic workloads of the benchmark (seeded; no dataset is involved).

Each workload is a uniform background B plus plane-wave modes, built on the
device by `Solver.init_waves` (include/ffe.h: ffe_init_waves).  A mode row is
(K[3], phi, a, u[3], n[3]):
    dB(x) = -a sin(K.x + phi) u,   dE(x) = -n x dB(x).
u is the unit vector along Kd x p, with Kd = 2 sin(K/2) the discrete
wavenumber of the Yee grid's one-cell differences and p the direction of the
wave's vector potential, so that dB is the exact discrete curl of
p (a/|Kd x p|) cos(K.x + phi) and its discrete divergence vanishes.

  alfven_packet : Bx = 1, dBy = A sin(2 pi x / L + phi) at By's points,
                  E = -x^ x dB (v along x at c); periodic.
  random_modes  : Bz = 1 plus `n` modes with integer wavevectors
                  0 < |k| <= kmax, amplitudes U[0, amax]; the first half
                  Alfven (dB || k x z^, E = -z^ x dB), the rest fast
                  (dB perpendicular to k in the k-z plane, E = -k^ x dB).
"""
import numpy as np


def _unit(v):
    n = np.linalg.norm(v)
    return v / n


def mode_row(kvec_int, size, phi, amp, p_dir, n_dir):
    K = 2.0 * np.pi * np.asarray(kvec_int, float) / np.asarray(size, float)
    Kd = 2.0 * np.sin(K / 2.0)
    u = _unit(np.cross(Kd, np.asarray(p_dir, float)))
    return np.concatenate([K, [phi, amp], u, np.asarray(n_dir, float)])


def alfven_packet(size=(64, 64, 64), seed=0, amp=0.1):
    """Background (1,0,0), dBy = amp sin(2 pi x/Lx + phi) (x at By's staggered point)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    phi = 2.0 * np.pi * rng.random()
    row = mode_row((1, 0, 0), size, phi, amp, p_dir=(0, 0, 1), n_dir=(1, 0, 0))
    return np.array([1.0, 0.0, 0.0]), row[None, :], {"phi": phi}


def random_modes(size=(512, 512, 512), seed=1, n=32, kmax=8, amax=0.02):
    rng = np.random.Generator(np.random.PCG64(seed))
    rows = []
    while len(rows) < n:
        k = rng.integers(-kmax, kmax + 1, size=3)
        if k[0] == 0 and k[1] == 0:        # needs a component across Bz for the polarisation
            continue
        if np.dot(k, k) > kmax * kmax:
            continue
        amp = amax * rng.random()
        phi = 2.0 * np.pi * rng.random()
        K = 2.0 * np.pi * k / np.asarray(size, float)
        Kd = 2.0 * np.sin(K / 2.0)
        if len(rows) < n // 2:            # Alfven: A || z^, dB || Kd x z^
            rows.append(mode_row(k, size, phi, amp, p_dir=(0, 0, 1), n_dir=(0, 0, 1)))
        else:                             # fast: A || Kd x z^, dB || Kd x (Kd x z^)
            p = _unit(np.cross(Kd, (0, 0, 1)))
            rows.append(mode_row(k, size, phi, amp, p_dir=p, n_dir=_unit(K)))
    return np.array([0.0, 0.0, 1.0]), np.array(rows), {"n": n, "kmax": kmax, "amax": amax}


def host_waves(size, bg, modes, dtype=np.float64):
    """The same fields computed with numpy (ghosted arrays), for small grids."""
    sx, sy, sz = size
    ng = 2
    i = np.arange(-ng, sx + ng, dtype=np.float64)[None, None, :]
    j = np.arange(-ng, sy + ng, dtype=np.float64)[None, :, None]
    k = np.arange(-ng, sz + ng, dtype=np.float64)[:, None, None]
    shape = (sz + 2 * ng, sy + 2 * ng, sx + 2 * ng)
    offs = {"ex": (0.5, 0, 0), "ey": (0, 0.5, 0), "ez": (0, 0, 0.5),
            "bx": (0, 0.5, 0.5), "by": (0.5, 0, 0.5), "bz": (0.5, 0.5, 0)}
    out = {}
    for c, name in enumerate(("ex", "ey", "ez", "bx", "by", "bz")):
        ox, oy, oz = offs[name]
        v = np.full(shape, bg[c - 3] if c >= 3 else 0.0)
        for m in modes:
            K, phi, a, u, n = m[0:3], m[3], m[4], m[5:8], m[8:11]
            # sin of a sum of separable phases, through complex exponentials
            s = (np.exp(1j * (K[2] * (k + oz) + phi)) * np.exp(1j * K[1] * (j + oy)) *
                 np.exp(1j * K[0] * (i + ox))).imag
            db = [-a * s * u[0], -a * s * u[1], -a * s * u[2]]
            if c < 3:
                cr = [n[1] * db[2] - n[2] * db[1], n[2] * db[0] - n[0] * db[2], n[0] * db[1] - n[1] * db[0]]
                v = v - cr[c]
            else:
                v = v + db[c - 3]
        out[name] = v.astype(dtype)
    return out
