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
  abc_nulls     : the ABC field (magnetic nulls in equilibrium) plus small
                  seeded waves.
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


def abc_nulls(size=(32, 32, 32), seed=3, amp=1e-3, n=6):
    """A field with magnetic nulls in equilibrium plus small waves: the ABC
    field with A = B = C = 1 (Bx = sin kz + cos ky, By = sin kx + cos kz,
    Bz = sin ky + cos kx, k = 2 pi / L; a Beltrami field, curl B = k B, with
    eight nulls per period; under the drift-only current the E that curl B
    drives lies along B and the cleaning removes it, so the field stands)
    and `n` seeded waves of amplitude up to `amp` (random_modes without the
    background).  Cubic, periodic."""
    L = size[0]
    k = 2.0 * np.pi / L

    def static(K, phi, u):  # dB = -sin(K.x + phi) u, no E
        return np.concatenate([K, [phi, 1.0], u, [0.0, 0.0, 0.0]])

    rows = [static((0, 0, k), np.pi, (1, 0, 0)), static((0, k, 0), -np.pi / 2, (1, 0, 0)),
            static((k, 0, 0), np.pi, (0, 1, 0)), static((0, 0, k), -np.pi / 2, (0, 1, 0)),
            static((0, k, 0), np.pi, (0, 0, 1)), static((k, 0, 0), -np.pi / 2, (0, 0, 1))]
    _, waves, _ = random_modes(size, seed=seed, n=n, kmax=3, amax=amp)
    return np.zeros(3), np.vstack([rows, waves]), {"amp": amp, "n": n}


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


# ---- many-grid workloads: batched boxes and served pulsar runs --------------
# A run spec is a dict: kind ("packet", "tube" or "psr"), size (sx, sy, sz),
# precision and the kind's parameters; build_solver turns it into a ready
# Solver (fields initialised, main-loop prologue done).

def tube_params(size, beta):
    """user_uniform parameters (L0, r_L0, t0, beta) of a footpoint-twisted flux
    tube: r0 = min(sx, sy) / 8, t0 = 50 steps."""
    return (min(size[0], size[1]) / 8.0, 1.0, 50.0, float(beta))


def psr_params(side, incl_deg, cc=0.45):
    """user_psr parameters (radius, inclination, period, mu scale) of a served
    pulsar run: R = side / 10, light cylinder 5 R, period 2 pi R_LC / c."""
    radius = side / 10.0
    period = 2.0 * np.pi * (5.0 * radius) / cc
    return (radius, float(incl_deg), period, 1.0)


def batch_boxes(n=64, seed=3, lo=48, hi=160, kind="mixed"):
    """The batched workload: n boxes with sides uniform in [lo, hi] per axis;
    the first half Alfven packets (periodic), the rest twisted flux tubes
    (periodic x, y; open z) with twist amplitude U[0.1, 0.5].  kind="packet":
    all Alfven packets."""
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = []
    for b in range(n):
        size = tuple(int(v) for v in rng.integers(lo, hi + 1, size=3))
        if b < n // 2 or kind == "packet":
            specs.append({"kind": "packet", "size": size, "seed": int(rng.integers(1 << 30))})
        else:
            specs.append({"kind": "tube", "size": size, "beta": float(rng.uniform(0.1, 0.5))})
    return specs


def served_requests(n, seed=4, rate=20.0, lo=96, hi=256, steps=(200, 2000), shell="true_y"):
    """The served workload: Poisson arrivals (mean `rate` per second) of pulsar
    runs, cubic side uniform in [lo, hi], inclination U[0, 90] degrees, step
    counts uniform in `steps`.  Returns dicts with an arrival time (s).
    shell: "true_y" (the absorbing shell measured with each cell's own y,
    FFE_FLAG_ABSORB_TRUE_Y) or "reference" (jg = i + y0, whose y faces are
    not damped and are numerically unstable for this setup)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for r in range(n):
        t += rng.exponential(1.0 / rate)
        side = int(rng.integers(lo, hi + 1))
        out.append({"kind": "psr", "size": (side, side, side), "incl": float(rng.uniform(0.0, 90.0)),
                    "steps": int(rng.integers(steps[0], steps[1] + 1)), "arrival": t, "id": r, "shell": shell})
    return out


def run_desc(spec, precision, path=None):
    """The descriptor of a run spec.  Pulsar runs use the clamped absorbing
    shell with TINY in the cleaning, and the true-y shell when
    spec["shell"] == "true_y"."""
    import ffe
    size = tuple(spec["size"])
    path = ffe.PATH_AUTO if path is None else path
    kind = spec["kind"]
    if kind == "packet":
        return ffe.make_desc(size, precision=precision, path=path)
    if kind == "tube":
        return ffe.make_desc(size, precision=precision, boundary=(ffe.PERIODIC, ffe.PERIODIC, ffe.OPEN),
                             setup=ffe.SETUP_UNIFORM, params=tube_params(size, spec["beta"]), path=path)
    if kind == "psr":
        side = size[0]
        buff = spec.get("absorb_buff", int(np.ceil(side * 48 / 512)))
        flags = ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY
        if spec.get("shell") == "true_y":
            flags |= ffe.FLAG_ABSORB_TRUE_Y
        return ffe.make_desc(size, precision=precision, boundary=(ffe.ABSORB,) * 3, absorb_buff=buff,
                             setup=ffe.SETUP_PSR, params=psr_params(side, spec["incl"]), path=path, flags=flags)
    raise ValueError("unknown run kind %r" % kind)


def init_run(s, spec):
    """Initial fields of a run spec on a Solver (or an oracle driven like one)
    and the main-loop prologue."""
    if spec["kind"] == "packet":
        bg, modes, _ = alfven_packet(tuple(spec["size"]), seed=spec.get("seed", 0), amp=spec.get("amp", 0.1))
        s.init_waves(bg, modes)
    else:
        s.userInitialize()
    s.mainloop_prologue()
    return s


def build_solver(spec, precision, path=None, lib_path=None):
    """A Solver for a run spec, initialised and past the main-loop prologue."""
    import ffe
    return init_run(ffe.Solver(run_desc(spec, precision, path), lib_path), spec)
