"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Bars:
  * staged and fused-exact paths: bit-exact with the oracle in FP64, FP32 and
    FP32C (no multiply-add contraction on either side, IEEE division/sqrt);
    the user boundary conditions use tanh/exp, compared with tolerances;
  * fused fast path (contraction on): FP64 rel. L2 <= 1e-12 and FP32/FP32C
    rel. L2 <= 1e-5 against the oracle of the same precision after 20 steps.
"""
import numpy as np
import pytest

import ffe
from ffe.workloads import random_modes, alfven_packet, host_waves
from conftest import rel_l2, rel_linf
from test_oracle_cpu import random_fields

pytestmark = pytest.mark.gpu

F6 = ("ex", "ey", "ez", "bx", "by", "bz")
PRECS = [ffe.FP64, ffe.FP32, ffe.FP32C, ffe.FP32CD]
BNDS = [(1, 1, 1), (0, 0, 0), (2, 2, 2), (1, 1, 0)]


def dtype_of(prec):
    return np.float64 if prec == ffe.FP64 else np.float32


def pair(oracle_mod, size, prec, bnd, path, seed=3, b0=True, **kw):
    d = ffe.make_desc(size, precision=prec, boundary=bnd, absorb_buff=3, path=path, **kw)
    g = ffe.Solver(d)
    o = oracle_mod.Oracle(d)
    f = random_fields(size, dtype_of(prec), seed=seed, e_scale=0.7, b0=b0)
    g.set_fields(f)
    o.set_fields(f)
    return g, o


def eb_errors(g, o):
    """Relative L2 of E = (ex, ey, ez) and of B = (bx, by, bz) over the ghosted arrays."""
    out = {}
    for name, comps in (("E", F6[:3]), ("B", F6[3:])):
        a = np.concatenate([g.download(k).astype(np.float64).ravel() for k in comps])
        b = np.concatenate([o.download(k).astype(np.float64).ravel() for k in comps])
        out[name] = rel_l2(a, b)
    return out


def assert_same(g, o, names=F6, exact=True, tol=0.0):
    if not exact:
        err = eb_errors(g, o)
        assert err["E"] <= tol and err["B"] <= tol, err
        return
    for k in names:
        a, b = g.download(k), o.download(k)
        bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
        assert not bad.any(), (k, int(bad.sum()), np.argwhere(bad)[:3].tolist())


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("bnd", BNDS)
def test_staged_procedures_bit_exact(oracle_mod, prec, bnd):
    """Each reference procedure alone, including the work arrays it writes."""
    g, o = pair(oracle_mod, (13, 9, 7), prec, bnd, ffe.PATH_STAGED)
    for s in (g, o):
        s.exchangeFields(True)
        s.initRKstep()
    assert_same(g, o, F6 + ("enx", "bnz", "b0x", "b0z"))
    for s in (g, o):
        s.computeRho()
    assert_same(g, o, ("rho",))
    for s in (g, o):
        s.rk3Push()
    assert_same(g, o, ("dex", "dey", "dez", "dbx", "dby", "dbz"))
    for s in (g, o):
        s.rk3Update(0.75, 0.25, 0.25)
    assert_same(g, o)
    for s in (g, o):
        s.exchangeFields()
        s.cleanEpar()
    assert_same(g, o, F6 + ("dex", "dey", "dez"))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("bnd", BNDS)
@pytest.mark.parametrize("path", [ffe.PATH_STAGED, ffe.PATH_FUSED_EXACT])
def test_steps_bit_exact(oracle_mod, prec, bnd, path):
    g, o = pair(oracle_mod, (37, 19, 11), prec, bnd, path)
    for s in (g, o):
        s.mainloop_prologue()
        s.mainloop(3, 0)
    g.synchronize()
    assert_same(g, o)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("bnd", [(1, 1, 1), (2, 2, 2), (0, 0, 0), (1, 1, 0), (0, 1, 1)])
def test_fused_fast_matches_oracle(oracle_mod, prec, bnd):
    size = (40, 24, 20)
    # without the clamp the absorbing corners amplify every rounding difference
    # by ~100 per stage, and the clamped shell zeroes B there (0/0 in the
    # cleaning), so the fast path is compared with both opt-in flags on
    flags = ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY if bnd[0] == 2 else 0
    d = ffe.make_desc(size, precision=prec, boundary=bnd, absorb_buff=4, path=ffe.PATH_FUSED, flags=flags)
    g = ffe.Solver(d)
    o = oracle_mod.Oracle(d)
    bg, modes, _ = random_modes(size, seed=4, n=8, kmax=3, amax=0.05)
    g.init_waves(bg, modes)
    f = g.fields()
    o.set_fields(f)
    for s in (g, o):
        s.mainloop_prologue()
        s.mainloop(20, 0)
    tol = 1e-12 if prec == ffe.FP64 else 1e-5
    assert_same(g, o, exact=False, tol=tol)


def test_fused_tiles_cover_ragged_sizes(oracle_mod):
    """Sizes that are not multiples of the 32x8 tile or of the z chunk."""
    for size in [(33, 9, 5), (70, 17, 13), (2, 2, 2), (5, 31, 3)]:
        for bnd in [(1, 1, 1), (1, 0, 1), (0, 1, 0)]:
            g, o = pair(oracle_mod, size, ffe.FP64, bnd, ffe.PATH_FUSED_EXACT, b0=False)
            for s in (g, o):
                s.mainloop_prologue()
                s.mainloop(2, 0)
            assert_same(g, o)


@pytest.mark.parametrize("prec", [ffe.FP32, ffe.FP32C])
def test_plain_fp32_tiles_cover_ragged_sizes(oracle_mod, prec):
    """The plain FP32 variant's 32 x 12 tile (two cells per thread) on sizes
    that are not multiples of it, below it, or leave one row of a pair:
    the fused-exact path bit for bit, the fast path within 1e-5."""
    sizes = [(33, 9, 5), (70, 17, 13), (2, 2, 2), (5, 31, 3), (37, 25, 14), (64, 13, 9), (31, 11, 40)]
    for size in sizes:
        for bnd in [(1, 1, 1), (1, 0, 1), (0, 1, 0), (0, 0, 0)]:
            g, o = pair(oracle_mod, size, prec, bnd, ffe.PATH_FUSED_EXACT, b0=False)
            for s in (g, o):
                s.mainloop_prologue()
                s.mainloop(2, 0)
            assert_same(g, o)
            g.close()
            d = ffe.make_desc(size, precision=prec, boundary=bnd, path=ffe.PATH_FUSED)
            h = ffe.Solver(d)
            bg, modes, _ = random_modes(size, seed=5, n=6, kmax=2, amax=0.05)
            h.init_waves(bg, modes)
            q = oracle_mod.Oracle(d)
            q.set_fields(h.fields())
            for s in (h, q):
                s.mainloop_prologue()
                s.mainloop(3, 0)
            assert_same(h, q, exact=False, tol=1e-5)
            h.close()


@pytest.mark.parametrize("prec", PRECS)
def test_waves_init_matches_host(prec):
    size = (20, 12, 10)
    bg, modes, _ = random_modes(size, seed=9, n=5, kmax=3, amax=0.1)
    g = ffe.Solver(ffe.make_desc(size, precision=prec))
    g.init_waves(bg, modes)
    ref = host_waves(size, bg, modes, np.float64)
    tol = 1e-13 if prec == ffe.FP64 else 1e-7
    for k in F6:
        a = g.download(k).astype(np.float64)
        assert np.max(np.abs(a - ref[k])) <= tol * max(1.0, np.max(np.abs(ref[k]))), k


@pytest.mark.parametrize("setup,bnd,params,flags", [
    (ffe.SETUP_PSR, (0, 0, 0), (5.0, 30.0, 200.0, 1.0), 0),
    (ffe.SETUP_PSR, (2, 2, 2), (5.0, 60.0, 150.0, 10.0), ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY),
    (ffe.SETUP_UNIFORM, (1, 1, 0), (10.0, 0.4, 5.0, 0.3), 0),
    (ffe.SETUP_LOOP, (1, 1, 0), (4.0, 1.0, 1.0, 0.5, 5.0, 0.3), 0),
])
@pytest.mark.parametrize("prec", PRECS)
def test_user_setups(oracle_mod, setup, bnd, params, flags, prec):
    size = (24, 24, 24)
    d = ffe.make_desc(size, precision=prec, boundary=bnd, setup=setup, params=params, absorb_buff=4,
                      flags=flags)
    g = ffe.Solver(d)
    o = oracle_mod.Oracle(d)
    for s in (g, o):
        s.userInitialize()
    # initial fields: sqrt and division only -> bit-exact
    assert_same(g, o, F6 + ("b0x", "b0y", "b0z"))
    for s in (g, o):
        s.mainloop_prologue()
        s.mainloop(4, 0)
    # tanh / exp of the boundary conditions round differently on the GPU
    tol = 1e-12 if prec == ffe.FP64 else 2e-5
    assert_same(g, o, exact=False, tol=tol)
    assert g.check_finite()


def test_check_finite_flags_nan():
    size = (8, 8, 8)
    g = ffe.Solver(ffe.make_desc(size, precision=ffe.FP32))
    a = np.zeros(g.shape, np.float32)
    assert g.check_finite()
    a[5, 5, 5] = np.nan
    g.upload("ey", a)
    assert not g.check_finite()


def test_errors_are_reported():
    with pytest.raises(ffe.FFEError) as e:
        ffe.Solver(ffe.make_desc((1, 8, 8)))
    assert "ghost zones" in str(e.value)
    g = ffe.Solver(ffe.make_desc((8, 8, 8), setup=ffe.SETUP_PSR, params=(2.0, 10.0, 100.0),
                                 path=ffe.PATH_FUSED))
    with pytest.raises(ffe.FFEError):
        g.mainloop(1)
    with pytest.raises(ffe.FFEError):
        g.upload("ex", np.zeros((3, 3, 3), np.float32))


def test_step_paths_and_launch_counts():
    g = ffe.Solver(ffe.make_desc((16, 16, 16)))  # stage kernel + ghost fill, three stages
    assert g.step_path() == ffe.PATH_FUSED and g.step_launches() == 6
    g = ffe.Solver(ffe.make_desc((16, 16, 16), boundary=(2, 2, 2)))
    assert g.step_path() == ffe.PATH_FUSED
    g = ffe.Solver(ffe.make_desc((16, 16, 16), boundary=(1, 1, 0)))
    assert g.step_path() == ffe.PATH_FUSED
    g = ffe.Solver(ffe.make_desc((16, 16, 16), setup=ffe.SETUP_PSR, params=(3.0, 10.0, 100.0),
                                 boundary=(0, 0, 0)))
    assert g.step_path() == ffe.PATH_FUSED and g.step_launches() == 12
    g = ffe.Solver(ffe.make_desc((16, 16, 16), setup=ffe.SETUP_UNIFORM, params=(8.0, 0.4, 5.0, 0.3),
                                 boundary=(1, 1, 0)))
    assert g.step_path() == ffe.PATH_FUSED and g.step_launches() == 3 * (1 + 1 + 2)
    g = ffe.Solver(ffe.make_desc((16, 16, 16), setup=ffe.SETUP_LOOP, params=(4.0, 1.0, 1.0, 0.5, 5.0, 0.3),
                                 boundary=(1, 1, 0)))
    assert g.step_path() == ffe.PATH_STAGED


def test_large_grid_fp32_vs_fp64_gpu():
    """256^3 random modes, 10 steps: FP32 and FP32C stay within 1e-5 of FP64."""
    size = (256, 256, 256)
    bg, modes, _ = random_modes(size, seed=1, n=32, kmax=8, amax=0.02)
    res = {}
    for prec in PRECS:
        g = ffe.Solver(ffe.make_desc(size, precision=prec))
        g.init_waves(bg, modes)
        g.mainloop_prologue()
        g.mainloop(10, 0)
        res[prec] = {k: ffe.interior(g.download(k)).astype(np.float64) for k in F6}
        g.close()
    for prec in (ffe.FP32, ffe.FP32C):
        eb = np.concatenate([res[prec][k].ravel() for k in F6])
        e64 = np.concatenate([res[ffe.FP64][k].ravel() for k in F6])
        assert rel_l2(eb, e64) < 1e-5, (prec, rel_l2(eb, e64))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("bnd,flags", [((0, 0, 0), 0),
                                       ((2, 2, 2), ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY),
                                       ((2, 2, 2), ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY |
                                        ffe.FLAG_ABSORB_TRUE_Y)])
def test_psr_fused_equals_staged(prec, bnd, flags):
    """The rotating-conductor BC on the fused path (fused stage + box fix-up)
    gives the staged path's result bit for bit when both skip contraction."""
    size = (40, 36, 34)
    prm = (5.0, 30.0, 120.0, 1.0)
    res = {}
    for path in (ffe.PATH_STAGED, ffe.PATH_FUSED_EXACT):
        g = ffe.Solver(ffe.make_desc(size, precision=prec, boundary=bnd, setup=ffe.SETUP_PSR, params=prm,
                                     absorb_buff=5, flags=flags, path=path))
        g.userInitialize()
        g.mainloop_prologue()
        g.mainloop(3, 7)
        res[path] = g.fields()
    for k in F6:
        a, b = res[ffe.PATH_STAGED][k], res[ffe.PATH_FUSED_EXACT][k]
        bad = a != b
        assert not bad.any(), (k, int(bad.sum()), np.argwhere(bad)[:4].tolist(),
                               float(np.nanmax(np.abs(a.astype(float) - b))))


def test_psr_fused_fast_matches_oracle(oracle_mod):
    size = (40, 36, 34)
    d = ffe.make_desc(size, precision=ffe.FP64, boundary=(0, 0, 0), setup=ffe.SETUP_PSR,
                      params=(5.0, 30.0, 120.0, 1.0), path=ffe.PATH_FUSED)
    g = ffe.Solver(d)
    o = oracle_mod.Oracle(d)
    for s in (g, o):
        s.userInitialize()
        s.mainloop_prologue()
        s.mainloop(4, 0)
    assert_same(g, o, exact=False, tol=1e-12)


@pytest.mark.parametrize("prec", PRECS)
def test_uniform_fused_equals_staged(prec):
    """The twisted-footpoint BC applied inside the fused kernel (plus the
    ghost-plane pass) gives the staged path's result bit for bit."""
    size = (40, 33, 21)
    prm = (8.0, 0.4, 5.0, 0.3)
    res = {}
    for path in (ffe.PATH_STAGED, ffe.PATH_FUSED_EXACT):
        g = ffe.Solver(ffe.make_desc(size, precision=prec, boundary=(1, 1, 0), setup=ffe.SETUP_UNIFORM,
                                     params=prm, path=path))
        g.userInitialize()
        g.mainloop_prologue()
        g.mainloop(4, 3)
        res[path] = g.fields()
    for k in F6:
        a, b = res[ffe.PATH_STAGED][k], res[ffe.PATH_FUSED_EXACT][k]
        assert np.array_equal(a, b), (k, int(np.sum(a != b)), np.argwhere(a != b)[:3].tolist())


@pytest.mark.parametrize("path", [ffe.PATH_STAGED, ffe.PATH_FUSED_EXACT])
def test_true_y_absorber_bit_exact(oracle_mod, path):
    """FFE_FLAG_ABSORB_TRUE_Y on both exact paths against the oracle."""
    size = (30, 26, 22)
    flags = ffe.FLAG_ABSORB_CLAMP | ffe.FLAG_CLEAN_TINY | ffe.FLAG_ABSORB_TRUE_Y
    d = ffe.make_desc(size, precision=ffe.FP32, boundary=(2, 2, 2), absorb_buff=6, flags=flags, path=path)
    g = ffe.Solver(d)
    o = oracle_mod.Oracle(d)
    bg, modes = random_modes(size, seed=4, n=6, kmax=3, amax=0.05)[:2]
    f = host_waves(size, bg, modes, np.float32)
    for s in (g, o):
        s.set_fields(f)
        s.mainloop_prologue()
        s.mainloop(3, 0)
    assert_same(g, o)
