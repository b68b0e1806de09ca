"""Batched stepping (ffe_batch_*): many meshblocks of uneven sizes and setups
advanced by one launch per stage.  A member's result does not depend on the
other members of its batch (bit for bit), and equals its own single-grid run."""
import numpy as np
import pytest

import ffe
from ffe import workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu

F6 = ("ex", "ey", "ez", "bx", "by", "bz")

SPECS = [
    {"kind": "packet", "size": (37, 24, 30), "seed": 5},
    {"kind": "tube", "size": (40, 33, 21), "beta": 0.4},
    {"kind": "psr", "size": (44, 44, 44), "incl": 30.0, "absorb_buff": 5},
    {"kind": "packet", "size": (64, 17, 9), "seed": 6},
    {"kind": "tube", "size": (29, 48, 35), "beta": 0.2},
]


def make(specs, prec, path=None):
    return [workloads.build_solver(s, prec, path=path) for s in specs]


def fields(solvers):
    return [s.fields() for s in solvers]


def close(solvers):
    for s in solvers:
        s.close()


def tol_of(prec):
    return 1e-13 if prec == ffe.FP64 else 2e-6


def assert_equal_fields(a, b, exact=True, tol=0.0):
    for m, (fa, fb) in enumerate(zip(a, b)):
        if exact:
            for k in F6:
                bad = fa[k] != fb[k]
                assert not bad.any(), (m, k, int(bad.sum()), np.argwhere(bad)[:3].tolist())
        else:
            for grp in (("ex", "ey", "ez"), ("bx", "by", "bz")):
                x = np.concatenate([ffe.interior(fa[k]).ravel().astype(np.float64) for k in grp])
                y = np.concatenate([ffe.interior(fb[k]).ravel().astype(np.float64) for k in grp])
                assert rel_l2(x, y) <= tol, (m, grp, rel_l2(x, y))


@pytest.mark.parametrize("prec", [ffe.FP32, ffe.FP32C, ffe.FP64])
def test_member_alone_equals_member_in_the_mix(prec):
    """Each member's fields after a batched run are bit-identical to the same
    member run in a batch of its own (the serving requirement)."""
    mix = make(SPECS, prec)
    with ffe.Batch(mix) as b:
        b.step(6, step0=[3, 0, 11, 2, 7])
        b.synchronize()
    got = fields(mix)
    close(mix)
    for m, (spec, s0) in enumerate(zip(SPECS, [3, 0, 11, 2, 7])):
        alone = make([spec], prec)
        with ffe.Batch(alone) as b:
            b.step(6, step0=[s0])
            b.synchronize()
        assert_equal_fields([got[m]], fields(alone))
        close(alone)


@pytest.mark.parametrize("prec", [ffe.FP32, ffe.FP32C, ffe.FP64])
def test_batch_matches_single_grid_fused_path(prec):
    """The batched kernel against ffe_step of every member (same tile shape)."""
    a, b_ = make(SPECS, prec), make(SPECS, prec)
    with ffe.Batch(a) as b:
        b.step(5, step0=[0, 4, 9, 1, 0])
        b.synchronize()
    for s, s0 in zip(b_, [0, 4, 9, 1, 0]):
        s.mainloop(5, s0)
        s.synchronize()
    assert_equal_fields(fields(a), fields(b_), exact=False, tol=tol_of(prec))
    close(a)
    close(b_)


@pytest.mark.parametrize("prec", [ffe.FP32, ffe.FP32C])
@pytest.mark.parametrize("kind", ["packet", "psr"])
def test_one_variant_batch_equals_single_grid_bit_for_bit(kind, prec):
    """A batch whose grids all have one variant (plain packets; pulsars with
    the absorbing layer) runs the single-grid kernel body at tile height 8:
    every member equals its own single-grid run bit for bit."""
    if kind == "packet":
        specs = [{"kind": "packet", "size": (37, 24, 30), "seed": 5},
                 {"kind": "packet", "size": (64, 17, 9), "seed": 6},
                 {"kind": "packet", "size": (70, 41, 19), "seed": 7}]
    else:
        specs = [{"kind": "psr", "size": (44, 44, 44), "incl": 30.0, "absorb_buff": 5, "shell": "true_y"},
                 {"kind": "psr", "size": (52, 40, 36), "incl": 60.0, "absorb_buff": 5, "shell": "true_y"}]
    a, b_ = make(specs, prec), make(specs, prec)
    s0 = [0, 3, 7][:len(specs)]
    with ffe.Batch(a) as b:
        b.set_tiling(8, 0, False)
        b.step(4, step0=s0)
        b.synchronize()
    for s, k0 in zip(b_, s0):
        s.mainloop(4, k0)
        s.synchronize()
    assert_equal_fields(fields(a), fields(b_))
    close(a)
    close(b_)


def test_batch_fp64_matches_oracle(oracle_mod):
    """Three members (one per setup) from the same initial state: the batch on
    the GPU, each member alone in the oracle."""
    specs = SPECS[:3]
    sols = make(specs, ffe.FP64)
    oras = []
    for s in sols:
        o = oracle_mod.Oracle(s.desc)
        o.set_fields(s.fields(F6 + ("b0x", "b0y", "b0z")))
        oras.append(o)
    with ffe.Batch(sols) as b:
        b.step(3, step0=[0, 1, 2])
        b.synchronize()
    for spec, s, o, s0 in zip(specs, sols, oras, [0, 1, 2]):
        o.mainloop(3, s0)
        for grp in (("ex", "ey", "ez"), ("bx", "by", "bz")):
            x = np.concatenate([ffe.interior(s.download(k)).ravel() for k in grp])
            y = np.concatenate([ffe.interior(o.download(k)).ravel() for k in grp])
            assert rel_l2(x, y) <= 1e-12, (spec["kind"], grp, rel_l2(x, y))
    close(sols)


@pytest.mark.parametrize("tiling", [(8, 8, False), (8, 32, True), (8, 0, True)])
def test_plane_chunks_and_persistence_do_not_change_results(tiling):
    """Planes per block and persistent blocks only regroup the work items of
    one kernel: bit-identical results."""
    ref, alt = make(SPECS, ffe.FP32), make(SPECS, ffe.FP32)
    with ffe.Batch(ref) as b:
        b.step(4)
        b.synchronize()
    with ffe.Batch(alt) as b:
        b.set_tiling(*tiling)
        assert b.tiling() == {"tile_y": tiling[0], "planes": tiling[1], "persistent": tiling[2]}
        b.step(4)
        b.synchronize()
    assert_equal_fields(fields(ref), fields(alt))
    close(ref)
    close(alt)


@pytest.mark.parametrize("prec", [ffe.FP32, ffe.FP32C])
def test_tile_height_16(prec):
    ref, alt = make(SPECS, prec), make(SPECS, prec)
    with ffe.Batch(ref) as b:
        b.step(4)
        b.synchronize()
    with ffe.Batch(alt) as b:
        b.set_tiling(16, 0, False)
        b.step(4)
        b.synchronize()
    assert_equal_fields(fields(ref), fields(alt), exact=False, tol=2e-6)
    close(ref)
    close(alt)


def test_repeated_calls_and_long_runs_equal_one_call():
    """Graph reuse across calls (updated in place) and runs longer than one
    captured chunk give the result of a single call."""
    specs = [{"kind": "packet", "size": (16, 12, 8), "seed": 1}, {"kind": "tube", "size": (12, 16, 10), "beta": 0.3}]
    one, many = make(specs, ffe.FP32), make(specs, ffe.FP32)
    with ffe.Batch(one) as b:
        b.step(300, step0=[0, 0])
        b.synchronize()
    with ffe.Batch(many) as b:
        for c in range(6):
            b.step(50, step0=[50 * c, 50 * c])
        b.synchronize()
    assert_equal_fields(fields(one), fields(many))
    close(one)
    close(many)


def test_more_members_than_one_launch_holds():
    """70 members: two launch groups per stage; each equals its own batch."""
    rng = np.random.Generator(np.random.PCG64(9))
    specs = []
    for i in range(70):
        size = tuple(int(v) for v in rng.integers(8, 20, size=3))
        specs.append({"kind": "packet", "size": size, "seed": i} if i % 2 else
                     {"kind": "tube", "size": size, "beta": 0.1 + 0.005 * i})
    mix = make(specs, ffe.FP32)
    with ffe.Batch(mix) as b:
        # 2 groups, each with one stage launch per variant (plain packets, tubes
        # with B0) and one of the tubes' ghost planes
        assert b.launches() == 3 * (2 * 2 + 2)
        b.step(3)
        b.synchronize()
    got = fields(mix)
    close(mix)
    for m in (0, 1, 63, 64, 69):
        alone = make([specs[m]], ffe.FP32)
        with ffe.Batch(alone) as b:
            b.step(3)
            b.synchronize()
        assert_equal_fields([got[m]], fields(alone))
        close(alone)


def test_autotune_keeps_state_and_picks_a_valid_tiling():
    sols = make(SPECS, ffe.FP32)
    before = fields(sols)
    with ffe.Batch(sols) as b:
        ms = b.autotune(reps=2)
        t = b.tiling()
        after = fields(sols)
        assert ms > 0 and t["tile_y"] in (8, 16) and t["planes"] in (0, 8, 16, 32, 64)
        assert_equal_fields(before, after)
        b.step(2)
        b.synchronize()
    ref = make(SPECS, ffe.FP32)
    with ffe.Batch(ref) as b:
        b.step(2)
        b.synchronize()
    assert_equal_fields(fields(ref), fields(sols), exact=False, tol=2e-6)
    close(sols)
    close(ref)


def test_batch_then_single_steps_continue_the_same_run():
    """The members' set rotation carries over between batched and single calls."""
    a, b_ = make(SPECS[:3], ffe.FP32C), make(SPECS[:3], ffe.FP32C)
    with ffe.Batch(a) as b:
        b.step(2)
        b.synchronize()
    for s in a:
        s.mainloop(2, 2)
    for s in b_:
        s.mainloop(4, 0)
        s.synchronize()
    assert_equal_fields(fields(a), fields(b_), exact=False, tol=2e-6)
    close(a)
    close(b_)


def test_batch_rejections():
    good = workloads.build_solver(SPECS[0], ffe.FP32)
    other = workloads.build_solver(SPECS[1], ffe.FP64)
    staged = workloads.build_solver(SPECS[0], ffe.FP32, path=ffe.PATH_STAGED)
    loop = ffe.Solver(ffe.make_desc((16, 16, 16), setup=ffe.SETUP_LOOP, params=(4.0, 0.5, 0.5)))
    cd = workloads.build_solver(SPECS[0], ffe.FP32CD)
    for members, status in (([good, other], -1), ([good, good], -1), ([staged], -7), ([loop], -7), ([cd], -7)):
        with pytest.raises(ffe.FFEError) as e:
            ffe.Batch(members)
        assert e.value.status == status
    with ffe.Batch([good]) as b:
        with pytest.raises(ffe.FFEError):
            b.set_tiling(12, 0, False)
        with pytest.raises(ffe.FFEError):
            b.step(-1)
    fp64 = workloads.build_solver(SPECS[0], ffe.FP64)
    with ffe.Batch([fp64]) as b:
        with pytest.raises(ffe.FFEError) as e:
            b.set_tiling(16, 0, False)
        assert e.value.status == -7
    close([good, other, staged, loop, cd, fp64])
