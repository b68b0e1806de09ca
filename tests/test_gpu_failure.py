"""Failure detection on the GPU, without faulting, trapping or hanging it.

* A bounded device wait that runs out: with FFE_FLAG_TEST_WITHHOLD_COPY the
  thread that issues a stage block's TMA plane copies leaves one copy out, so
  the block's wait for that plane gives up after a short probe limit, sets the
  error word and returns.  ffe_synchronize (or ffe_batch_synchronize) must
  report FFE_ETIMEOUT, report it once, and the CUDA context must stay usable:
  a new handle steps and matches the oracle.
* The host watchdog on the stream: ffe_synchronize_timeout gives up on work
  that is still running and a later plain synchronize succeeds.
* The serving loop: a run whose fields become non-finite (a NaN written into
  one member from the host) is marked failed at its end while the others
  finish with the results they have alone.
The reference has none of this: its fatal paths print and stop
(src/tools/error_handling.F90:8-13).
"""
import time

import numpy as np
import pytest

import ffe
from conftest import rel_l2
from ffe import serve, workloads
from ffe.workloads import random_modes

pytestmark = pytest.mark.gpu

F6 = ("ex", "ey", "ez", "bx", "by", "bz")
ETIMEOUT = -6


def _solver(size, prec, flags=0, path=ffe.PATH_FUSED, seed=7):
    bg, modes, _ = random_modes(size, seed=seed, n=6, kmax=3, amax=0.05)
    g = ffe.Solver(ffe.make_desc(size, precision=prec, path=path, flags=flags))
    g.init_waves(bg, modes)
    g.mainloop_prologue()
    return g


@pytest.mark.parametrize("prec", [ffe.FP32C, ffe.FP64])
def test_withheld_copy_times_out_and_the_context_survives(prec, oracle_mod):
    size = (40, 36, 30)
    g = _solver(size, prec, flags=ffe.FLAG_TEST_WITHHOLD_COPY)
    t0 = time.perf_counter()
    g.mainloop(1, 0)
    with pytest.raises(ffe.FFEError) as e:
        g.synchronize()
    assert e.value.status == ETIMEOUT, e.value
    assert time.perf_counter() - t0 < 60.0
    g.synchronize()          # reported once: the error word is cleared
    g.download("ex")         # the context is still usable
    g.close()
    # a handle without the flag steps normally and matches the oracle
    h = _solver(size, prec)
    o = oracle_mod.Oracle(ffe.make_desc(size, precision=prec))
    o.set_fields(h.fields())
    o.mainloop_prologue()
    o.mainloop(2, 0)
    h.mainloop(2, 0)
    h.synchronize()
    tol = 1e-12 if prec == ffe.FP64 else 1e-5
    for grp in (F6[:3], F6[3:]):
        a = np.concatenate([h.download(k).ravel() for k in grp])
        b = np.concatenate([o.download(k).ravel() for k in grp])
        assert rel_l2(a, b) <= tol
    h.close()
    o.close()


def test_withheld_copy_in_a_batch_times_out():
    sols = [_solver((40, 20, 16), ffe.FP32C, flags=ffe.FLAG_TEST_WITHHOLD_COPY),
            _solver((24, 36, 12), ffe.FP32C, seed=3)]
    b = ffe.Batch(sols)
    b.step(1)
    with pytest.raises(ffe.FFEError) as e:
        b.synchronize()
    assert e.value.status == ETIMEOUT
    b.synchronize()
    b.close()
    for s in sols:
        s.close()


def test_synchronize_timeout_gives_up_on_running_work():
    g = _solver((256, 256, 256), ffe.FP32C)
    g.synchronize()
    g.mainloop(60, 0)        # ~0.5 s of work
    with pytest.raises(ffe.FFEError) as e:
        g.synchronize(timeout_ms=1)
    assert e.value.status == ETIMEOUT
    g.synchronize()          # the work itself completes
    assert g.check_finite()
    g.close()


def test_a_poisoned_served_run_fails_alone():
    rng = np.random.Generator(np.random.PCG64(5))
    reqs = [{"kind": "psr", "size": (int(s),) * 3, "incl": 20.0 + 10 * i, "steps": int(st), "arrival": 0.001 * i,
             "id": i} for i, (s, st) in enumerate(zip(rng.integers(24, 40, 5), rng.integers(8, 24, 5)))]
    poisoned = 2

    def build(spec, prec):
        s = workloads.build_solver(spec, prec)
        if spec["id"] == poisoned:   # a NaN injected from the host into one member
            ex = s.download("ex")
            ex[ex.shape[0] // 2, ex.shape[1] // 2, ex.shape[2] // 2] = np.nan
            s.upload("ex", ex)
        return s

    budget = 4.0 * max(serve._desc_bytes(q, ffe.FP32C) for q in reqs)
    srv = serve.Server(precision=ffe.FP32C, hbm_budget=budget, epoch_steps=8, keep_results=True, build=build)
    recs = {r.id: r for r in srv.serve(reqs)}
    assert recs[poisoned].status == "failed" and recs[poisoned].result is None
    assert srv.peak_runs >= 2
    for q in reqs:
        if q["id"] == poisoned:
            continue
        r = recs[q["id"]]
        assert r.status == "ok"
        alone = workloads.build_solver(q, ffe.FP32C)
        with ffe.Batch([alone]) as b:
            b.step(q["steps"], step0=[0])
            b.synchronize()
        f = alone.fields()
        alone.close()
        for k in F6:
            assert np.array_equal(f[k], r.result[k]), (q["id"], k)
