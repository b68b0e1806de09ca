"""The serving loop on the GPU: runs admitted while others compute advance in
one batch, and each result is bit-identical to the same run alone."""
import numpy as np
import pytest

import ffe
from ffe import serve, workloads
from conftest import rel_l2

pytestmark = pytest.mark.gpu

F6 = ("ex", "ey", "ez", "bx", "by", "bz")


def small_requests(n=8, rate=400.0, seed=11):
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        side = int(rng.integers(24, 44))
        out.append({"kind": "psr", "size": (side,) * 3, "incl": float(rng.uniform(0, 90)),
                    "steps": int(rng.integers(8, 40)), "arrival": t, "id": i})
    return out


def eb_err(a, b):
    out = []
    for grp in (("ex", "ey", "ez"), ("bx", "by", "bz")):
        x = np.concatenate([ffe.interior(a[k]).ravel().astype(np.float64) for k in grp])
        y = np.concatenate([ffe.interior(b[k]).ravel().astype(np.float64) for k in grp])
        out.append(rel_l2(x, y))
    return max(out)


@pytest.fixture(scope="module")
def served():
    reqs = small_requests()
    budget = 3.5 * max(serve._desc_bytes(q, ffe.FP32C) for q in reqs)
    srv = serve.Server(precision=ffe.FP32C, hbm_budget=budget, epoch_steps=8, keep_results=True)
    recs = srv.serve(reqs)
    return reqs, srv, recs


def test_runs_overlap_and_all_finish(served):
    reqs, srv, recs = served
    assert len(recs) == len(reqs) and all(r.result is not None for r in recs)
    assert srv.peak_runs >= 2 and srv.batches_built >= 2
    assert all(used <= srv.budget for _, _, used, _ in srv.log)
    rep = serve.report(recs)
    assert rep["cell_updates_per_s"] > 0 and rep["time_to_result_s"]["p99"] >= rep["time_to_result_s"]["p50"]


def test_each_result_equals_the_run_alone(served):
    reqs, srv, recs = served
    for r in recs:
        alone = workloads.build_solver(r.spec, ffe.FP32C)
        with ffe.Batch([alone]) as b:
            b.step(r.steps, step0=[0])
            b.synchronize()
        f = alone.fields()
        alone.close()
        for k in F6:
            bad = f[k] != r.result[k]
            assert not bad.any(), (r.id, k, int(bad.sum()))


def test_served_matches_plain_path_and_fp64(served):
    reqs, srv, recs = served
    plain = serve.serve_plain(reqs[:3], precision=ffe.FP32C, keep_results=True)
    for p in plain:
        r = next(x for x in recs if x.id == p.id)
        assert eb_err(p.result, r.result) <= 2e-6, (p.id, eb_err(p.result, r.result))
    # accuracy of the served FP32 run against the same run in FP64
    r = recs[0]
    g = workloads.build_solver(r.spec, ffe.FP64)
    g.mainloop(r.steps, 0)
    g.synchronize()
    assert eb_err(g.fields(), r.result) <= 1e-5
    g.close()


def test_served_runs_match_the_oracle(served, oracle_mod):
    """The two smallest served runs against the CPU oracle (FP32C, the same
    arithmetic with exact quotients and no contraction) after their full step
    counts: the served fast path stays within 2e-5 relative L2."""
    reqs, srv, recs = served
    for r in sorted(recs, key=lambda x: x.cells * x.steps)[:2]:
        o = workloads.init_run(oracle_mod.Oracle(workloads.run_desc(r.spec, ffe.FP32C)), r.spec)
        o.mainloop(r.steps, 0)
        err = eb_err(o.fields(), r.result)
        o.close()
        assert err <= 2e-5, (r.id, r.steps, err)
