"""The serving loop's scheduling on the CPU, with stand-ins for the device
objects: first come first served admission under the HBM budget, epochs that
end when a run finishes, every request served exactly once."""
import numpy as np

import ffe
from ffe import serve, workloads


class FakeSolver:
    def check_finite(self):
        return True

    def __init__(self, spec):
        self.spec = spec
        self.steps_run = 0
        self.closed = False

    def fields(self):
        return {"steps": self.steps_run}

    def close(self):
        self.closed = True


class FakeBatch:
    built = []

    def __init__(self, solvers):
        self.solvers = solvers
        FakeBatch.built.append(len(solvers))

    def set_tiling(self, *a):
        pass

    def step(self, n, step0=None):
        assert step0 is not None and len(step0) == len(self.solvers)
        for s, s0 in zip(self.solvers, step0):
            assert s.steps_run == s0, "each run continues from its own step"
            s.steps_run += n

    def launches(self):
        return 3

    def synchronize(self):
        pass

    def close(self):
        pass


def requests(n=12, rate=500.0):
    rng = np.random.Generator(np.random.PCG64(2))
    t, out = 0.0, []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        side = int(rng.integers(16, 40))
        out.append({"kind": "psr", "size": (side,) * 3, "incl": 30.0, "steps": int(rng.integers(5, 70)),
                    "arrival": t, "id": i})
    return out


def test_admission_budget_and_completion():
    reqs = requests(rate=1e6)  # all waiting at once: admission is limited by the budget
    sizes = [serve._desc_bytes(q, ffe.FP32C) for q in reqs]
    budget = 3.5 * max(sizes)
    srv = serve.Server(precision=ffe.FP32C, hbm_budget=budget, epoch_steps=16, keep_results=True,
                       build=lambda spec, prec: FakeSolver(spec), batch_cls=FakeBatch)
    recs = srv.serve(reqs)
    assert len(recs) == len(reqs)
    for r in recs:
        assert r.result == {"steps": r.steps}, "every run gets exactly its steps"
        assert r.admitted >= r.arrival - 1e-9 and r.finished >= r.admitted
    assert all(used <= budget for _, _, used, _ in srv.log)
    assert all(0 < n <= 16 for _, n, _, _ in srv.log)
    assert srv.peak_runs >= 2, "runs overlap on the device"
    # first come, first served: admission order follows arrival order
    order = sorted(recs, key=lambda r: r.admitted)
    assert [r.id for r in order] == sorted(r.id for r in recs)
    rep = serve.report(recs)
    assert rep["requests"] == len(reqs) and rep["time_to_result_s"]["p99"] >= rep["time_to_result_s"]["p50"]


def test_shortest_job_first_admits_small_runs_first():
    reqs = requests(rate=1e6)
    srv = serve.Server(hbm_budget=1e15, epoch_steps=16, max_active_cells=1, policy="sjf",
                       build=lambda spec, prec: FakeSolver(spec), batch_cls=FakeBatch)
    recs = srv.serve(reqs)
    order = [r for r in sorted(recs, key=lambda r: r.admitted)]
    work = [r.cells * r.steps for r in order]
    assert work[1:] == sorted(work[1:]), "after the first admission, least work goes first"
    assert all(r.result is None and r.finished is not None for r in recs)


def test_oversized_request_is_refused():
    q = requests(1)
    srv = serve.Server(hbm_budget=1000.0, build=lambda s, p: FakeSolver(s), batch_cls=FakeBatch)
    (r,) = srv.serve(q)
    assert r.status == "rejected" and r.result is None and "budget" in r.error
    assert srv.epochs == 0


def test_served_workload_is_seeded():
    a = workloads.served_requests(8)
    b = workloads.served_requests(8)
    assert a == b
    assert all(96 <= q["size"][0] <= 256 and 200 <= q["steps"] <= 2000 and 0 <= q["incl"] <= 90 for q in a)
    assert all(x["arrival"] < y["arrival"] for x, y in zip(a, a[1:]))


def test_cell_cap_limits_concurrency():
    reqs = requests(rate=1e6)
    cells = [q["size"][0] ** 3 for q in reqs]
    cap = 2 * max(cells)
    srv = serve.Server(hbm_budget=1e15, epoch_steps=16, max_active_cells=cap,
                       build=lambda spec, prec: FakeSolver(spec), batch_cls=FakeBatch)
    recs = srv.serve(reqs)
    assert all(c <= cap for _, _, _, c in srv.log)
    assert all(r.finished is not None for r in recs)
    # a run larger than the cap still runs, alone
    srv = serve.Server(hbm_budget=1e15, max_active_cells=1, build=lambda s, p: FakeSolver(s), batch_cls=FakeBatch)
    recs = srv.serve(reqs[:3])
    assert all(n == 1 for n, _, _, _ in srv.log) and all(r.finished is not None for r in recs)


class FakeFiniteSolver(FakeSolver):
    """A stand-in whose fields turn non-finite (a NaN injected on the host)."""

    def __init__(self, spec, bad):
        super().__init__(spec)
        self.bad = bad

    def check_finite(self):
        return not self.bad


def test_failures_stay_with_their_run():
    """An oversized request is rejected alone, a malformed one too, and a run
    whose fields are not finite at the end is marked failed; the reference
    stops the whole job instead (src/tools/error_handling.F90:8-13)."""
    reqs = requests(n=10, rate=1e6)
    sizes = [serve._desc_bytes(q, ffe.FP32C) for q in reqs]
    budget = 2.5 * max(sizes)
    big = {"kind": "psr", "size": (4096,) * 3, "incl": 10.0, "steps": 5, "arrival": 0.0, "id": "big"}
    bad_kind = {"kind": "nonsense", "size": (16,) * 3, "steps": 5, "arrival": 0.0, "id": "bad-kind"}
    poisoned = reqs[3]["id"]
    srv = serve.Server(precision=ffe.FP32C, hbm_budget=budget, epoch_steps=16, keep_results=True,
                       build=lambda spec, prec: FakeFiniteSolver(spec, spec["id"] == poisoned),
                       batch_cls=FakeBatch)
    recs = srv.serve(reqs + [big, bad_kind])
    by_id = {r.id: r for r in recs}
    assert by_id["big"].status == "rejected" and "budget" in by_id["big"].error
    assert by_id["bad-kind"].status == "rejected"
    assert by_id[poisoned].status == "failed" and by_id[poisoned].result is None
    for q in reqs:
        if q["id"] != poisoned:
            r = by_id[q["id"]]
            assert r.status == "ok" and r.result == {"steps": r.steps}
    rep = serve.report(recs)
    assert (rep["completed"], rep["rejected"], rep["failed"]) == (len(reqs) - 1, 2, 1)
