"""Serving loop: continuous batching of force-free runs on one GPU.

No counterpart in the reference (one run per job there).  A request is a run
spec (see workloads.build_solver) with a step count and an arrival time.
Requests are admitted first come, first served as long as the device bytes
of the admitted runs (ffe_desc_device_bytes) stay within the HBM budget and
their cells within `max_active_cells` (enough cells to fill the GPU: more
runs at once add no throughput, only delay every run's result); an admitted
run keeps its fields on the device until it finishes.  All admitted
runs advance together: an epoch is one batched call (ffe_batch_step: one
launch per SSP-RK3 stage for every run, captured into a CUDA graph) of
min(epoch_steps, fewest steps left) steps.  At each epoch boundary finished
runs leave (their fields are copied to the host while the next epoch already
runs on the device), newly arrived runs join, and the batch is rebuilt when
its membership changed.

`serve_plain` is the one-grid-at-a-time baseline on the same requests: each
run alone on the single-grid fused path, in arrival order.

Time-to-result of a request = from its arrival to the moment its result is
on the host.  Times are wall-clock seconds from the start of serving.

Failures stay with their run.  The reference stops the whole job on an error
(src/tools/error_handling.F90:8-13); here a request that cannot fit the HBM
budget is rejected alone (status "rejected"), and a run whose fields are no
longer finite when it finishes (ffe_check_finite) is marked "failed" with
no result; every other run goes on and finishes as it would have alone.
"""
import time

import numpy as np

import ffe
from ffe import workloads


class Record:
    __slots__ = ("id", "spec", "steps", "done", "solver", "bytes", "arrival", "admitted", "finished", "cells",
                 "result", "status", "error")

    def __init__(self, spec):
        self.id = spec.get("id")
        self.spec = spec
        self.steps = int(spec["steps"])
        self.done = 0
        self.solver = None
        self.bytes = 0
        self.arrival = float(spec.get("arrival", 0.0))
        self.admitted = None
        self.finished = None
        s = spec["size"]
        self.cells = int(s[0]) * int(s[1]) * int(s[2])
        self.result = None
        self.status = "queued"   # then "ok", "rejected" or "failed"
        self.error = None

    def summary(self):
        return {"id": self.id, "size": list(self.spec["size"]), "steps": self.steps, "arrival": self.arrival,
                "admitted": self.admitted, "finished": self.finished, "status": self.status, "error": self.error,
                "time_to_result": None if self.finished is None else self.finished - self.arrival}


def _desc_bytes(spec, precision):
    """Device bytes of a run, from the descriptor build_solver would use."""
    return ffe.desc_device_bytes(workloads.run_desc(spec, precision))


def _finish(r, now, keep):
    """Check that the run's fields are finite, copy its E, B to the host (kept
    when `keep` is true or holds the run's id), record the time, free the
    run's device memory.  A run with NaN or Inf in E or B is marked failed and
    gives no result."""
    if r.solver.check_finite():
        fields = r.solver.fields()
        r.result = fields if (keep is True or (keep and r.id in keep)) else None
        r.status = "ok"
    else:
        r.result = None
        r.status = "failed"
        r.error = "non-finite E or B after %d steps" % r.done
    r.finished = now()
    r.solver.close()
    r.solver = None


def _reject(r, budget, now):
    r.status = "rejected"
    r.error = "needs %d device bytes, more than the budget of %d" % (r.bytes, int(budget))
    r.finished = now()


class Server:
    """Continuous batching under an HBM budget (bytes).  keep_results: True,
    or a set of request ids whose final fields are kept on the host.
    policy: "fifo" admits in arrival order; "sjf" admits the waiting request
    with the least work (cells x steps) first, which shortens the median time
    to result at the cost of the largest runs."""

    def __init__(self, precision=ffe.FP32C, hbm_budget=180e9, epoch_steps=32, tiling=(8, 0, False),
                 keep_results=False, build=None, batch_cls=None, max_active_cells=64 << 20, policy="fifo"):
        if policy not in ("fifo", "sjf"):
            raise ValueError("policy must be 'fifo' or 'sjf'")
        self.policy = policy
        self.build = build or workloads.build_solver
        self.batch_cls = batch_cls or ffe.Batch
        self.precision = precision
        self.budget = float(hbm_budget)
        self.max_cells = int(max_active_cells)
        self.epoch_steps = int(epoch_steps)
        self.tiling = tuple(tiling)
        self.keep = keep_results
        self.epochs = 0
        self.batches_built = 0
        self.peak_bytes = 0
        self.peak_runs = 0
        self.launches = 0
        self.log = []  # per epoch: (runs, steps, device bytes in use, cells in the batch)
        # host seconds: waiting for epochs to finish, admitting runs (set-up on
        # the device), rebuilding batches, and copying finished runs out
        self.t_wait = self.t_admit = self.t_build = self.t_finish = 0.0

    def serve(self, requests):
        recs = sorted((Record(q) for q in requests), key=lambda r: r.arrival)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        for r in recs:
            try:
                r.bytes = _desc_bytes(r.spec, self.precision)
            except (ffe.FFEError, ValueError, KeyError) as e:  # a malformed request fails alone
                r.status, r.error, r.finished = "rejected", str(e), now()
        pending = [r for r in recs if r.status == "queued"]
        queue, active = [], []
        used = 0
        cells = 0
        batch, members = None, ()
        leaving = []  # finished in the last epoch; copied out while the next one runs
        while pending or queue or active or leaving:
            t = now()
            while pending and pending[0].arrival <= t:
                r = pending.pop(0)
                if r.bytes > self.budget:  # can never fit: rejected alone
                    _reject(r, self.budget, now)
                else:
                    queue.append(r)
            if self.policy == "sjf":  # least work (cells x steps) first among the waiting
                queue.sort(key=lambda r: (r.cells * r.steps, r.arrival))
            while queue and used + queue[0].bytes <= self.budget and (
                    not active or cells + queue[0].cells <= self.max_cells):
                r = queue.pop(0)
                ta = time.perf_counter()
                r.solver = self.build(r.spec, self.precision)
                self.t_admit += time.perf_counter() - ta
                r.admitted = now()
                used += r.bytes
                cells += r.cells
                active.append(r)
            self.peak_bytes = max(self.peak_bytes, used)
            self.peak_runs = max(self.peak_runs, len(active))
            if active:
                ids = tuple(id(r) for r in active)
                if ids != members:
                    tb = time.perf_counter()
                    if batch is not None:
                        batch.close()
                    batch = self.batch_cls([r.solver for r in active])
                    batch.set_tiling(*self.tiling)
                    members = ids
                    self.batches_built += 1
                    self.t_build += time.perf_counter() - tb
                n = min(self.epoch_steps, min(r.steps - r.done for r in active))
                batch.step(n, step0=[r.done for r in active])
                self.log.append((len(active), n, used, cells))
                self.launches += batch.launches() * n
                self.epochs += 1
            # results of the previous epoch leave while this one computes
            tf = time.perf_counter()
            for r in leaving:
                _finish(r, now, self.keep)
                used -= r.bytes
            self.t_finish += time.perf_counter() - tf
            leaving = []
            if active:
                tw = time.perf_counter()
                batch.synchronize()
                self.t_wait += time.perf_counter() - tw
                for r in active:
                    r.done += n
                leaving = [r for r in active if r.done >= r.steps]
                active = [r for r in active if r.done < r.steps]
                cells -= sum(r.cells for r in leaving)
            elif pending and not queue:
                time.sleep(max(0.0, pending[0].arrival - now()))
        if batch is not None:
            batch.close()
        return recs


def serve_plain(requests, precision=ffe.FP32C, keep_results=False, policy="fifo"):
    """The one-grid-at-a-time path: each run alone (single-grid fused path,
    ffe_step), next in arrival order ("fifo") or, among the requests that
    have arrived, least work first ("sjf")."""
    recs = sorted((Record(q) for q in requests), key=lambda r: r.arrival)
    t0 = time.perf_counter()
    now = lambda: time.perf_counter() - t0
    pending = list(recs)
    while pending:
        wait = pending[0].arrival - now()
        if wait > 0:
            time.sleep(wait)
        t = now()
        ready = [r for r in pending if r.arrival <= t]
        r = min(ready, key=lambda x: (x.cells * x.steps, x.arrival)) if policy == "sjf" else ready[0]
        pending.remove(r)
        r.solver = workloads.build_solver(r.spec, precision)
        r.admitted = now()
        r.solver.mainloop(r.steps, 0)
        r.solver.synchronize()
        r.done = r.steps
        _finish(r, now, keep_results)
    return recs


def report(recs):
    """Aggregate throughput (cell-updates of the completed runs over the span
    from the first arrival to the last result), time-to-result percentiles of
    the completed runs, and how many requests were rejected or failed."""
    ok = [r for r in recs if r.status == "ok"]
    out = {"requests": len(recs), "completed": len(ok),
           "rejected": sum(r.status == "rejected" for r in recs), "failed": sum(r.status == "failed" for r in recs)}
    if not ok:
        return out
    ttr = np.array([r.finished - r.arrival for r in ok])
    first = min(r.arrival for r in ok)
    last = max(r.finished for r in ok)
    work = float(sum(r.cells * r.steps for r in ok))
    out.update({"cell_updates": work, "span_s": last - first, "cell_updates_per_s": work / (last - first),
                "time_to_result_s": {"p50": float(np.percentile(ttr, 50)), "p99": float(np.percentile(ttr, 99)),
                                     "max": float(ttr.max())}})
    return out
