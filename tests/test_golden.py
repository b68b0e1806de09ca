"""Golden fixtures (tests/golden/, made by make_golden.py): the oracle must
reproduce them bit for bit on the CPU, and the GPU library through its C ABI
must reproduce them bit for bit (tanh/exp setups: within 1e-12 / 2e-5)."""
import json
import os

import numpy as np
import pytest

import ffe
from conftest import ROOT, rel_l2

GOLD = os.path.join(ROOT, "tests", "golden")
INDEX = json.load(open(os.path.join(GOLD, "index.json")))
F6 = ("ex", "ey", "ez", "bx", "by", "bz")


def load(name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    c = INDEX[name]
    d = ffe.make_desc(tuple(c["size"]), precision=c["precision"], boundary=tuple(c["boundary"]),
                      setup=c["setup"], params=tuple(c["params"]), absorb_buff=c["absorb_buff"], cc=c["cc"])
    ins = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return d, ins, outs, c["steps"]


@pytest.mark.parametrize("name", sorted(INDEX))
def test_oracle_reproduces_golden(oracle_mod, name):
    d, ins, outs, steps = load(name)
    o = oracle_mod.Oracle(d)
    o.set_fields(ins)
    o.mainloop_prologue()
    o.mainloop(steps, 0)
    for k in F6:
        assert np.array_equal(o.download(k), outs[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("path", [ffe.PATH_STAGED, ffe.PATH_AUTO])
@pytest.mark.parametrize("name", sorted(INDEX))
def test_gpu_reproduces_golden(name, path):
    d, ins, outs, steps = load(name)
    d.path = path
    g = ffe.Solver(d)
    g.set_fields(ins)
    g.mainloop_prologue()
    g.mainloop(steps, 0)
    exact = d.setup == ffe.SETUP_NONE and (path == ffe.PATH_STAGED or g.step_path() == ffe.PATH_STAGED)
    if exact:
        for k in F6:
            a = g.download(k)
            assert np.array_equal(a, outs[k]), (k, float(np.max(np.abs(a.astype(float) - outs[k]))))
        return
    tol = 1e-12 if d.precision == ffe.FP64 else 2e-5
    for comps in (F6[:3], F6[3:]):
        a = np.concatenate([g.download(k).astype(np.float64).ravel() for k in comps])
        b = np.concatenate([outs[k].astype(np.float64).ravel() for k in comps])
        assert rel_l2(a, b) <= tol, (comps, rel_l2(a, b))
