"""ffe_output on the GPU against the restatement of writeOutput's datasets:
bit for bit (the output kernel is built without multiply-add contraction)."""
import numpy as np
import pytest

import ffe
from conftest import ROOT  # noqa: F401
import ffe_output_ref as ref

pytestmark = pytest.mark.gpu


def random_fields(size, dtype, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    shp = (size[2] + 4, size[1] + 4, size[0] + 4)
    return {n: rng.standard_normal(shp).astype(dtype) for n in ("ex", "ey", "ez", "bx", "by", "bz")}


@pytest.mark.parametrize("prec", [ffe.FP32, ffe.FP64])
@pytest.mark.parametrize("istep", [1, 2, 3])
@pytest.mark.parametrize("setup", [ffe.SETUP_NONE, ffe.SETUP_UNIFORM])
def test_output_matches_restatement(prec, istep, setup):
    size, offset, gsize = (19, 14, 11), (5, 3, 7), (40, 30, 25)
    prm = (4.0, 1.0, 50.0, 0.3) if setup == ffe.SETUP_UNIFORM else ()
    d = ffe.make_desc(size, precision=prec, setup=setup, params=prm, offset=offset, gsize=gsize,
                      boundary=(0, 0, 0))
    g = ffe.Solver(d)
    dt = np.float64 if prec == ffe.FP64 else np.float32
    f = random_fields(size, dt, 3 + istep)
    g.set_fields(f)
    got = g.output(istep)
    want = ref.node_output(f, size, istep, offset=offset, gsize=gsize, uniform=setup == ffe.SETUP_UNIFORM)
    assert g.output_dims(istep) == tuple(want["ex"].shape[::-1])
    for n in ffe.OUTPUT_VARS:
        a, b = got[n], want[n]
        bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
        assert not bad.any(), (n, int(bad.sum()), np.argwhere(bad)[:3].tolist())
    g.close()


def test_output_after_fused_steps_and_npz(tmp_path):
    from ffe.workloads import alfven_packet
    size = (32, 16, 16)
    g = ffe.Solver(ffe.make_desc(size))
    bg, modes, _ = alfven_packet(size, seed=2)
    g.init_waves(bg, modes)
    g.mainloop_prologue()
    g.mainloop(5, 0)
    out = g.output(2)
    want = ref.node_output(g.fields(), size, 2)
    for n in ffe.OUTPUT_VARS:
        assert np.array_equal(out[n], want[n]), n
    p = tmp_path / "flds.tot.00005.npz"
    ffe.write_output(str(p), 5, out)
    z = np.load(str(p))
    assert set(ffe.OUTPUT_VARS) <= set(z.files) and int(z["timestep"][0]) == 5
    g.close()
    with pytest.raises(ffe.FFEError):
        ffe.Solver(ffe.make_desc(size)).output(0)
