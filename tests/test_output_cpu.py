"""The output path's restatement (oracle/ffe_output_ref.py) on the CPU: node
ranges of write_output.F90 and exactness on fields that are linear in space."""
import numpy as np
import pytest

from conftest import ROOT  # noqa: F401  (puts oracle/ on the path)
import ffe_output_ref as ref


def test_node_axis_follows_the_reference_ceilings():
    import math
    for x0 in (0, 1, 5, 16, 33):
        for s in (4, 7, 16, 31):
            for istep in (1, 2, 3, 4, 8):
                a = math.ceil(x0 / istep) * istep - x0
                b = (math.ceil((x0 + s) / istep) - 1) * istep - x0
                n = (b - a) // istep + 1 if b >= a else 0
                assert ref.node_axis(x0, s, istep) == (a, n), (x0, s, istep)
    assert ref.node_axis(0, 16, 1) == (0, 16)
    assert ref.node_axis(0, 16, 4) == (0, 4)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_linear_fields_interpolate_exactly(dtype):
    """Each component a.x + b at its staggered point gives a.x_node + b at the
    nodes (dyadic coefficients, so every step is exact)."""
    size = (12, 10, 8)
    sx, sy, sz = size
    k, j, i = np.meshgrid(np.arange(-2, sz + 2), np.arange(-2, sy + 2), np.arange(-2, sx + 2), indexing="ij")
    offs = {"ex": (0.5, 0, 0), "ey": (0, 0.5, 0), "ez": (0, 0, 0.5),
            "bx": (0, 0.5, 0.5), "by": (0.5, 0, 0.5), "bz": (0.5, 0.5, 0)}
    coef = {"ex": (0.25, -0.5, 0.125, 1.0), "ey": (-0.125, 0.25, 0.5, -2.0), "ez": (0.5, 0.5, -0.25, 0.0),
            "bx": (1.0, -0.25, 0.25, 3.0), "by": (0.125, 0.125, 0.5, -1.0), "bz": (-0.5, 0.25, 1.0, 0.5)}
    f = {}
    for n, (ox, oy, oz) in offs.items():
        a, b, c, d = coef[n]
        f[n] = (a * (i + ox) + b * (j + oy) + c * (k + oz) + d).astype(dtype)
    for istep in (1, 2, 3):
        out = ref.node_output(f, size, istep)
        i0, nx = ref.node_axis(0, sx, istep)
        j0, ny = ref.node_axis(0, sy, istep)
        k0, nz = ref.node_axis(0, sz, istep)
        kk, jj, ii = np.meshgrid(k0 + istep * np.arange(nz), j0 + istep * np.arange(ny),
                                 i0 + istep * np.arange(nx), indexing="ij")
        for n in offs:
            a, b, c, d = coef[n]
            assert np.array_equal(out[n], (a * ii + b * jj + c * kk + d).astype(dtype)), (n, istep)
        assert np.array_equal(out["xx"], ii.astype(dtype)) and np.array_equal(out["zz"], kk.astype(dtype))
        # rho of the linear E: a_x + b_y + c_z (divergence)
        assert np.allclose(out["var1"], 0.25 + 0.25 - 0.25)
        assert not out["var2"].any() and not out["var3"].any()
