"""Generate the golden fixtures of tests/golden/ (run from the repo root).

    python tests/golden/make_golden.py

Each case stores its inputs (E, B, B0 ghosted arrays), its descriptor and the
oracle's E, B after `steps` main-loop steps (prologue first).  Cases without a
user boundary condition are first checked bit for bit against the independent
numpy restatement; a mismatch aborts.  The reference itself cannot run in this
image, so these vectors pin the restatement against regressions and give the
GPU tests expected values that need no compiler; they do not pin it to the
reference's own output.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "tristan-ff_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

import ffe  # noqa: E402
import oracle as O  # noqa: E402
from ffe.workloads import alfven_packet, host_waves  # noqa: E402
from ffe_numpy import NumpySolver  # noqa: E402

F6 = ("ex", "ey", "ez", "bx", "by", "bz")


def rand_fields(size, dt, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    shp = (size[2] + 4, size[1] + 4, size[0] + 4)
    f = {n: (0.7 * rng.standard_normal(shp)).astype(dt) for n in ("ex", "ey", "ez")}
    f.update({n: rng.standard_normal(shp).astype(dt) for n in ("bx", "by", "bz")})
    f.update({n: (0.3 * rng.standard_normal(shp)).astype(dt) for n in ("b0x", "b0y", "b0z")})
    return f


def cabi_fields(size):
    """Inputs of the plain-C ABI program (tests/c/abi_roundtrip.c): small
    integers over powers of two, exact in float32, indexed by the element's
    position i in the ghosted array, so C and numpy give identical values."""
    shp = (size[2] + 4, size[1] + 4, size[0] + 4)
    i = np.arange(int(np.prod(shp)), dtype=np.int64)
    def f(mul, mod, off, den, base=0.0):
        return (base + ((i * mul) % mod - off).astype(np.float32) / np.float32(den)).astype(np.float32).reshape(shp)
    return {"ex": f(37, 101, 50, 4096), "ey": f(53, 97, 48, 4096), "ez": f(29, 89, 44, 4096),
            "bx": f(17, 83, 41, 8192), "by": f(41, 79, 39, 8192), "bz": f(13, 73, 36, 8192, 1.0)}


CASES = [
    # name, size, precision, boundary, setup, params, steps, input kind
    ("alfven_fp64_periodic", (16, 4, 4), ffe.FP64, (1, 1, 1), 0, (), 10, "alfven"),
    ("random_fp32_absorb", (11, 9, 8), ffe.FP32, (2, 2, 2), 0, (), 2, "random"),
    ("random_fp64_mixed", (10, 7, 6), ffe.FP64, (1, 1, 0), 0, (), 2, "random"),
    ("random_fp32c_periodic", (9, 8, 7), ffe.FP32C, (1, 1, 1), 0, (), 2, "random"),
    ("random_fp32cd_periodic", (9, 8, 7), ffe.FP32CD, (1, 1, 1), 0, (), 2, "random"),
    ("psr_fp64_open", (20, 20, 20), ffe.FP64, (0, 0, 0), 1, (4.0, 30.0, 120.0, 1.0), 3, "setup"),
    ("uniform_fp32_tube", (12, 12, 10), ffe.FP32, (1, 1, 0), 2, (8.0, 0.4, 5.0, 0.3), 3, "setup"),
    ("loop_fp64", (12, 12, 10), ffe.FP64, (1, 1, 0), 3, (3.0, 1.0, 1.0, 0.5, 5.0, 0.3), 3, "setup"),
    ("cabi_fp32_periodic", (16, 12, 8), ffe.FP32, (1, 1, 1), 0, (), 3, "cabi"),
]


def main():
    O.build()
    index = {}
    for name, size, prec, bnd, setup, params, steps, kind in CASES:
        dt = np.float64 if prec == ffe.FP64 else np.float32
        d = ffe.make_desc(size, precision=prec, boundary=bnd, setup=setup, params=params, absorb_buff=3)
        o = O.Oracle(d)
        if kind == "alfven":
            bg, modes, _ = alfven_packet(size, seed=0, amp=0.1)
            f = host_waves(size, bg, modes, dt)
            o.set_fields(f)
        elif kind == "cabi":
            f = cabi_fields(size)
            o.set_fields(f)
        elif kind == "random":
            f = rand_fields(size, dt, seed=sum(map(ord, name)))
            o.set_fields(f)
        else:
            o.userInitialize()
            f = o.fields(F6 + ("b0x", "b0y", "b0z"))
        o.mainloop_prologue()
        o.mainloop(steps, 0)
        out = o.fields()
        if setup == 0 and prec in (ffe.FP32, ffe.FP64):
            n = NumpySolver(*size, dt, boundary=bnd, absorb_buff=3)
            for k, v in f.items():
                n.f[k][...] = v
            n.exchange(True)
            n.step(steps)
            for k in F6:
                if not np.array_equal(n.f[k], out[k]):
                    raise SystemExit("numpy restatement disagrees with the oracle on %s/%s" % (name, k))
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            **{"in_" + k: v for k, v in f.items()}, **{"out_" + k: v for k, v in out.items()})
        index[name] = {"size": size, "precision": prec, "boundary": bnd, "setup": setup,
                       "params": list(params), "steps": steps, "absorb_buff": 3, "cc": 0.45}
        print(name, "ok")
    with open(os.path.join(HERE, "index.json"), "w") as fh:
        json.dump(index, fh, indent=1)


if __name__ == "__main__":
    main()
