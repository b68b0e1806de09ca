"""ffe_clean_epar_noalloc: the cleaning for callers that own all of their device
memory and cannot let the library allocate (a driver whose arrays were
reserved up front, or a run loop where an allocation call is not acceptable).

The caller's arrays here are torch CUDA tensors in the reference's layout; the
test calls the new entry point through the C ABI twice in a row and checks each
result against the existing entry point (ffe_clean_epar on a handle), bit for
bit as the staged parity tests do (both run the same cleaning arithmetic with
no multiply-add contraction).  It also checks the set-up call (after it, a
cleaning call takes no device memory), and that a size beyond the 24 MiB
scratch is refused with a clear message.
"""
import ctypes

import numpy as np
import pytest

import ffe

pytestmark = pytest.mark.gpu

F3 = ("ex", "ey", "ez")
SCRATCH_BYTES = 24 << 20


def _fields(size, dt, seed):
    rng = np.random.default_rng(seed)
    shp = (size[2] + 4, size[1] + 4, size[0] + 4)
    f = {n: (0.7 * rng.standard_normal(shp)).astype(dt) for n in F3}
    f.update({n: rng.standard_normal(shp).astype(dt) for n in ("bx", "by", "bz")})
    return f


def _clean(lib, size, prec, dev, stream):
    return lib.ffe_clean_epar_noalloc(size[0], size[1], size[2], prec,
                                      dev["ex"].data_ptr(), dev["ey"].data_ptr(), dev["ez"].data_ptr(),
                                      dev["bx"].data_ptr(), dev["by"].data_ptr(), dev["bz"].data_ptr(),
                                      stream)


def test_clean_epar_noalloc_setup_then_no_device_memory():
    torch = pytest.importorskip("torch")
    lib = ffe.load_library()
    size = (40, 24, 12)
    f = _fields(size, np.float32, seed=3)
    dev = {n: torch.from_numpy(a.copy()).cuda() for n, a in f.items()}
    torch.cuda.synchronize()
    rc = lib.ffe_clean_epar_noalloc(0, 0, 0, ffe.FP32, None, None, None, None, None, None, None)
    assert rc == 0, ffe._last_error(lib, None)
    free0, _ = torch.cuda.mem_get_info()
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        assert _clean(lib, size, ffe.FP32, dev, stream) == 0, ffe._last_error(lib, None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    # the scratch was placed by the set-up call: the cleanings took none of it
    assert free0 - free1 < SCRATCH_BYTES, (free0, free1)


@pytest.mark.parametrize("prec", [ffe.FP32, ffe.FP64, ffe.FP32C, ffe.FP32CD])
def test_clean_epar_noalloc_matches_handle_path(prec):
    torch = pytest.importorskip("torch")
    lib = ffe.load_library()
    dt = np.float64 if prec == ffe.FP64 else np.float32
    size = (37, 21, 13)
    f = _fields(size, dt, seed=5)

    # existing entry point: a handle, two cleanings in a row
    g = ffe.Solver(ffe.make_desc(size, precision=prec, path=ffe.PATH_STAGED))
    g.set_fields(f)
    g.cleanEpar()
    want1 = {n: g.download(n) for n in F3}
    g.cleanEpar()
    want2 = {n: g.download(n) for n in F3}
    g.close()

    # new entry point on caller-owned device arrays
    dev = {n: torch.from_numpy(a.copy()).cuda() for n, a in f.items()}
    stream = torch.cuda.current_stream().cuda_stream
    for want in (want1, want2):
        rc = _clean(lib, size, prec, dev, stream)
        assert rc == 0, ffe._last_error(lib, None)
        torch.cuda.synchronize()
        for n in F3:
            got = dev[n].cpu().numpy()
            assert np.array_equal(got, want[n]), (n, float(np.max(np.abs(got.astype(float) - want[n]))))
    # B is read only
    for n in ("bx", "by", "bz"):
        assert np.array_equal(dev[n].cpu().numpy(), f[n])


def test_clean_epar_noalloc_tall_block():
    """sz beyond the 65,535 blocks a grid's z dimension allows (a handle
    refuses such a block): the kernels loop over cells, so it is cleaned like
    any other; checked against the oracle's cleanEpar, which the handle path
    matches bit for bit."""
    torch = pytest.importorskip("torch")
    import oracle as O
    lib = ffe.load_library()
    size = (2, 2, 70000)
    f = _fields(size, np.float32, seed=9)
    o = O.Oracle(ffe.make_desc(size, precision=ffe.FP32))
    o.set_fields(f)
    o.cleanEpar()
    want = {n: o.download(n) for n in F3}
    o.close()
    dev = {n: torch.from_numpy(a.copy()).cuda() for n, a in f.items()}
    assert _clean(lib, size, ffe.FP32, dev, torch.cuda.current_stream().cuda_stream) == 0, \
        ffe._last_error(lib, None)
    torch.cuda.synchronize()
    for n in F3:
        assert np.array_equal(dev[n].cpu().numpy(), want[n]), n


def test_clean_epar_noalloc_rejects_oversize():
    lib = ffe.load_library()
    p = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.ffe_clean_epar_noalloc(256, 256, 256, ffe.FP32, p, p, p, p, p, p, None)
    assert rc == -1
    msg = ffe._last_error(lib, None)
    assert "24 MiB" in msg
