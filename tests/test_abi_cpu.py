"""CPU checks of the C-ABI library: it builds for sm_103a, loads without a GPU,
and exports every function include/ffe.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

import ffe
from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "ffe.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(ffe_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    import build as ffe_build
    ffe_build.build()
    return ctypes.CDLL(ffe.LIB_PATH)


def test_header_declares_the_abi():
    names = declared_functions()
    assert "ffe_create" in names and "ffe_step" in names and len(names) >= 20
    assert set(names) == set(ffe.ABI_SYMBOLS), set(names) ^ set(ffe.ABI_SYMBOLS)


def test_library_exports_every_declared_symbol(lib):
    for n in declared_functions():
        assert hasattr(lib, n), n


def test_abi_version_and_descriptor_defaults(lib):
    L = ffe.load_library()
    assert L.ffe_abi_version() == 1
    d = ffe.GridDesc()
    assert L.ffe_desc_default(ctypes.byref(d), 16, 8, 4) == 0
    assert (d.sx, d.sy, d.sz, d.gsx) == (16, 8, 4, 16)
    assert list(d.boundary) == [1, 1, 1] and d.absorb_buff == 20 and abs(d.cc - 0.45) < 1e-15


def test_descriptor_layout_matches_header():
    # int32 x 18, then double cc at offset 72, params, stream pointer
    assert ffe.GridDesc.cc.offset == 72
    assert ffe.GridDesc.params.offset == 80
    assert ffe.GridDesc.stream.offset == 144
    assert ctypes.sizeof(ffe.GridDesc) == 152


def test_create_rejects_bad_descriptors_without_a_gpu(lib):
    L = ffe.load_library()
    h = ctypes.c_void_p()
    d = ffe.make_desc((1, 8, 8))
    assert L.ffe_create(ctypes.byref(h), ctypes.byref(d)) == -1
    buf = ctypes.create_string_buffer(256)
    assert L.ffe_last_error(None, buf, 256) == -1
    assert b"ghost zones" in buf.value


def test_batch_entry_points_validate_arguments_without_a_gpu(lib):
    L = ffe.load_library()
    b = ctypes.c_void_p()
    assert L.ffe_batch_create(ctypes.byref(b), None, 0, None) == -1
    assert L.ffe_batch_step(None, 1, None) == -1
    assert L.ffe_batch_set_tiling(None, 8, 0, 0) == -1
    assert L.ffe_batch_autotune(None, 1, None) == -1
    n = ctypes.c_int32()
    assert L.ffe_batch_launches(None, ctypes.byref(n)) == -1
    assert L.ffe_batch_destroy(None) == 0


def test_footprint_query_needs_no_gpu(lib):
    d = ffe.make_desc((64, 48, 32), precision=ffe.FP32)
    b = ffe.desc_device_bytes(d)
    px = (2 + 64 + 2 + 31) // 32 * 32
    arr = (px * 52 * 36 * 4 + 255) // 256 * 256
    assert b >= 22 * arr and b < 22 * arr + (1 << 20)
    d64 = ffe.make_desc((64, 48, 32), precision=ffe.FP64)
    assert ffe.desc_device_bytes(d64) > 1.5 * b  # rows padded to 128 bytes in both
    psr = ffe.make_desc((64, 64, 64), setup=ffe.SETUP_PSR, params=(6.0, 30.0, 100.0, 1.0), boundary=(2, 2, 2))
    assert ffe.desc_device_bytes(psr) > ffe.desc_device_bytes(ffe.make_desc((64, 64, 64)))
    with pytest.raises(ffe.FFEError):
        ffe.desc_device_bytes(ffe.make_desc((1, 8, 8)))
    # in-plane offsets of the fused kernels are 32-bit: planes of 2^31 elements are refused
    assert ffe.desc_device_bytes(ffe.make_desc((46000, 46000, 2))) > 0
    with pytest.raises(ffe.FFEError):
        ffe.desc_device_bytes(ffe.make_desc((50000, 50000, 2)))


def test_descriptor_rejects_grids_beyond_the_launch_limits(lib):
    """The per-cell kernels put the z planes (ghosts included) on a grid's z
    dimension: a block taller than 65531 cells is refused with a clear message
    instead of failing at its first launch."""
    assert ffe.desc_device_bytes(ffe.make_desc((2, 2, 65531))) > 0
    with pytest.raises(ffe.FFEError) as e:
        ffe.desc_device_bytes(ffe.make_desc((2, 2, 65532)))
    assert "65535" in str(e.value)
