"""Python mirror of tristan-ff's field-solver interface over libffe_gb300.so.

The reference's hot path is a set of Fortran module procedures acting on
module-global arrays (src/algorithms/field_solver.F90, src/tristanmainloop.F90,
src/logistics/exchange_fields.F90, user/user_*.F90).  `Solver` exposes the same
procedures, by the same names, on one meshblock resident on one GPU:

    initRKstep()                      field_solver.F90:15
    rk3Step(c1, c2, c3)               field_solver.F90:35
    computeRho() / rk3Push() / rk3Update(c1, c2, c3)
    cleanEpar()                       field_solver.F90:273
    exchangeFields(exchangeB0=False)  exchange_fields.F90:11
    userInitialize()                  user_*.F90
    userFieldBoundaryConditions(step) user_*.F90
    mainloop(steps, step0)            tristanmainloop.F90:41-84 (step body)

Arrays cross the boundary in the reference's allocation shape: numpy arrays
of shape (sz+4, sy+4, sx+4) (memory order = Fortran (sx+4, sy+4, sz+4)),
float64 for FP64 and float32 otherwise.  Every call goes through the C ABI
(include/ffe.h); there is no CPU fallback: without the library or a GPU the
constructor raises.
"""
import ctypes
import os

import numpy as np

from .inputfile import read_input, desc_from_input  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libffe_gb300.so")

NG = 2
FP64, FP32, FP32C, FP32CD = 0, 1, 2, 3
OPEN, PERIODIC, ABSORB = 0, 1, 2
SETUP_NONE, SETUP_PSR, SETUP_UNIFORM, SETUP_LOOP = 0, 1, 2, 3
PATH_AUTO, PATH_STAGED, PATH_FUSED, PATH_FUSED_EXACT = 0, 1, 2, 3
FLAG_ABSORB_CLAMP = 1
FLAG_CLEAN_TINY = 2
FLAG_ABSORB_TRUE_Y = 4
FLAG_TEST_WITHHOLD_COPY = 8  # failure-detection tests only (include/ffe.h)
FIELDS = ("ex", "ey", "ez", "bx", "by", "bz", "b0x", "b0y", "b0z",
          "dex", "dey", "dez", "dbx", "dby", "dbz",
          "enx", "eny", "enz", "bnx", "bny", "bnz", "rho")
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
STATUS = {0: "OK", -1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "ESTATE",
          -5: "ENONFINITE", -6: "ETIMEOUT", -7: "EUNSUPPORTED"}
PRECISIONS = {"fp64": FP64, "fp32": FP32, "fp32c": FP32C, "fp32cd": FP32CD}
SETUPS = {"none": SETUP_NONE, "psr": SETUP_PSR, "uniform": SETUP_UNIFORM, "loop": SETUP_LOOP}

# (ex, ey, ez, bx, by, bz) staggering offsets (user/user_psr.F90:54-63, 157-221)
STAGGER = {"ex": (0.5, 0, 0), "ey": (0, 0.5, 0), "ez": (0, 0, 0.5),
           "bx": (0, 0.5, 0.5), "by": (0.5, 0, 0.5), "bz": (0.5, 0.5, 0)}

# Exported symbols of the C ABI (kept in step with include/ffe.h).
ABI_SYMBOLS = (
    "ffe_abi_version", "ffe_desc_default", "ffe_create", "ffe_destroy", "ffe_last_error",
    "ffe_field_elems", "ffe_device_bytes", "ffe_upload", "ffe_download",
    "ffe_init_rk_step", "ffe_compute_rho", "ffe_rk3_push", "ffe_rk3_update", "ffe_rk3_stage",
    "ffe_clean_epar", "ffe_exchange_fields", "ffe_user_initialize", "ffe_user_bc",
    "ffe_mainloop_prologue", "ffe_step", "ffe_step_path", "ffe_step_launches",
    "ffe_check_finite", "ffe_synchronize", "ffe_synchronize_timeout", "ffe_init_waves",
    "ffe_clean_epar_noalloc",
    "ffe_desc_device_bytes", "ffe_output_dims", "ffe_output", "ffe_upload_many", "ffe_download_many",
    "ffe_batch_create", "ffe_batch_destroy", "ffe_batch_step", "ffe_batch_set_tiling",
    "ffe_batch_get_tiling", "ffe_batch_autotune", "ffe_batch_launches", "ffe_batch_synchronize",
)


class GridDesc(ctypes.Structure):
    """ffe_grid_desc of include/ffe.h."""
    _fields_ = [
        ("sx", ctypes.c_int32), ("sy", ctypes.c_int32), ("sz", ctypes.c_int32),
        ("x0", ctypes.c_int32), ("y0", ctypes.c_int32), ("z0", ctypes.c_int32),
        ("gsx", ctypes.c_int32), ("gsy", ctypes.c_int32), ("gsz", ctypes.c_int32),
        ("boundary", ctypes.c_int32 * 3),
        ("absorb_buff", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("setup", ctypes.c_int32),
        ("path", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("cc", ctypes.c_double),
        ("params", ctypes.c_double * 8),
        ("stream", ctypes.c_void_p),
    ]


def make_desc(size, precision=FP32, boundary=(PERIODIC,) * 3, cc=0.45, absorb_buff=20,
              setup=SETUP_NONE, params=(), path=PATH_AUTO, offset=(0, 0, 0), gsize=None,
              stream=None, flags=0):
    """Descriptor with the reference's defaults (src/logistics/initialize.F90:139-190)."""
    sx, sy, sz = size
    d = GridDesc()
    d.sx, d.sy, d.sz = sx, sy, sz
    d.x0, d.y0, d.z0 = offset
    d.gsx, d.gsy, d.gsz = gsize or size
    d.boundary[:] = list(boundary)
    d.absorb_buff = absorb_buff
    d.precision = PRECISIONS.get(precision, precision) if isinstance(precision, str) else precision
    d.setup = SETUPS.get(setup, setup) if isinstance(setup, str) else setup
    d.path = path
    d.flags = flags
    d.cc = cc
    p = list(params) + [0.0] * (8 - len(params))
    d.params[:] = p[:8]
    d.stream = stream
    return d


_lib = None


def load_library(path=None):
    """Load libffe_gb300.so and declare the C signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FFEError("libffe_gb300.so not built (%s): run tristan-ff_gb300/build.py" % p, -7)
    lib = ctypes.CDLL(p)
    H = ctypes.c_void_p
    i32, dbl, szt = ctypes.c_int32, ctypes.c_double, ctypes.c_size_t
    sig = {
        "ffe_abi_version": [],
        "ffe_desc_default": [ctypes.POINTER(GridDesc), i32, i32, i32],
        "ffe_create": [ctypes.POINTER(H), ctypes.POINTER(GridDesc)],
        "ffe_destroy": [H],
        "ffe_last_error": [H, ctypes.c_char_p, szt],
        "ffe_field_elems": [H, ctypes.POINTER(szt)],
        "ffe_device_bytes": [H, ctypes.POINTER(szt)],
        "ffe_upload": [H, i32, ctypes.c_void_p, szt],
        "ffe_download": [H, i32, ctypes.c_void_p, szt],
        "ffe_init_rk_step": [H],
        "ffe_compute_rho": [H],
        "ffe_rk3_push": [H],
        "ffe_rk3_update": [H, dbl, dbl, dbl],
        "ffe_rk3_stage": [H, dbl, dbl, dbl],
        "ffe_clean_epar": [H],
        "ffe_exchange_fields": [H, i32],
        "ffe_user_initialize": [H],
        "ffe_user_bc": [H, i32],
        "ffe_mainloop_prologue": [H],
        "ffe_step": [H, i32, i32],
        "ffe_step_path": [H, ctypes.POINTER(i32)],
        "ffe_step_launches": [H, ctypes.POINTER(i32)],
        "ffe_check_finite": [H, ctypes.POINTER(i32)],
        "ffe_synchronize": [H],
        "ffe_synchronize_timeout": [H, i32],
        "ffe_init_waves": [H, ctypes.POINTER(ctypes.c_double), i32, ctypes.POINTER(ctypes.c_double)],
        "ffe_clean_epar_noalloc": [i32, i32, i32, i32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
        "ffe_desc_device_bytes": [ctypes.POINTER(GridDesc), ctypes.POINTER(szt)],
        "ffe_output_dims": [H, i32, ctypes.POINTER(i32)],
        "ffe_output": [H, i32, ctypes.c_void_p, szt],
        "ffe_upload_many": [H, i32, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_void_p), szt],
        "ffe_download_many": [H, i32, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_void_p), szt],
        "ffe_batch_create": [ctypes.POINTER(H), ctypes.POINTER(H), i32, ctypes.c_void_p],
        "ffe_batch_destroy": [H],
        "ffe_batch_step": [H, i32, ctypes.POINTER(i32)],
        "ffe_batch_set_tiling": [H, i32, i32, i32],
        "ffe_batch_get_tiling": [H, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32)],
        "ffe_batch_autotune": [H, i32, ctypes.POINTER(dbl)],
        "ffe_batch_launches": [H, ctypes.POINTER(i32)],
        "ffe_batch_synchronize": [H],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    if path is None:
        _lib = lib
    return lib


class FFEError(RuntimeError):
    def __init__(self, msg, status=None):
        super().__init__(msg)
        self.status = status


def _last_error(lib, h):
    buf = ctypes.create_string_buffer(512)
    lib.ffe_last_error(h, buf, 512)
    return buf.value.decode(errors="replace")


class Solver:
    """One meshblock on one GPU; method names follow the reference procedures."""

    def __init__(self, desc, lib_path=None):
        self.lib = load_library(lib_path)
        self.desc = desc
        self.h = ctypes.c_void_p()
        rc = self.lib.ffe_create(ctypes.byref(self.h), ctypes.byref(desc))
        if rc != 0:
            raise FFEError("ffe_create: %s (%s)" % (_last_error(self.lib, None), STATUS.get(rc, rc)), rc)
        self.dtype = np.float64 if desc.precision == FP64 else np.float32
        self.shape = (desc.sz + 2 * NG, desc.sy + 2 * NG, desc.sx + 2 * NG)

    # -- plumbing ---------------------------------------------------------
    def _ck(self, rc, what):
        if rc != 0:
            raise FFEError("%s: %s (%s)" % (what, _last_error(self.lib, self.h), STATUS.get(rc, rc)), rc)

    def close(self):
        if self.h:
            self.lib.ffe_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.shape != self.shape:
            raise FFEError("upload %s: shape %s, need %s" % (name, a.shape, self.shape), -1)
        self._ck(self.lib.ffe_upload(self.h, FIELD_ID[name], a.ctypes.data, a.size), "upload " + name)

    def download(self, name):
        a = np.empty(self.shape, self.dtype)
        self._ck(self.lib.ffe_download(self.h, FIELD_ID[name], a.ctypes.data, a.size), "download " + name)
        return a

    def fields(self, names=("ex", "ey", "ez", "bx", "by", "bz")):
        out = {n: np.empty(self.shape, self.dtype) for n in names}
        self.download_into(out)
        return out

    def download_into(self, arrays):
        """Download several arrays in one call into the given host arrays (dict name -> array)."""
        names = list(arrays)
        for n in names:
            a = arrays[n]
            if a.shape != self.shape or a.dtype != self.dtype or not a.flags.c_contiguous:
                raise FFEError("download %s: need a contiguous %s array of %s" % (n, self.shape, self.dtype), -1)
        ids = (ctypes.c_int32 * len(names))(*[FIELD_ID[n] for n in names])
        ptrs = (ctypes.c_void_p * len(names))(*[arrays[n].ctypes.data for n in names])
        self._ck(self.lib.ffe_download_many(self.h, len(names), ids, ptrs, int(np.prod(self.shape))), "download")

    def set_fields(self, d):
        """Upload several arrays in one call (B0 arrays one by one)."""
        b0 = {n: a for n, a in d.items() if n in ("b0x", "b0y", "b0z")}
        rest = {n: np.ascontiguousarray(a, dtype=self.dtype) for n, a in d.items() if n not in b0}
        for n, a in rest.items():
            if a.shape != self.shape:
                raise FFEError("upload %s: shape %s, need %s" % (n, a.shape, self.shape), -1)
        if rest:
            names = list(rest)
            ids = (ctypes.c_int32 * len(names))(*[FIELD_ID[n] for n in names])
            ptrs = (ctypes.c_void_p * len(names))(*[rest[n].ctypes.data for n in names])
            self._ck(self.lib.ffe_upload_many(self.h, len(names), ids, ptrs, int(np.prod(self.shape))), "upload")
        for n, a in b0.items():
            self.upload(n, a)

    def device_bytes(self):
        b = ctypes.c_size_t()
        self._ck(self.lib.ffe_device_bytes(self.h, ctypes.byref(b)), "device_bytes")
        return b.value

    def step_path(self):
        p = ctypes.c_int32()
        self._ck(self.lib.ffe_step_path(self.h, ctypes.byref(p)), "step_path")
        return p.value

    def step_launches(self):
        n = ctypes.c_int32()
        self._ck(self.lib.ffe_step_launches(self.h, ctypes.byref(n)), "step_launches")
        return n.value

    # -- the reference's procedures ----------------------------------------
    def initRKstep(self):
        self._ck(self.lib.ffe_init_rk_step(self.h), "initRKstep")

    def computeRho(self):
        self._ck(self.lib.ffe_compute_rho(self.h), "computeRho")

    def rk3Push(self):
        self._ck(self.lib.ffe_rk3_push(self.h), "rk3Push")

    def rk3Update(self, c1, c2, c3):
        self._ck(self.lib.ffe_rk3_update(self.h, c1, c2, c3), "rk3Update")

    def rk3Step(self, c1, c2, c3):
        self._ck(self.lib.ffe_rk3_stage(self.h, c1, c2, c3), "rk3Step")

    def cleanEpar(self):
        self._ck(self.lib.ffe_clean_epar(self.h), "cleanEpar")

    def exchangeFields(self, exchangeB0=False):
        self._ck(self.lib.ffe_exchange_fields(self.h, 1 if exchangeB0 else 0), "exchangeFields")

    def userInitialize(self):
        self._ck(self.lib.ffe_user_initialize(self.h), "userInitialize")

    def userFieldBoundaryConditions(self, step):
        self._ck(self.lib.ffe_user_bc(self.h, step), "userFieldBoundaryConditions")

    def mainloop_prologue(self):
        self._ck(self.lib.ffe_mainloop_prologue(self.h), "mainloop prologue")

    def mainloop(self, steps, step0=0):
        """`steps` repetitions of the main-loop body (asynchronous)."""
        self._ck(self.lib.ffe_step(self.h, steps, step0), "step")

    step = mainloop

    def synchronize(self, timeout_ms=None):
        if timeout_ms is None:
            self._ck(self.lib.ffe_synchronize(self.h), "synchronize")
        else:
            self._ck(self.lib.ffe_synchronize_timeout(self.h, int(timeout_ms)), "synchronize")

    def init_waves(self, bg, modes):
        """Synthetic plane-wave workload; modes: array (n, 11), see include/ffe.h."""
        bgv = (ctypes.c_double * 3)(*[float(x) for x in bg])
        m = np.ascontiguousarray(np.asarray(modes, np.float64).reshape(-1, 11))
        self._ck(self.lib.ffe_init_waves(self.h, bgv, m.shape[0],
                                         m.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "init_waves")

    def output_dims(self, istep=1):
        d = (ctypes.c_int32 * 3)()
        self._ck(self.lib.ffe_output_dims(self.h, int(istep), d), "output_dims")
        return tuple(d)

    def output(self, istep=1):
        """writeOutput's twelve node datasets (OUTPUT_VARS), each shaped
        (nz, ny, nx) with x fastest, at every istep-th node."""
        nx, ny, nz = self.output_dims(istep)
        a = np.empty((12, nz, ny, nx), self.dtype)
        self._ck(self.lib.ffe_output(self.h, int(istep), a.ctypes.data, a.size), "output")
        return {name: a[v] for v, name in enumerate(OUTPUT_VARS)}

    def check_finite(self):
        ok = ctypes.c_int32()
        rc = self.lib.ffe_check_finite(self.h, ctypes.byref(ok))
        if rc not in (0, -5):
            self._ck(rc, "check_finite")
        return bool(ok.value)


def desc_device_bytes(desc, lib_path=None):
    """Device bytes a Solver of this descriptor would allocate (no device call)."""
    lib = load_library(lib_path)
    b = ctypes.c_size_t()
    rc = lib.ffe_desc_device_bytes(ctypes.byref(desc), ctypes.byref(b))
    if rc != 0:
        raise FFEError("ffe_desc_device_bytes: %s (%s)" % (_last_error(lib, None), STATUS.get(rc, rc)), rc)
    return b.value


# dataset names of the reference's field output (src/io/write_output.F90:48-51)
OUTPUT_VARS = ("ex", "ey", "ez", "bx", "by", "bz", "var1", "var2", "var3", "xx", "yy", "zz")


def write_output(path, step, datasets, params=None):
    """Store one output step: the twelve datasets plus `timestep` (and the
    run's parameters as `group:name` entries) in an .npz file, the place of
    the reference's flds.tot.NNNNN HDF5 file (HDF5 is not available here)."""
    d = {name: datasets[name] for name in OUTPUT_VARS}
    d["timestep"] = np.array([step], np.int32)
    for k, v in (params or {}).items():
        d[k] = np.array([v])
    np.savez(path, **d)


class Batch:
    """Many Solvers advanced together (ffe_batch_*): one launch per SSP-RK3
    stage for all members, a CUDA graph per chunk of steps.  The batch does
    not own the solvers; close it before closing them."""

    def __init__(self, solvers, stream=None):
        self.lib = solvers[0].lib
        self.solvers = list(solvers)
        hs = (ctypes.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        self.b = ctypes.c_void_p()
        rc = self.lib.ffe_batch_create(ctypes.byref(self.b), hs, len(self.solvers), stream)
        if rc != 0:
            raise FFEError("ffe_batch_create: %s (%s)" % (_last_error(self.lib, None), STATUS.get(rc, rc)), rc)

    def _ck(self, rc, what):
        if rc != 0:
            raise FFEError("%s: %s (%s)" % (what, _last_error(self.lib, None), STATUS.get(rc, rc)), rc)

    def close(self):
        if self.b:
            self.lib.ffe_batch_destroy(self.b)
            self.b = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, nsteps, step0=None):
        """Advance every member nsteps steps; step0: per-member first step (default 0)."""
        s0 = None
        if step0 is not None:
            s0 = (ctypes.c_int32 * len(self.solvers))(*[int(x) for x in step0])
        self._ck(self.lib.ffe_batch_step(self.b, int(nsteps), s0), "batch step")

    def set_tiling(self, tile_y=8, planes=0, persistent=False):
        self._ck(self.lib.ffe_batch_set_tiling(self.b, tile_y, planes, 1 if persistent else 0), "batch tiling")

    def tiling(self):
        t, k, p = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._ck(self.lib.ffe_batch_get_tiling(self.b, ctypes.byref(t), ctypes.byref(k), ctypes.byref(p)), "tiling")
        return {"tile_y": t.value, "planes": k.value, "persistent": bool(p.value)}

    def autotune(self, reps=3):
        """Time every tiling candidate, keep the fastest; returns its ms per stage."""
        ms = ctypes.c_double()
        self._ck(self.lib.ffe_batch_autotune(self.b, int(reps), ctypes.byref(ms)), "autotune")
        return ms.value

    def launches(self):
        n = ctypes.c_int32()
        self._ck(self.lib.ffe_batch_launches(self.b, ctypes.byref(n)), "batch launches")
        return n.value

    def synchronize(self):
        self._ck(self.lib.ffe_batch_synchronize(self.b), "batch synchronize")


def interior(a):
    """Interior view [2:-2] on every axis of a ghosted array."""
    return a[NG:-NG, NG:-NG, NG:-NG]
