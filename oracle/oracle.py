"""TEST INFRASTRUCTURE ONLY — ctypes wrapper of the CPU oracle (ffe_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the reference the results are compared with; the product path never
imports it.  PARITY UNPINNED:
see the header of ffe_oracle.cpp.

`Oracle` has the same method names as the product's `ffe.Solver`, so a test
runs one sequence of reference procedures on both and compares the arrays.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libffe_oracle.so")
NG = 2
FIELDS = ("ex", "ey", "ez", "bx", "by", "bz", "b0x", "b0y", "b0z",
          "dex", "dey", "dez", "dbx", "dby", "dbz",
          "enx", "eny", "enz", "bnx", "bny", "bnz", "rho")
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}


def build(force=False):
    """Compile the oracle with its Makefile (portable flags, no -march=native)."""
    src = os.path.join(HERE, "ffe_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "libffe_oracle.so"], check=True)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        V = ctypes.c_void_p
        lib.ora_create.restype = V
        lib.ora_create.argtypes = [V]
        lib.ora_error.restype = ctypes.c_char_p
        lib.ora_elem_size.restype = ctypes.c_size_t
        lib.ora_field_elems.restype = ctypes.c_size_t
        for n in ("ora_destroy", "ora_init_rk_step", "ora_compute_rho", "ora_push", "ora_clean",
                  "ora_user_init", "ora_prologue", "ora_elem_size", "ora_field_elems"):
            getattr(lib, n).argtypes = [V]
        lib.ora_set_threads.argtypes = [V, ctypes.c_int, ctypes.c_int]
        lib.ora_set_field.argtypes = [V, ctypes.c_int, V]
        lib.ora_get_field.argtypes = [V, ctypes.c_int, V]
        lib.ora_update.argtypes = [V, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.ora_rk3_stage.argtypes = [V, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.ora_exchange.argtypes = [V, ctypes.c_int]
        lib.ora_user_bc.argtypes = [V, ctypes.c_int]
        lib.ora_step.argtypes = [V, ctypes.c_int, ctypes.c_int]
        lib.ora_init_waves.argtypes = [V, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_double)]
        _lib = lib
    return _lib


class Oracle:
    """CPU restatement of one meshblock, driven like ffe.Solver."""

    def __init__(self, desc, threads=1, loop_order=1):
        self.lib = load()
        self.desc = desc
        self.h = self.lib.ora_create(ctypes.addressof(desc))
        if not self.h:
            raise ValueError("ora_create: " + self.lib.ora_error().decode())
        self.lib.ora_set_threads(self.h, threads, loop_order)
        self.dtype = np.float64 if desc.precision == 0 else np.float32
        self.shape = (desc.sz + 2 * NG, desc.sy + 2 * NG, desc.sx + 2 * NG)

    def close(self):
        if self.h:
            self.lib.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n, loop_order=1):
        self.lib.ora_set_threads(self.h, n, loop_order)

    def upload(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        assert a.shape == self.shape, (a.shape, self.shape)
        self.lib.ora_set_field(self.h, FIELD_ID[name], a.ctypes.data)

    def download(self, name):
        a = np.empty(self.shape, self.dtype)
        self.lib.ora_get_field(self.h, FIELD_ID[name], a.ctypes.data)
        return a

    def fields(self, names=("ex", "ey", "ez", "bx", "by", "bz")):
        return {n: self.download(n) for n in names}

    def set_fields(self, d):
        for n, a in d.items():
            self.upload(n, a)

    def initRKstep(self):
        self.lib.ora_init_rk_step(self.h)

    def computeRho(self):
        self.lib.ora_compute_rho(self.h)

    def rk3Push(self):
        self.lib.ora_push(self.h)

    def rk3Update(self, c1, c2, c3):
        self.lib.ora_update(self.h, c1, c2, c3)

    def rk3Step(self, c1, c2, c3):
        self.lib.ora_rk3_stage(self.h, c1, c2, c3)

    def cleanEpar(self):
        self.lib.ora_clean(self.h)

    def exchangeFields(self, exchangeB0=False):
        self.lib.ora_exchange(self.h, 1 if exchangeB0 else 0)

    def userInitialize(self):
        self.lib.ora_user_init(self.h)

    def userFieldBoundaryConditions(self, step):
        self.lib.ora_user_bc(self.h, step)

    def mainloop_prologue(self):
        self.lib.ora_prologue(self.h)

    def mainloop(self, steps, step0=0):
        self.lib.ora_step(self.h, steps, step0)

    step = mainloop

    def init_waves(self, bg, modes):
        """Synthetic plane-wave fields (same formula as ffe.Solver.init_waves;
        the sines come from products of per-axis exponentials, so values may
        differ from the library's in the last bit: for timing samples)."""
        import numpy as np
        bgv = (ctypes.c_double * 3)(*[float(x) for x in bg])
        m = np.ascontiguousarray(np.asarray(modes, np.float64).reshape(-1, 11))
        self.lib.ora_init_waves(self.h, bgv, m.shape[0], m.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))

    def synchronize(self, timeout_ms=None):
        pass
