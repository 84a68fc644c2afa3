"""ORACLE -- test infrastructure.  ctypes binding of the C restatement
(oracle/port/*.c).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline import this module, always as the checker / baseline, never as the
measured product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
LIB = ROOT / "oracle" / "_build" / "libmahyco_port.so"


def build() -> Path:
    subprocess.run(["make", "-s", "-f", "oracle/Makefile"], cwd=ROOT, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        from mahyco_gb300 import HydroSpec
        L = C.CDLL(str(LIB))
        vp = C.c_void_p
        L.port_create.argtypes = [C.POINTER(HydroSpec)]
        L.port_create.restype = vp
        L.port_step.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
        L.port_fetch.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double), C.c_size_t]
        L.port_field_size.argtypes = [vp, C.c_char_p]
        L.port_field_size.restype = C.c_size_t
        L.port_time.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_long)]
        L.port_error.argtypes = [vp, C.POINTER(C.c_uint), C.POINTER(C.c_long)]
        L.port_destroy.argtypes = [vp]
        L.port_destroy.restype = None
        L.port_last_error.restype = C.c_char_p
        L.port_num_threads.restype = C.c_int
        _lib = L
    return _lib


class PortRun:
    def __init__(self, spec):
        self.h = lib().port_create(C.byref(spec))
        if not self.h:
            raise RuntimeError("port_create: " + lib().port_last_error().decode())

    def step(self, n: int) -> bool:
        done = C.c_int(0)
        lib().port_step(self.h, n, C.byref(done))
        return bool(done.value)

    def simulate(self, chunk: int = 1000) -> None:
        while not self.step(chunk):
            pass

    def fetch(self, name: str) -> np.ndarray:
        n = lib().port_field_size(self.h, name.encode())
        if n == 0:
            raise KeyError(name)
        out = np.empty(n, dtype=np.float64)
        rc = lib().port_fetch(self.h, name.encode(),
                              out.ctypes.data_as(C.POINTER(C.c_double)), n)
        if rc:
            raise RuntimeError(lib().port_last_error().decode())
        return out

    def time(self):
        t, dt, n = C.c_double(), C.c_double(), C.c_long()
        lib().port_time(self.h, C.byref(t), C.byref(dt), C.byref(n))
        return t.value, dt.value, n.value

    def error(self):
        code, cell = C.c_uint(), C.c_long()
        lib().port_error(self.h, C.byref(code), C.byref(cell))
        return code.value, cell.value

    def close(self):
        if self.h:
            lib().port_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def num_threads() -> int:
    return int(lib().port_num_threads())
