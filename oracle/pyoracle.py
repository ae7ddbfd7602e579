"""ctypes binding of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``; the GPU
product never imports it. ``build()`` compiles the library with the oracle's Makefile.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
# the reference's default FP32 build of the path (REAL = float): CPU timing beside the mixed form
LIB32_PATH = os.path.join(HERE, "_build", "liboracle32.so")
_libs: Dict[bool, ctypes.CDLL] = {}


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < os.path.getmtime(src) for p in (LIB_PATH, LIB32_PATH)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib(fp32: bool = False) -> ctypes.CDLL:
    if fp32 not in _libs:
        build()
        L = ctypes.CDLL(LIB32_PATH if fp32 else LIB_PATH)
        L.orc_open.restype = ctypes.c_void_p
        L.orc_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        L.orc_close.argtypes = [ctypes.c_void_p]
        L.orc_iterate.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        L.orc_iterate.restype = ctypes.c_int
        L.orc_resflux.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_dims.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.orc_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p,
                              ctypes.POINTER(ctypes.c_double), ctypes.c_long]
        L.orc_get.restype = ctypes.c_long
        L.orc_set_cv.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_long]
        L.orc_set_cv.restype = ctypes.c_int
        L.orc_cfl.argtypes = [ctypes.c_void_p]
        L.orc_cfl.restype = ctypes.c_double
        _libs[fp32] = L
    return _libs[fp32]


SHAPES = {
    "cv": lambda I, J, K: (I + 1, J + 1, K + 1, 5), "pv": lambda I, J, K: (I + 1, J + 1, K + 1, 6),
    "mut": lambda I, J, K: (I + 1, J + 1, K + 1, 1),
    "res": lambda I, J, K: (I - 1, J - 1, K - 1, 5), "Fc": lambda I, J, K: (I - 1, J - 1, K - 1, 5),
    "Fv": lambda I, J, K: (I - 1, J - 1, K - 1, 5),
    "FcI": lambda I, J, K: (I, J - 1, K - 1, 5), "FcJ": lambda I, J, K: (I - 1, J, K - 1, 5),
    "FcK": lambda I, J, K: (I - 1, J - 1, K, 5),
    "FvI": lambda I, J, K: (I, J - 1, K - 1, 5), "FvJ": lambda I, J, K: (I - 1, J, K - 1, 5),
    "FvK": lambda I, J, K: (I - 1, J - 1, K, 5),
    "faceI": lambda I, J, K: (I, J - 1, K - 1, 18), "faceJ": lambda I, J, K: (I - 1, J, K - 1, 18),
    "faceK": lambda I, J, K: (I - 1, J - 1, K, 18), "cell": lambda I, J, K: (I - 1, J - 1, K - 1, 13),
    "totalvol": lambda I, J, K: (1,),
}
for _n in ("dt", "omega", "lamcI", "lamcJ", "lamcK", "lamvI", "lamvJ", "lamvK"):
    SHAPES[_n] = lambda I, J, K: (I - 1, J - 1, K - 1, 1)
for _d, _f in (("I", lambda I, J, K: (2, J - 1, K - 1)), ("J", lambda I, J, K: (I - 1, 2, K - 1)),
               ("K", lambda I, J, K: (I - 1, J - 1, 2))):
    for _s in ("S", "P"):
        SHAPES[f"d{_d}{_s}_cv"] = (lambda f: lambda I, J, K: f(I, J, K) + (5,))(_f)
        SHAPES[f"d{_d}{_s}_pv"] = (lambda f: lambda I, J, K: f(I, J, K) + (6,))(_f)


class Oracle:
    """One CPU solve of a case directory (config.dat + grid + BoundaryDefinition.dat)."""

    def __init__(self, case_dir: str, fp32: bool = False):
        self._L = lib(fp32)
        err = ctypes.create_string_buffer(512)
        h = self._L.orc_open(case_dir.encode(), err, 512)
        if not h:
            raise RuntimeError("oracle: " + err.value.decode())
        self.h = ctypes.c_void_p(h)

    def close(self) -> None:
        if self.h:
            self._L.orc_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dims(self, level: int = 1):
        d = (ctypes.c_int * 4)()
        self._L.orc_dims(self.h, level, d)
        return d[0], d[1], d[2], d[3]

    def iterate(self) -> np.ndarray:
        row = (ctypes.c_double * 12)()
        self._L.orc_iterate(self.h, row)
        return np.array(row[:])

    def run(self, n: int) -> np.ndarray:
        return np.stack([self.iterate() for _ in range(n)])

    def resflux(self, level: int = 1) -> None:
        self._L.orc_resflux(self.h, level)

    def get(self, name: str, level: int = 1) -> np.ndarray:
        I, J, K, _ = self.dims(level)
        shape = SHAPES[name](I, J, K)
        out = np.zeros(int(np.prod(shape)))
        n = self._L.orc_get(self.h, level, name.encode(),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size)
        if n < 0:
            raise KeyError(name)
        return out.reshape(shape)

    def set_cv(self, cv: np.ndarray, level: int = 1) -> None:
        a = np.ascontiguousarray(cv, dtype=np.float64).ravel()
        if self._L.orc_set_cv(self.h, level, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), a.size):
            raise ValueError("bad state size")

    def cfl(self) -> float:
        return float(self._L.orc_cfl(self.h))
