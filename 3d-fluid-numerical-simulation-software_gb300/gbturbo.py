"""Python host of the GB300 residual-and-update path: a thin ctypes layer over the C-ABI in
include/gbturbo.h (libgbturbo.so, built in-tree by build.py).

The method names follow the reference solver's call surface (CSolver::Solver, CMesh::ResFlux,
CMesh::Time_Marching, CMesh::Res_Calculate, COutput::OutputGeneralParameters, ...). There is no
CPU fallback: if the library is missing, importing the solver raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence, Union

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbturbo.so")

FP64 = 0
MIXED = 1

_lib: Optional[ctypes.CDLL] = None


def load() -> ctypes.CDLL:
    """Loads libgbturbo.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run build.py (the GPU path has no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
    sig = {
        "gb_solver_create": ([ctypes.POINTER(ctypes.c_char_p), ip, ip, ctypes.POINTER(vp)], ip),
        "gb_solver_create_levels": ([ctypes.POINTER(ctypes.c_char_p), ip, ip, ip, ctypes.POINTER(vp)], ip),
        "gb_solver_destroy": ([vp], ip),
        "gb_last_error": ([], ctypes.c_char_p),
        "gb_dims": ([vp, ip, ip, ctypes.POINTER(ip)], ip),
        "gb_num_blocks": ([vp, ctypes.POINTER(ip), ctypes.POINTER(ip)], ip),
        "gb_case_blocks": ([vp, ip, ctypes.POINTER(ip)], ip),
        "gb_case_info": ([ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong), dp, ctypes.c_longlong], ip),
        "gb_init_uniform": ([vp], ip),
        "gb_start_from_fine_state": ([vp], ip),
        "gb_ws_create": ([ctypes.c_uint, ctypes.POINTER(vp)], ip),
        "gb_ws_destroy": ([vp], ip),
        "gb_ws_num_params": ([], ctypes.c_long),
        "gb_ws_add_solves": ([vp, vp, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_samples": ([vp], ctypes.c_longlong),
        "gb_ws_train": ([vp, ip, ip, ctypes.c_float, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_apply": ([vp, vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ip), dp, dp], ip),
        "gb_ws_get_params": ([vp, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_set_params": ([vp, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_get_norm": ([vp, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_set_norm": ([vp, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_forward": ([vp, ctypes.POINTER(ctypes.c_float), ip, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_forward_backward": ([vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ip,
                                    ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)], ip),
        "gb_ws_benchmark": ([vp, ctypes.c_longlong, ip, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                             ctypes.POINTER(ctypes.c_float), dp], ip),
        "gb_resflux": ([vp, ip], ip),
        "gb_time_marching": ([vp, ip], ip),
        "gb_res_calculate": ([vp, ip, dp], ip),
        "gb_res_calculate_noalloc": ([vp, ip, dp], ip),
        "gb_primitive_vars": ([vp, ip], ip),
        "gb_limit_vars": ([vp, ip], ip),
        "gb_corner_treatment": ([vp, ip], ip),
        "gb_restrict": ([vp], ip),
        "gb_interpolate": ([vp, ip], ip),
        "gb_delta_cons": ([vp], ip),
        "gb_set_use_force": ([vp, ip, ip], ip),
        "gb_solver_step": ([vp], ip),
        "gb_integrals": ([vp, ip, dp], ip),
        "gb_iterate": ([vp, ip, dp], ip),
        "gb_get_status": ([vp, ctypes.POINTER(ip)], ip),
        "gb_get_field": ([vp, ip, ip, ctypes.c_char_p, dp, ctypes.c_long], ctypes.c_long),
        "gb_set_cv": ([vp, ip, ip, dp, ctypes.c_long], ip),
        "gb_sync": ([vp], ip),
        "gb_mass_flow_imposed": ([vp], ip),
        "gb_get_outlet_pressure": ([vp, dp], ip),
        "gb_read_restart": ([vp, ip, ctypes.c_char_p], ip),
        "gb_write_restart": ([vp, ip, ctypes.c_char_p], ip),
        "gb_write_solution": ([vp, ip, ctypes.c_char_p], ip),
        "gb_set_graphs": ([vp, ip], ip),
        "gb_sweep_tuning": ([vp, ip, ctypes.POINTER(ip)], ip),
        "gb_face_staging": ([vp, ip, ctypes.POINTER(ip)], ip),
        "gb_profile_begin": ([vp], ip),
        "gb_profile_end": ([vp, ctypes.c_char_p, ip], ip),
        "gb_timer_start": ([vp], ip),
        "gb_timer_stop": ([vp, ctypes.POINTER(ctypes.c_float)], ip),
        "gb_fp64_rate": ([dp], ip),
        "gb_fp64_arith_check": ([ip, dp, dp, ctypes.c_longlong, dp], ip),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


EXPORTED = ["gb_solver_create", "gb_solver_destroy", "gb_last_error", "gb_dims", "gb_init_uniform",
            "gb_resflux", "gb_time_marching", "gb_res_calculate", "gb_primitive_vars", "gb_limit_vars",
            "gb_corner_treatment", "gb_restrict", "gb_interpolate", "gb_delta_cons", "gb_set_use_force",
            "gb_solver_step", "gb_integrals", "gb_iterate", "gb_get_status", "gb_get_field", "gb_set_cv",
            "gb_sync", "gb_set_graphs", "gb_timer_start", "gb_timer_stop", "gb_profile_begin", "gb_profile_end",
            "gb_res_calculate_noalloc", "gb_sweep_tuning", "gb_read_restart", "gb_write_restart",
            "gb_write_solution", "gb_mass_flow_imposed", "gb_get_outlet_pressure", "gb_num_blocks",
            "gb_case_blocks", "gb_case_info", "gb_solver_create_levels", "gb_start_from_fine_state", "gb_ws_create", "gb_ws_destroy",
            "gb_ws_num_params", "gb_ws_add_solves", "gb_ws_samples", "gb_ws_train", "gb_ws_apply", "gb_ws_get_params",
            "gb_ws_set_params", "gb_ws_get_norm", "gb_ws_set_norm", "gb_ws_forward", "gb_ws_forward_backward",
            "gb_ws_benchmark", "gb_fp64_rate", "gb_fp64_arith_check", "gb_face_staging"]


class GBError(RuntimeError):
    pass


CASE_INFO_KEYS = ["blocks", "levels", "inlets", "outlets", "walls", "periodic_pairs", "interfaces", "mixing_planes", "nodes"]


def case_info(case_dir: str, nodes: bool = False):
    """Reads a case directory on the host only (the solver's reader and checks, no GPU): a dict of
    CASE_INFO_KEYS, and with nodes=True also the (n, 3) node coordinates, block after block."""
    L = load()
    info = (ctypes.c_longlong * 9)()
    rc = L.gb_case_info(os.path.abspath(case_dir).encode(), info, None, 0)
    if rc != 0:
        raise GBError(L.gb_last_error().decode())
    d = dict(zip(CASE_INFO_KEYS, [int(v) for v in info]))
    if not nodes:
        return d
    xyz = np.zeros(3 * d["nodes"])
    rc = L.gb_case_info(os.path.abspath(case_dir).encode(), info, _dp(xyz), xyz.size)
    if rc != 0:
        raise GBError(L.gb_last_error().decode())
    return d, xyz.reshape(-1, 3)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fp64_rate() -> float:
    """FP64 arithmetic rate of the current device in FLOP/s (two per FMA), measured by a device-timed
    loop of independent FMA chains over every SM: the roof of the FP64 form's compute-bound kernels."""
    L = load()
    v = ctypes.c_double(0.0)
    rc = L.gb_fp64_rate(ctypes.byref(v))
    if rc != 0:
        raise GBError(f"gb_fp64_rate failed ({rc})")
    return float(v.value)


def fp64_arith_check(op: int, x: np.ndarray, y: Optional[np.ndarray] = None) -> np.ndarray:
    """the device's FP64 arithmetic on host arrays: op 0 x / y, 1 sqrt(x), 2 1 / x as the FP64 form's
    kernels compute them (Newton-refined), 3 and 4 the IEEE x / y and sqrt(x); 5 x split into a
    pair of FP32 numbers and summed back, 6 and 7 x rounded to FP32 and widened back by integer
    operations / by the conversion instructions"""
    L = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    yy = None if y is None else np.ascontiguousarray(y, dtype=np.float64)
    out = np.empty_like(x)
    rc = L.gb_fp64_arith_check(op, _dp(x), None if yy is None else _dp(yy), x.size, _dp(out))
    if rc != 0:
        raise GBError(f"gb_fp64_arith_check failed ({rc})")
    return out


FIELD_SHAPES = {
    "cv": lambda I, J, K: (I + 1, J + 1, K + 1, 5), "pv": lambda I, J, K: (I + 1, J + 1, K + 1, 6),
    "mut": lambda I, J, K: (I + 1, J + 1, K + 1, 1),
    "res": lambda I, J, K: (I - 1, J - 1, K - 1, 5), "dq": lambda I, J, K: (I - 1, J - 1, K - 1, 5),
    "FcI": lambda I, J, K: (I, J - 1, K - 1, 5), "FcJ": lambda I, J, K: (I - 1, J, K - 1, 5),
    "FcK": lambda I, J, K: (I - 1, J - 1, K, 5), "FvI": lambda I, J, K: (I, J - 1, K - 1, 5),
    "FvJ": lambda I, J, K: (I - 1, J, K - 1, 5), "FvK": lambda I, J, K: (I - 1, J - 1, K, 5),
    "faceI": lambda I, J, K: (I, J - 1, K - 1, 18), "faceJ": lambda I, J, K: (I - 1, J, K - 1, 18),
    "faceK": lambda I, J, K: (I - 1, J - 1, K, 18), "cell": lambda I, J, K: (I - 1, J - 1, K - 1, 13),
    "totalvol": lambda I, J, K: (1,),
}
FIELD_SHAPES["ev"] = lambda I, J, K: (I + 1, J + 1, K + 1, 1)        # Spalart-Allmaras cases
for _n in ("dt", "omega", "lamcI", "lamcJ", "lamcK", "lamvI", "lamvJ", "lamvK", "res_ev", "dwall"):
    FIELD_SHAPES[_n] = lambda I, J, K: (I - 1, J - 1, K - 1, 1)
for _d, _f in (("I", lambda I, J, K: (2, J - 1, K - 1)), ("J", lambda I, J, K: (I - 1, 2, K - 1)),
               ("K", lambda I, J, K: (I - 1, J - 1, 2))):
    for _s in ("S", "P"):
        FIELD_SHAPES[f"d{_d}{_s}_cv"] = (lambda f: lambda I, J, K: f(I, J, K) + (5,))(_f)
        FIELD_SHAPES[f"d{_d}{_s}_pv"] = (lambda f: lambda I, J, K: f(I, J, K) + (6,))(_f)

HIST_COLUMNS = ["iter", "res_dens", "res_xmom", "res_ymom", "res_zmom", "res_ener", "m_in", "m_out", "PR",
                "eta", "m_ratio", "CFL"]


class Solver:
    """A batch of operating points, each read from a reference case directory. Per-solve results
    (norms, integrals, history, status) have one entry per case directory; box access (dims, get,
    set_cv) takes a slot: the blocks of case 0 come first, then those of case 1, ... (slots())."""

    def __init__(self, case_dirs: Union[str, Sequence[str]], precision: int = FP64, levels: int = 2):
        self._L = load()
        if isinstance(case_dirs, str):
            case_dirs = [case_dirs]
        self.case_dirs = [os.path.abspath(d) for d in case_dirs]
        arr = (ctypes.c_char_p * len(self.case_dirs))(*[d.encode() for d in self.case_dirs])
        h = ctypes.c_void_p()
        if levels == 2:
            rc = self._L.gb_solver_create(arr, len(self.case_dirs), precision, ctypes.byref(h))
        else:       # the three-level V-cycle extension
            rc = self._L.gb_solver_create_levels(arr, len(self.case_dirs), precision, levels, ctypes.byref(h))
        if rc != 0:
            raise GBError(self._L.gb_last_error().decode())
        self.h = h
        self.n = len(self.case_dirs)
        nc, nb = ctypes.c_int(), ctypes.c_int()
        self._ck(self._L.gb_num_blocks(self.h, ctypes.byref(nc), ctypes.byref(nb)))
        self.n_slots = nb.value
        self.precision = precision
        self.ng = self.dims(0, 1)[3]

    def _ck(self, rc: int) -> None:
        if rc != 0:
            raise GBError(self._L.gb_last_error().decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            self._L.gb_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def slots(self, solve: int = 0) -> range:
        """the slots holding the blocks of one case, in block order"""
        v = (ctypes.c_int * 2)()
        self._ck(self._L.gb_case_blocks(self.h, solve, v))
        return range(v[0], v[0] + v[1])

    # ---- reference call surface
    def dims(self, solve: int = 0, level: int = 1):
        d = (ctypes.c_int * 4)()
        self._ck(self._L.gb_dims(self.h, solve, level, d))
        return tuple(d)

    def init_uniform(self) -> None:
        self._ck(self._L.gb_init_uniform(self.h))

    def resflux(self, level: int = 1) -> None:
        self._ck(self._L.gb_resflux(self.h, level))

    def time_marching(self, level: int = 1) -> None:
        self._ck(self._L.gb_time_marching(self.h, level))

    def res_calculate(self, level: int = 1) -> np.ndarray:
        out = np.zeros(5 * self.n)
        self._ck(self._L.gb_res_calculate(self.h, level, _dp(out)))
        return out.reshape(self.n, 5)

    def res_calculate_noalloc(self, level: int = 1) -> np.ndarray:
        """gb_res_calculate_noalloc: the same norms with the library's static scratch, no allocation."""
        out = np.zeros(5 * self.n)
        self._ck(self._L.gb_res_calculate_noalloc(self.h, level, _dp(out)))
        return out.reshape(self.n, 5)

    def primitive_vars(self, level: int = 1) -> None:
        self._ck(self._L.gb_primitive_vars(self.h, level))

    def limit_vars(self, level: int = 1) -> None:
        self._ck(self._L.gb_limit_vars(self.h, level))

    def corner_treatment(self, level: int = 2) -> None:
        self._ck(self._L.gb_corner_treatment(self.h, level))

    def restrict(self) -> None:
        self._ck(self._L.gb_restrict(self.h))

    def interpolate(self, init: bool = False) -> None:
        self._ck(self._L.gb_interpolate(self.h, int(init)))

    def delta_cons(self) -> None:
        self._ck(self._L.gb_delta_cons(self.h))

    def set_use_force(self, level: int, on: bool) -> None:
        self._ck(self._L.gb_set_use_force(self.h, level, int(on)))

    def solver_step(self) -> None:
        self._ck(self._L.gb_solver_step(self.h))

    def integrals(self, level: int = 1) -> np.ndarray:
        out = np.zeros(5 * self.n)
        self._ck(self._L.gb_integrals(self.h, level, _dp(out)))
        return out.reshape(self.n, 5)

    def iterate(self, n: int, history: bool = True) -> Optional[np.ndarray]:
        """n driver iterations; with history, returns an array (n, n_solves, 12) of HIST_COLUMNS."""
        if history:
            out = np.zeros((n, self.n, 12))
            self._ck(self._L.gb_iterate(self.h, n, _dp(out)))
            return out
        self._ck(self._L.gb_iterate(self.h, n, None))
        return None

    def status(self) -> np.ndarray:
        out = (ctypes.c_int * self.n)()
        self._ck(self._L.gb_get_status(self.h, out))
        return np.array(out[:])

    def get(self, name: str, solve: int = 0, level: int = 1) -> np.ndarray:
        I, J, K, _ = self.dims(solve, level)
        shape = FIELD_SHAPES[name](I, J, K)
        out = np.zeros(int(np.prod(shape)))
        n = self._L.gb_get_field(self.h, solve, level, name.encode(), _dp(out), out.size)
        if n < 0:
            raise GBError(self._L.gb_last_error().decode())
        return out.reshape(shape)

    def set_cv(self, cv: np.ndarray, solve: int = 0, level: int = 1) -> None:
        a = np.ascontiguousarray(cv, dtype=np.float64).ravel()
        self._ck(self._L.gb_set_cv(self.h, solve, level, _dp(a), a.size))

    def start_from_fine_state(self) -> None:
        """after init_uniform and set_cv of the fine level of every slot: the iterations run full
        cycles from that field"""
        self._ck(self._L.gb_start_from_fine_state(self.h))

    # ---- the reference's solution files (a None path: the file in the solve's case directory)
    def read_restart(self, solve: int = 0, path: Optional[str] = None) -> None:
        self._ck(self._L.gb_read_restart(self.h, solve, path.encode() if path else None))

    def write_restart(self, solve: int = 0, path: Optional[str] = None) -> None:
        self._ck(self._L.gb_write_restart(self.h, solve, path.encode() if path else None))

    def write_solution(self, solve: int = 0, path: Optional[str] = None) -> None:
        self._ck(self._L.gb_write_solution(self.h, solve, path.encode() if path else None))

    def mass_flow_imposed(self) -> None:
        self._ck(self._L.gb_mass_flow_imposed(self.h))

    def outlet_pressure(self) -> np.ndarray:
        """current nondimensional back pressure of every solve"""
        out = np.zeros(self.n)
        self._ck(self._L.gb_get_outlet_pressure(self.h, _dp(out)))
        return out

    def sync(self) -> None:
        self._ck(self._L.gb_sync(self.h))

    def sweep_tuning(self, level: int = 1) -> tuple:
        """(cells per warp, warps per block) the sweep autotuner chose for a level"""
        v = (ctypes.c_int * 2)()
        self._ck(self._L.gb_sweep_tuning(self.h, level, v))
        return int(v[0]), int(v[1])

    def face_staging(self, level: int = 1) -> bool:
        """True when the level's face stage runs on TMA-staged tiles (the mixed form's default scheme
        on meshes with KM = 4n + 1 >= 33)"""
        v = ctypes.c_int(0)
        self._ck(self._L.gb_face_staging(self.h, level, ctypes.byref(v)))
        return bool(v.value)

    def set_graphs(self, on: bool) -> None:
        self._ck(self._L.gb_set_graphs(self.h, int(on)))

    def profile_begin(self) -> None:
        self._ck(self._L.gb_profile_begin(self.h))

    def profile_end(self) -> dict:
        """stage -> (device milliseconds, kernel launches, [evaluations on level 1, 2, 3])"""
        buf = ctypes.create_string_buffer(8192)
        self._ck(self._L.gb_profile_end(self.h, buf, 8192))
        out = {}
        for item in buf.value.decode().split(";"):
            if item:
                name, ms, n, per_level = item.split(":")
                out[name] = (float(ms), int(n), [int(v) for v in per_level.split(",")])
        return out

    def timer_start(self) -> None:
        self._ck(self._L.gb_timer_start(self.h))

    def timer_stop(self) -> float:
        ms = ctypes.c_float()
        self._ck(self._L.gb_timer_stop(self.h, ctypes.byref(ms)))
        return float(ms.value)


WS_IN, WS_OUT, WS_OUT_USED, WS_PARAMS, WS_NORM = 64, 16, 6, 3, 24


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class WarmStart:
    """The learned warm start (gb_ws_*): a coordinate MLP trained on fine-level fields of solves
    this library ran, giving new cases their starting field, with the uniform start as the
    fallback. Case parameters: WS_PARAMS floats per case (operating-point descriptors)."""

    def __init__(self, seed: int = 0):
        self._L = load()
        h = ctypes.c_void_p()
        if self._L.gb_ws_create(int(seed), ctypes.byref(h)) != 0:
            raise GBError(self._L.gb_last_error().decode())
        self.h = h
        self.n_params = int(self._L.gb_ws_num_params())

    def close(self):
        if self.h:
            self._L.gb_ws_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise GBError(self._L.gb_last_error().decode())

    @staticmethod
    def _params(params, n):
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).reshape(n, WS_PARAMS))
        return p

    def add_solves(self, solver: "Solver", params) -> None:
        p = self._params(params, solver.n)
        self._check(self._L.gb_ws_add_solves(self.h, solver.h, _fptr(p)))

    @property
    def samples(self) -> int:
        return int(self._L.gb_ws_samples(self.h))

    def train(self, steps: int, batch: int = 32768, lr: float = 1e-3) -> float:
        loss = ctypes.c_float()
        self._check(self._L.gb_ws_train(self.h, int(steps), int(batch), float(lr), ctypes.byref(loss)))
        return float(loss.value)

    def apply(self, solver: "Solver", params):
        """per case: (used, residual sum of the network's field, of the uniform start)"""
        p = self._params(params, solver.n)
        used = (ctypes.c_int * solver.n)()
        rw = np.zeros(solver.n)
        ru = np.zeros(solver.n)
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self._L.gb_ws_apply(self.h, solver.h, _fptr(p), used, rw.ctypes.data_as(dp), ru.ctypes.data_as(dp)))
        return np.array(list(used), dtype=np.int32), rw, ru

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        self._check(self._L.gb_ws_get_params(self.h, _fptr(out)))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(np.asarray(p, dtype=np.float32).reshape(self.n_params))
        self._check(self._L.gb_ws_set_params(self.h, _fptr(p)))

    def get_norm(self) -> np.ndarray:
        out = np.zeros(WS_NORM, dtype=np.float32)
        self._check(self._L.gb_ws_get_norm(self.h, _fptr(out)))
        return out

    def set_norm(self, v) -> None:
        v = np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(WS_NORM))
        self._check(self._L.gb_ws_set_norm(self.h, _fptr(v)))

    def forward(self, feat) -> np.ndarray:
        f = np.ascontiguousarray(np.asarray(feat, dtype=np.float32))
        n = f.shape[0]
        y = np.zeros((n, WS_OUT), dtype=np.float32)
        self._check(self._L.gb_ws_forward(self.h, _fptr(f), n, _fptr(y)))
        return y

    def forward_backward(self, feat, target):
        f = np.ascontiguousarray(np.asarray(feat, dtype=np.float32))
        t = np.ascontiguousarray(np.asarray(target, dtype=np.float32).reshape(f.shape[0], WS_OUT_USED))
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_float()
        self._check(self._L.gb_ws_forward_backward(self.h, _fptr(f), _fptr(t), f.shape[0], ctypes.byref(loss), _fptr(g)))
        return float(loss.value), g

    def benchmark(self, rows: int, iters: int = 20):
        """device ms per layer-by-layer forward pass, per forward-and-backward pass and per fused
        inference pass over rows random rows, and the largest difference between the two forward
        passes' outputs"""
        f, b, i, dmax = ctypes.c_float(), ctypes.c_float(), ctypes.c_float(), ctypes.c_double()
        self._check(self._L.gb_ws_benchmark(self.h, int(rows), int(iters), ctypes.byref(f), ctypes.byref(b),
                                            ctypes.byref(i), ctypes.byref(dmax)))
        return float(f.value), float(b.value), float(i.value), float(dmax.value)
