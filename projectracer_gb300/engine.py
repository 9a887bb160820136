"""Python binding of the C ABI in include/ptgpu.h (the engine behind the Fortran drop-in).

``Engine`` drives one GPU context exactly as the reference's time loop drives its subroutines
(main.f90:245-300): ``upload`` = restart read, ``solve_psi`` = velocity solve at the top of a
step, ``step`` = energy_time, ``stats`` = the stats.dat row.  There is no CPU implementation
behind this module: if libptgpu.so is missing or no GPU is present the calls raise.
"""

from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from .config import PtConfig

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libptgpu.so")
HEADER = os.path.join(HERE, "..", "include", "ptgpu.h")

F_T, F_TRATIO, F_TVIS, F_TBUOY, F_CNEW, F_CVIS, F_CBUOY, F_SF, F_U, F_W, F_VIS, F_NEMPTY, F_RHS, F_COUNT_TYPE = range(14)
F_TRACER_R, F_TRACER_S, F_TRACER_T, F_TRACER_C, F_TRACER_TYPE = 20, 21, 22, 23, 24

ERRORS = {-1: "PT_ERR_CONFIG", -2: "PT_ERR_TRACER_OUT_OF_DOMAIN", -3: "PT_ERR_MG_DIVERGED",
          -4: "PT_ERR_MG_MAX_CYCLES", -5: "PT_ERR_SINGULAR_COARSE", -6: "PT_ERR_CUDA", -7: "PT_ERR_STATE",
          -8: "PT_ERR_ITER_CAP", -9: "PT_ERR_ARG", -10: "PT_ERR_NOT_FINITE"}


class PtError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SolveInfo(ctypes.Structure):
    _fields_ = [("cycles", ctypes.c_int32), ("refinements", ctypes.c_int32), ("n_eta", ctypes.c_int32),
                ("n_temp", ctypes.c_int32), ("resid_ratio", ctypes.c_double), ("eig_fine", ctypes.c_double),
                ("ms", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class StatsRow(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("time", "Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg", "mobility",
                                                 "strain_max", "q1", "q2", "q3", "q4")] + \
               [("empty_cells", ctypes.c_int32), ("tracer_min", ctypes.c_int32), ("tracer_max", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("Cavg", ctypes.c_double), ("entrainment", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "pad"}


class EqualizeInfo(ctypes.Structure):
    """pt_equalize_info: the columns of the reference's equalize.dat line."""
    _fields_ = [("tpc_type", ctypes.c_int32 * 2), ("minexcess", ctypes.c_int32 * 2), ("deficit", ctypes.c_int64),
                ("moved", ctypes.c_int64), ("nfree", ctypes.c_int64), ("count_type", ctypes.c_int64 * 2),
                ("passes", ctypes.c_int32), ("nequalize", ctypes.c_int32)]

    def as_dict(self):
        out = {}
        for n, _ in self._fields_:
            v = getattr(self, n)
            out[n] = list(v) if isinstance(v, ctypes.Array) else v
        return out


_LIB = None


def header_symbols() -> list[str]:
    """Entry points declared in include/*.h."""
    inc = os.path.dirname(HEADER)
    names = set()
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(pt_[a-z_0-9]+)\s*\(", text, re.M))
    return sorted(names)


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(path)
    vp, i32, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.pt_init.argtypes = [ctypes.POINTER(PtConfig)]
    L.pt_last_error.restype = ctypes.c_char_p
    L.pt_field_extent.argtypes = [i32] + [ctypes.POINTER(ctypes.c_int32)] * 5
    L.pt_set_field.argtypes = [i32, vp]
    L.pt_get_field.argtypes = [i32, vp]
    L.pt_upload_state.argtypes = [vp] * 10
    L.pt_download_state.argtypes = [vp] * 8
    L.pt_solve_psi.argtypes = [ctypes.POINTER(SolveInfo)]
    L.pt_step.argtypes = [ctypes.POINTER(f64), ctypes.POINTER(SolveInfo)]
    L.pt_stats.argtypes = [ctypes.POINTER(StatsRow)]
    L.pt_equalize_tracers.argtypes = [ctypes.POINTER(EqualizeInfo)]
    L.pt_tracers_to_corners.argtypes = [vp, i32]
    L.pt_time.argtypes = [ctypes.POINTER(f64), ctypes.POINTER(f64)]
    L.pt_set_guess_mode.argtypes = [i32, ctypes.c_char_p]
    L.pt_phase_times.argtypes = [ctypes.POINTER(f64)]
    L.pt_prof_enable.argtypes = [i32]
    L.pt_prof_kernel.argtypes = [i32, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(f64)]
    L.pt_prof_launches.restype = ctypes.c_int64
    L.pt_prof_tracer_order.argtypes = [ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(f64)]
    L.pt_prof_table.argtypes = [i32, vp]
    L.pt_prof_region.argtypes = [i32, ctypes.POINTER(f64)]
    L.pt_prof_residuals.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_int)]
    L.pt_write_snapshot.argtypes = [ctypes.c_char_p, i32]
    L.pt_write_restart.argtypes = [ctypes.c_char_p]
    L.pt_read_restart.argtypes = [ctypes.c_char_p]
    L.pt_prof_record_limit.argtypes = [ctypes.c_int64]
    _LIB = L
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Engine:
    """One engine context (the library keeps one per process)."""

    def __init__(self, cfg: PtConfig):
        self.L = load_library()
        self.cfg = cfg.copy()
        self._check(self.L.pt_init(ctypes.byref(self.cfg)))
        self.nx, self.nz = cfg.nx, cfg.nz

    def _check(self, rc: int):
        if rc != 0:
            raise PtError(rc, self.L.pt_last_error().decode())

    def close(self):
        self.L.pt_finalize()

    def extent(self, field: int):
        v = [ctypes.c_int32() for _ in range(5)]
        self._check(self.L.pt_field_extent(field, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def get(self, field: int) -> np.ndarray:
        lox, hix, loz, hiz, eb = self.extent(field)
        if field >= F_TRACER_R:
            out = np.empty(hix, dtype=np.int32 if eb == 4 else np.float64)
        else:
            out = np.empty((hiz - loz + 1, hix - lox + 1), dtype=np.int32 if eb == 4 else np.float64)
        self._check(self.L.pt_get_field(field, _ptr(out)))
        return out

    def set(self, field: int, arr: np.ndarray):
        arr = np.ascontiguousarray(arr, dtype=np.int32 if field == F_TRACER_TYPE else np.float64)
        self._check(self.L.pt_set_field(field, _ptr(arr)))

    def upload(self, st: dict):
        """Restart upload; st holds the restart arrays, and "Ttype" (int32 0/1) for an engine with
        discrete tracer types (its "Ctr" is then ignored)."""
        arrs = [np.ascontiguousarray(st[k], dtype=np.float64)
                for k in ("xg", "zg", "T", "Cnew", "SF", "rtr", "str", "Ctr", "Ttr")]
        ty = None
        if self.cfg.discrete_types:
            ty = np.ascontiguousarray(st["Ttype"], dtype=np.int32)
        self._check(self.L.pt_upload_state(*[_ptr(a) for a in arrs], None if ty is None else _ptr(ty)))

    def solve_psi(self) -> dict:
        info = SolveInfo()
        self._check(self.L.pt_solve_psi(ctypes.byref(info)))
        return info.as_dict()

    def step(self) -> tuple[float, dict]:
        dt = ctypes.c_double()
        info = SolveInfo()
        self._check(self.L.pt_step(ctypes.byref(dt), ctypes.byref(info)))
        return dt.value, info.as_dict()

    def equalize(self) -> dict:
        """pt_equalize_tracers: one tracer equalisation and the projection that follows it."""
        info = EqualizeInfo()
        self._check(self.L.pt_equalize_tracers(ctypes.byref(info)))
        return info.as_dict()

    def stats(self) -> dict:
        row = StatsRow()
        self._check(self.L.pt_stats(ctypes.byref(row)))
        return row.as_dict()

    def project(self, T0: np.ndarray | None = None, smooth: int = 1):
        t0 = None if T0 is None else np.ascontiguousarray(T0, dtype=np.float64)
        self._check(self.L.pt_tracers_to_corners(None if t0 is None else _ptr(t0), smooth))

    def time(self) -> tuple[float, float]:
        t, dt = ctypes.c_double(), ctypes.c_double()
        self._check(self.L.pt_time(ctypes.byref(t), ctypes.byref(dt)))
        return t.value, dt.value

    def set_guess_mode(self, mode: int, weights: str | None = None):
        self._check(self.L.pt_set_guess_mode(mode, None if weights is None else weights.encode()))

    def prof_enable(self, on: bool = True):
        self._check(self.L.pt_prof_enable(1 if on else 0))

    def prof_reset(self):
        self._check(self.L.pt_prof_reset())

    def prof_kernel(self, kid: int) -> tuple[int, float]:
        n, ms = ctypes.c_int64(), ctypes.c_double()
        self._check(self.L.pt_prof_kernel(kid, ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value

    def region_begin(self):
        self._check(self.L.pt_prof_region(0, None))

    def region_end(self) -> float:
        ms = ctypes.c_double()
        self._check(self.L.pt_prof_region(1, ctypes.byref(ms)))
        return ms.value

    def launches(self) -> int:
        return int(self.L.pt_prof_launches())

    def tracer_order(self) -> tuple[int, float]:
        """(re-sorts by cell since the upload, cell runs per projection thread in the last
        projection); mixed precision, where the tracer order is internal."""
        n, runs = ctypes.c_int64(), ctypes.c_double()
        self._check(self.L.pt_prof_tracer_order(ctypes.byref(n), ctypes.byref(runs)))
        return n.value, runs.value

    def resorts(self) -> int:
        return self.tracer_order()[0]

    def table(self, which: int) -> np.ndarray:
        """The mixed RK stage's FP32 table `which` (0 u, 1 w, 2 tracer-space term): array of
        shape (nz+7, nx+1, 4), rows k = -3..nz+3, [value, d/dx, d2/dx2, d3/dx3]."""
        out = np.empty((self.nz + 7, self.nx + 1, 4), dtype=np.float32)
        self._check(self.L.pt_prof_table(which, _ptr(out)))
        return out

    def write_snapshot(self, directory: str, fcount: int = 0):
        """T<10000+fcount> and P<10000+fcount> of the current state (asynchronous: see io_wait)."""
        self._check(self.L.pt_write_snapshot(directory.encode(), fcount))

    def write_restart(self, directory: str):
        """Trestart and restart_tracers of the current state (asynchronous: see io_wait)."""
        self._check(self.L.pt_write_restart(directory.encode()))

    def read_restart(self, directory: str):
        """Restart read of Trestart and restart_tracers, then the upload (pt_read_restart)."""
        self._check(self.L.pt_read_restart(directory.encode()))

    def io_wait(self):
        self._check(self.L.pt_io_wait())

    def residuals(self) -> list[float]:
        """Relative residual at each convergence test of the last psi solve (kept after a failed
        solve)."""
        n = ctypes.c_int()
        self._check(self.L.pt_prof_residuals(None, 0, ctypes.byref(n)))
        out = np.zeros(max(1, n.value))
        self._check(self.L.pt_prof_residuals(_ptr(out), n.value, ctypes.byref(n)))
        return list(out[:n.value])

    def phase_times(self) -> list[float]:
        v = (ctypes.c_double * 8)()
        self._check(self.L.pt_phase_times(v))
        return list(v)
