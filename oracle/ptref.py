"""ctypes wrapper of the CPU oracle (libptref.so).

Test infrastructure only: imported by tests/, by __graft_entry__.smoke() to check its GPU result, and by
bench.py's CPU-baseline leg.  The product package never imports this module.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from projectracer_gb300.config import PtConfig

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build(force: bool = False) -> str:
    path = os.path.join(_HERE, "libptref.so")
    srcs = [os.path.join(_HERE, f) for f in os.listdir(_HERE) if f.endswith((".c", ".h"))]
    srcs.append(os.path.join(_HERE, "..", "include", "ptgpu.h"))
    stale = not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in srcs)
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE, "libptref.so"], check=True)
    return path


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build())
        L = _LIB
        vp, i32, f64, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64
        L.ptref_create.restype = vp
        L.ptref_create.argtypes = [ctypes.POINTER(PtConfig), i32, i32]
        L.ptref_error.restype = ctypes.c_char_p
        L.ptref_error.argtypes = [vp]
        L.ptref_init_reference.argtypes = [vp, i32, i32, f64, f64, i32]
        L.ptref_load_restart.argtypes = [vp] + [vp] * 9
        L.ptref_set_types.argtypes = [vp, vp]
        L.ptref_solve_psi.argtypes = [vp]
        L.ptref_step.argtypes = [vp]
        L.ptref_equalize.argtypes = [vp, ctypes.c_int64, vp]
        L.ptref_stats.argtypes = [vp, vp]
        L.ptref_project.argtypes = [vp, vp, vp, vp, vp, i32]
        L.ptref_get_field.argtypes = [vp, i32, vp]
        L.ptref_set_field.argtypes = [vp, i32, vp]
        L.ptref_get_scalar.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(f64)]
        L.ptref_compute_derivatives.argtypes = [vp, vp, vp]
        L.ptref_interpolate.restype = f64
        L.ptref_interpolate.argtypes = [vp, f64, f64, vp, vp]
        L.ptref_load_tracer_space.argtypes = [vp, vp]
        L.ptref_velocities.argtypes = [vp]
        L.ptref_smoother_T.argtypes = [vp, vp]
        L.ptref_band_lu.argtypes = [i32, i32, i32, vp, i32, vp]
        L.ptref_band_solve.argtypes = [i32, i32, i32, vp, i32, vp, vp]
        L.ptref_band_equ.argtypes = [i32, i32, i32, vp, i32, vp]
        del i64
    return _LIB


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class StatsRow(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("time", "Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg",
                                                 "mobility", "strain_max", "q1", "q2", "q3", "q4")] + \
               [("empty_cells", ctypes.c_int32), ("tracer_min", ctypes.c_int32),
                ("tracer_max", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("Cavg", ctypes.c_double), ("entrainment", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "pad"}


FIELD_GHOST = {0: 3, 1: 3, 2: 3, 3: 3, 4: 5, 5: 5, 6: 5, 7: 3, 8: 3, 9: 3, 10: 3}


class Oracle:
    """One oracle state.  iterate=1 multigrid, 0 direct banded solve.  nparts: emulated OpenMP
    partitions of the reference's sums (>=1), or 0 for the GPU's canonical projection order."""

    def __init__(self, cfg: PtConfig, iterate: int = 1, nparts: int = 1):
        self.cfg = cfg
        self.L = lib()
        self.h = self.L.ptref_create(ctypes.byref(cfg), iterate, nparts)
        self.nx, self.nz = cfg.nx, cfg.nz
        self.check(0)

    def check(self, rc: int):
        if rc != 0:
            raise RuntimeError(f"oracle error {rc}: {self.L.ptref_error(self.h).decode()}")
        err = self.L.ptref_error(self.h).decode()
        if err:
            raise RuntimeError(f"oracle error: {err}")

    def shape(self, field_id: int):
        g = FIELD_GHOST[field_id]
        return (self.nz + 2 * g + 1, self.nx + 2 * g + 1)

    def get(self, field_id: int) -> np.ndarray:
        if field_id in (11, 13):
            out = np.zeros((self.nz + 1, self.nx + 1), dtype=np.int32)
        elif field_id == 24:
            out = np.zeros(self.cfg.ntr, dtype=np.int32)
        elif field_id == 12:
            out = np.zeros((self.nz - 1, self.nx - 1), dtype=np.float64)
        elif field_id >= 20:
            out = np.zeros(self.cfg.ntr, dtype=np.float64)
        else:
            out = np.zeros(self.shape(field_id), dtype=np.float64)
        self.check(self.L.ptref_get_field(self.h, field_id, _ptr(out)))
        return out

    def set(self, field_id: int, arr: np.ndarray):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        self.check(self.L.ptref_set_field(self.h, field_id, _ptr(arr)))

    def scalar(self, name: str) -> float:
        v = ctypes.c_double()
        self.check(self.L.ptref_get_scalar(self.h, name.encode(), ctypes.byref(v)))
        return v.value

    def init_reference(self, tpc: int, nthreads_rng: int, klayer: float, dlayer: float,
                       boundary_heating: int = 1):
        self.check(self.L.ptref_init_reference(self.h, tpc, nthreads_rng, klayer, dlayer, boundary_heating))

    def set_types(self, Ttype):
        """Discrete tracer types 0/1 (call before load_restart): the projection becomes
        tracers_to_corners_OG."""
        self._types = np.ascontiguousarray(Ttype, dtype=np.int32)
        self.check(self.L.ptref_set_types(self.h, _ptr(self._types)))

    def load_restart(self, xg, zg, T, Cnew, SF, rtr, str_, Ctr, Ttr):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (xg, zg, T, Cnew, SF, rtr, str_, Ctr, Ttr)]
        self._keep = arrs
        self.check(self.L.ptref_load_restart(self.h, *[_ptr(a) for a in arrs]))

    def solve_psi(self):
        self.check(self.L.ptref_solve_psi(self.h))

    def step(self):
        self.check(self.L.ptref_step(self.h))

    def equalize(self, call_index: int | None = None) -> dict:
        """ptref_equalize: the equalisation with call index `call_index` (default: the next one of
        this run), then the projection."""
        from projectracer_gb300.engine import EqualizeInfo

        info = EqualizeInfo()
        call_index = -1 if call_index is None else call_index
        self.check(self.L.ptref_equalize(self.h, call_index, ctypes.byref(info)))
        return info.as_dict()

    def stats(self) -> dict:
        row = StatsRow()
        self.check(self.L.ptref_stats(self.h, ctypes.byref(row)))
        return row.as_dict()

    def project(self, r, s, T, T0=None, smooth=1):
        r, s, T = (np.ascontiguousarray(a, dtype=np.float64) for a in (r, s, T))
        t0 = None if T0 is None else np.ascontiguousarray(T0, dtype=np.float64)
        self.check(self.L.ptref_project(self.h, _ptr(r), _ptr(s), _ptr(T),
                                        None if t0 is None else _ptr(t0), smooth))

    def compute_derivatives(self, f: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.zeros((self.nz + 7, self.nx + 1, 3), dtype=np.float64)
        self.check(self.L.ptref_compute_derivatives(self.h, _ptr(f), _ptr(out)))
        return out

    def interpolate(self, r: float, s: float, DERr: np.ndarray, f: np.ndarray) -> float:
        return self.L.ptref_interpolate(self.h, r, s, _ptr(DERr), _ptr(f))

    def tracer_space(self) -> np.ndarray:
        out = np.zeros((self.nz + 7, self.nx + 7), dtype=np.float64)
        self.check(self.L.ptref_load_tracer_space(self.h, _ptr(out)))
        return out


def band_lu(ab: np.ndarray, n: int, kl: int, ku: int):
    """LU of a band matrix in LAPACK storage ab[ldab, n] (Fortran order), in place."""
    ab = np.asfortranarray(ab)
    ipiv = np.zeros(n, dtype=np.int32)
    info = lib().ptref_band_lu(n, kl, ku, _ptr(ab), ab.shape[0], _ptr(ipiv))
    return ab, ipiv, info


def band_solve(ab: np.ndarray, ipiv: np.ndarray, b: np.ndarray, n: int, kl: int, ku: int):
    b = np.ascontiguousarray(b, dtype=np.float64).copy()
    lib().ptref_band_solve(n, kl, ku, _ptr(ab), ab.shape[0], _ptr(ipiv), _ptr(b))
    return b
