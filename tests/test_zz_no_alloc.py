"""pt_tracers_to_corners_noalloc, the projection for drivers that cannot allocate device memory
(their pool owns the GPU, or cudaMalloc would stall other streams), against pt_tracers_to_corners
on the same engine and tracer state, in both precisions: two consecutive calls of each give
bit-identical T, C and tracer counts (FP64: the sorted sums; mixed precision: the integer
fixed-point sums, which reuse the same static scratch as their accumulator); states above the
static scratch limits are rejected.  Collected last (file name) so that it also runs after the
rest of the suite has used the device."""
import ctypes

import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from tests.helpers import small_case

pytestmark = pytest.mark.gpu


def _fields(e):
    return [e.get(f) for f in (eng.F_TRATIO, eng.F_CNEW, eng.F_NEMPTY, eng.F_T)]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_noalloc_projection_matches_existing_entry_point(precision):
    cfg, st = small_case("chem")
    cfg.precision = precision
    e = eng.Engine(cfg)
    e.upload(st)
    e.solve_psi()
    e.step()  # tracers off their initial positions
    L = e.L
    L.pt_tracers_to_corners_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int]
    T0 = e.get(eng.F_T)
    ref = []
    for _ in range(2):
        e._check(L.pt_tracers_to_corners(T0.ctypes.data_as(ctypes.c_void_p), 1))
        ref.append(_fields(e))
    got = []
    for _ in range(2):
        e._check(L.pt_tracers_to_corners_noalloc(T0.ctypes.data_as(ctypes.c_void_p), 1))
        got.append(_fields(e))
    for a, b in zip(ref, got):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    e.close()


def test_noalloc_projection_rejects_oversize():
    cfg, st = small_case("iso", nx=256, nz=256, tpc=2)  # 66049 nodes > PT_NOALLOC_MAX_NODES
    e = eng.Engine(cfg)
    e.upload(st)
    L = e.L
    L.pt_tracers_to_corners_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int]
    rc = L.pt_tracers_to_corners_noalloc(None, 1)
    assert rc == -9  # PT_ERR_ARG
    assert b"PT_NOALLOC" in L.pt_last_error() or b"tracers or" in L.pt_last_error()
    e.close()
