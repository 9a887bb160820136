"""The GCR-accelerated mixed-precision solve (pt_config.krylov > 0): the mixed cycle as the
preconditioner of a flexible GCR iteration, same convergence test as the plain mixed solve.

  * the solution agrees with the plain FP64 solve to the solve tolerance, like the plain mixed
    solve, and needs no more cycles than it;
  * a full step agrees with the FP64 step as closely as the plain mixed step does;
  * restarts (krylov smaller than the iterations a solve needs) still converge;
  * it is deterministic (fixed-order reductions): two runs give the same bits;
  * krylov is rejected outside 0..8 and with FP64 precision.
"""
import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from projectracer_gb300.config import PT_CYCLE_V, PT_GUESS_EXTRAPOLATE, PT_PREC_FP64, PT_PREC_MIXED
from tests.helpers import small_case

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _case(krylov, tol=1e-8, nx=128, nz=64):
    cfg, st = small_case("c3", nx=nx, nz=nz)
    cfg.tolerance = tol
    cfg.precision = PT_PREC_MIXED
    cfg.mg_cycle = PT_CYCLE_V
    cfg.nstageS, cfg.nstageC, cfg.dampingS = 10, 8, 30.0
    cfg.krylov = krylov
    return cfg, st


def _solve(cfg, st):
    e = eng.Engine(cfg)
    e.upload(st)
    info = e.solve_psi()
    sf = e.get(eng.F_SF)
    e.close()
    return info, sf


def test_gcr_solve_matches_fp64_in_fewer_cycles():
    cfg, st = _case(0)
    c64 = cfg.copy()
    c64.precision, c64.krylov, c64.mg_cycle = PT_PREC_FP64, 0, 0
    _, sf64 = _solve(c64, st)
    i0, sf0 = _solve(cfg, st)
    cfg.krylov = 6
    i6, sf6 = _solve(cfg, st)
    for info in (i0, i6):
        assert info["resid_ratio"] <= cfg.tolerance
    assert rel_err(sf6, sf64) < 1e-6
    assert rel_err(sf6, sf0) < 1e-6
    assert i6["cycles"] <= i0["cycles"]


def test_gcr_with_restarts_converges():
    cfg, st = _case(2)
    info, sf = _solve(cfg, st)
    assert info["resid_ratio"] <= cfg.tolerance
    cfg.krylov = 8
    _, sf8 = _solve(cfg, st)
    assert rel_err(sf, sf8) < 1e-6


def test_gcr_is_deterministic():
    cfg, st = _case(6)
    _, a = _solve(cfg, st)
    _, b = _solve(cfg, st)
    assert np.array_equal(a, b)


def test_gcr_step_close_to_fp64():
    cfg, st = _case(6, tol=1e-8)
    cfg.guess_mode = PT_GUESS_EXTRAPOLATE
    out = {}
    for prec in (PT_PREC_FP64, PT_PREC_MIXED):
        c = cfg.copy()
        c.precision = prec
        if prec == PT_PREC_FP64:
            c.krylov, c.mg_cycle = 0, 0
        e = eng.Engine(c)
        e.upload(st)
        for _ in range(2):
            e.solve_psi()
            dt, info = e.step()
        assert info["resid_ratio"] <= cfg.tolerance
        out[prec] = {f: e.get(f) for f in (eng.F_TRACER_R, eng.F_TRACER_S, eng.F_TRACER_T, eng.F_T)}
        out[prec]["dt"] = dt
        e.close()
    a, b = out[PT_PREC_FP64], out[PT_PREC_MIXED]
    assert abs(a["dt"] - b["dt"]) <= 1e-6 * a["dt"]
    for f in (eng.F_TRACER_R, eng.F_TRACER_S):
        assert rel_err(b[f], a[f]) < 1e-7, f
    assert rel_err(b[eng.F_TRACER_T], a[eng.F_TRACER_T]) < 1e-6
    assert rel_err(b[eng.F_T], a[eng.F_T]) < 1e-6


@pytest.mark.parametrize("krylov,prec", [(9, PT_PREC_MIXED), (-1, PT_PREC_MIXED), (4, PT_PREC_FP64)])
def test_gcr_config_checks(krylov, prec):
    cfg, _ = _case(0, nx=64, nz=32)
    cfg.krylov = krylov
    cfg.precision = prec
    with pytest.raises(eng.PtError) as ex:
        eng.Engine(cfg)
    assert "krylov" in str(ex.value)
