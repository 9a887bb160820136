"""Failure detection, injected on the host: each case feeds the engine an input that the reference
would stop on (or, for the coarse LU, silently mis-solve), and checks that the C ABI returns the
status code and message that replace the reference's `write` + `stop`, in both precisions.  After
each failure a fresh pt_init on the same process runs a normal solve, so the context stays usable.

  tracer pushed outside the domain   PT_ERR_TRACER_OUT_OF_DOMAIN   composition.f90:1007-1010
  NaN in the buoyancy temperature     PT_ERR_NOT_FINITE             (no check in the reference)
  cycle cap below what the solve needs PT_ERR_MG_MAX_CYCLES         iterative_solver.f90:325-334
  viscosity that vanishes everywhere  PT_ERR_SINGULAR_COARSE        DGBTRF INFO>0 (unchecked there)

No case faults or hangs the GPU: out-of-domain tracers are clamped for the interpolation reads
and skipped by the projection, NaN only flows through arithmetic (no index depends on it), the
viscosity smoother's loops are bounded, and the band LU's pivot search stays inside the band for
zero and NaN columns.
"""
import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from projectracer_gb300.config import PT_PREC_FP64, PT_PREC_MIXED
from tests.helpers import small_case

pytestmark = pytest.mark.gpu

PRECISIONS = pytest.mark.parametrize("precision", [PT_PREC_FP64, PT_PREC_MIXED], ids=["fp64", "mixed"])


def _engine(precision, **kw):
    cfg, st = small_case("chem", **kw)
    cfg.precision = precision
    e = eng.Engine(cfg)
    e.upload(st)
    return cfg, st, e


def _still_usable(cfg, st):
    """A fresh context after the failure solves and steps normally."""
    e = eng.Engine(cfg)
    e.upload(st)
    info = e.solve_psi()
    assert info["resid_ratio"] <= cfg.tolerance
    e.step()
    assert np.all(np.isfinite(e.get(eng.F_TRACER_R)))
    e.close()


@PRECISIONS
def test_tracer_outside_domain_in_projection(precision):
    cfg, st, e = _engine(precision)
    r = e.get(eng.F_TRACER_R)
    r[1234] = 1.5 * cfg.aspect
    e.set(eng.F_TRACER_R, r)
    with pytest.raises(eng.PtError) as ex:
        e.project()
    assert ex.value.code == -2
    assert b"outside of domain" in e.L.pt_last_error()
    e.close()
    _still_usable(cfg, st)


@PRECISIONS
def test_tracer_outside_domain_during_step(precision):
    """A tracer below the bottom wall: the RK stage interpolates at a clamped node, and the stage-2
    projection reports it, as the reference's projection stops on it."""
    cfg, st, e = _engine(precision)
    e.solve_psi()
    s = e.get(eng.F_TRACER_S)
    s[77] = -0.25
    e.set(eng.F_TRACER_S, s)
    with pytest.raises(eng.PtError) as ex:
        e.step()
    assert ex.value.code == -2
    e.close()
    _still_usable(cfg, st)


@PRECISIONS
def test_nan_buoyancy_is_reported(precision):
    cfg, st, e = _engine(precision)
    tb = e.get(eng.F_TBUOY)
    tb[10, 20] = np.nan
    e.set(eng.F_TBUOY, tb)
    with pytest.raises(eng.PtError) as ex:
        e.solve_psi()
    assert ex.value.code == -10
    assert b"non-finite" in e.L.pt_last_error()
    e.close()
    _still_usable(cfg, st)


@PRECISIONS
def test_cycle_cap(precision):
    cfg, st = small_case("chem")
    cfg.precision = precision
    cfg.max_cycles = 1
    cfg.tolerance = 1e-13
    e = eng.Engine(cfg)
    e.upload(st)
    with pytest.raises(eng.PtError) as ex:
        e.solve_psi()
    assert ex.value.code == -4
    msg = e.L.pt_last_error().lower()
    assert b"cycles" in msg
    hist = e.residuals()  # kept after the failure: how far the solve got
    assert 1 <= len(hist) <= 3 and all(np.isfinite(hist)) and hist[-1] > cfg.tolerance
    e.close()
    cfg.max_cycles, cfg.tolerance = 1000, 1e-8
    _still_usable(cfg, st)


@PRECISIONS
def test_vanishing_viscosity_is_a_singular_coarse_operator(precision):
    """T_vis = 1000 makes eta = exp(-1000 ln 1e3) underflow to 0 everywhere: every interior row of
    the coarse banded operator is zero, which the equilibration step reports (DGBTRF would return
    INFO > 0; the reference does not check it)."""
    cfg, st, e = _engine(precision)
    tv = e.get(eng.F_TVIS)
    tv[:, :] = 1000.0
    e.set(eng.F_TVIS, tv)
    with pytest.raises(eng.PtError) as ex:
        e.solve_psi()
    assert ex.value.code == -5
    assert b"coarse banded LU" in e.L.pt_last_error()
    e.close()
    _still_usable(cfg, st)


def test_calls_out_of_order():
    """pt_step before pt_upload_state is refused without touching the device state."""
    cfg, st = small_case("chem")
    e = eng.Engine(cfg)
    with pytest.raises(eng.PtError) as ex:
        e.step()
    assert ex.value.code == -7
    e.upload(st)
    e.solve_psi()
    e.close()
