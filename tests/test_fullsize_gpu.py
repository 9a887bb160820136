"""The 1024x512 workload at full size (16,777,216 tracers, 32 per cell) on the GPU.  The oracle
needs minutes per step at this size, so these tests check properties that hold at any size:
  * the integer projection does not depend on the tracer order: a shuffled upload gives the same
    grid T, C and per-node counts bit for bit, and the counts add up to the number of tracers;
  * it agrees with the FP64 path's sorted projection to its 2^-28 fixed-point resolution, with
    identical counts;
  * a mixed-precision solve and step is deterministic (fixed-order reductions, integer sums):
    two runs from the same state give the same bits;
  * one mixed-precision solve and step agrees with one plain FP64 solve and step from the same
    state to the solve tolerance, and both conserve the tracers and keep them in the domain.
"""
import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from projectracer_gb300.config import PT_PREC_FP64, PT_PREC_MIXED, workload
from projectracer_gb300.inputs import make_state

pytestmark = pytest.mark.gpu


def _cfg(precision):
    cfg, w = workload("C3", 1.0, precision)
    cfg.tolerance = w.get("bench_tolerance", cfg.tolerance)
    return cfg, w


@pytest.fixture(scope="module")
def state():
    cfg, w = _cfg(PT_PREC_MIXED)
    return make_state(cfg, 3, noise=w.get("noise", 1e-3))


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _upload(cfg, st, fields):
    e = eng.Engine(cfg)
    e.upload(st)
    out = {f: e.get(f) for f in fields}
    e.close()
    return out


def test_fullsize_projection_order_independent_and_conserving(state):
    cfg, _ = _cfg(PT_PREC_MIXED)
    n = len(state["rtr"])
    assert n == cfg.ntr == 16777216
    fields = (eng.F_T, eng.F_TRATIO, eng.F_CNEW, eng.F_NEMPTY)
    a = _upload(cfg, state, fields)
    p = np.random.default_rng(7).permutation(n)
    shuffled = dict(state)
    for f in ("rtr", "str", "Ttr", "Ctr"):
        shuffled[f] = state[f][p]
    b = _upload(cfg, shuffled, fields)
    for f in fields:
        assert np.array_equal(a[f], b[f]), f
    assert int(a[eng.F_NEMPTY].sum()) == n
    # the FP64 path's sorted projection: the same counts, the same fields to 2^-28
    c64, _ = _cfg(PT_PREC_FP64)
    c = _upload(c64, state, fields)
    assert np.array_equal(a[eng.F_NEMPTY], c[eng.F_NEMPTY])
    for f in (eng.F_T, eng.F_TRATIO, eng.F_CNEW):
        assert rel(a[f], c[f]) < 1e-7, f


def _solve_step(cfg, st):
    e = eng.Engine(cfg)
    e.upload(st)
    i0 = e.solve_psi()
    dt, i1 = e.step()
    out = {f: e.get(f) for f in (eng.F_SF, eng.F_T, eng.F_CNEW, eng.F_NEMPTY, eng.F_TRACER_R, eng.F_TRACER_S,
                                 eng.F_TRACER_T, eng.F_TRACER_C)}
    out["dt"] = dt
    out["resid"] = max(i0["resid_ratio"], i1["resid_ratio"])
    e.close()
    return out


def test_fullsize_mixed_step_deterministic_and_close_to_fp64(state):
    cfg, _ = _cfg(PT_PREC_MIXED)
    a = _solve_step(cfg, state)
    b = _solve_step(cfg, state)
    for k in a:
        if k != "dt" and k != "resid":
            assert np.array_equal(a[k], b[k]), k
    assert a["dt"] == b["dt"]
    assert a["resid"] <= cfg.tolerance
    c64, _ = _cfg(PT_PREC_FP64)
    f = _solve_step(c64, state)
    assert f["resid"] <= c64.tolerance
    n = cfg.ntr
    for out in (a, f):
        assert int(out[eng.F_NEMPTY].sum()) == n
        r, s = out[eng.F_TRACER_R], out[eng.F_TRACER_S]
        assert np.all((r >= 0) & (r <= cfg.aspect) & (s >= 0) & (s <= 1))
    # both solves stop at a relative residual of at most 1e-6: their psi agree to about that
    assert abs(a["dt"] - f["dt"]) <= 1e-5 * f["dt"]
    assert rel(a[eng.F_SF], f[eng.F_SF]) < 1e-4
    for k in (eng.F_TRACER_R, eng.F_TRACER_S):
        assert rel(a[k], f[k]) < 1e-7, k
    assert rel(a[eng.F_TRACER_T], f[eng.F_TRACER_T]) < 1e-6
    assert rel(a[eng.F_T], f[eng.F_T]) < 1e-6
    assert np.array_equal(a[eng.F_TRACER_C], f[eng.F_TRACER_C])
