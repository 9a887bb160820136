"""Tracer equalisation on the GPU (pt_equalize_tracers; equalize_tracers, composition.f90:266-763)
against the oracle's restatement of the same deterministic algorithm (ptref_equalize):

  * FP64: positions and types of every tracer bit for bit, the moved tracers' temperatures to
    1e-12, the equalize.dat columns, and the projection that follows (counts bit for bit);
  * mixed precision (tracers re-sorted on the device, the fixed-point projection): positions and
    types bit for bit in the caller's order, temperatures to 1e-8;
  * comp=0 (thermal tracers, target tpc);
  * a step with equalize=1 (equalisation first, as energy_time does) to 1e-10 against the oracle.
"""
import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from projectracer_gb300.config import PT_PREC_MIXED
from tests.helpers import rel_err
from tests.test_equalize_oracle import clustered, oracle_for

pytestmark = pytest.mark.gpu


def _compare(cfg, st, t_tol, shuffle=False):
    o = oracle_for(cfg, st)
    e = eng.Engine(cfg)
    e.upload(st)
    gi = e.equalize()
    oi = o.equalize()
    assert gi == oi
    assert gi["moved"] > 0
    assert np.array_equal(e.get(eng.F_TRACER_R), o.get(20))
    assert np.array_equal(e.get(eng.F_TRACER_S), o.get(21))
    if cfg.comp:
        assert np.array_equal(e.get(eng.F_TRACER_TYPE), o.get(24))
    assert rel_err(e.get(eng.F_TRACER_T), o.get(22)) <= t_tol
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    e.close()
    return gi


@pytest.mark.parametrize("kind,frac", [("chem", 0.05), ("chem", 0.01), ("iso", 0.05)])
def test_equalize_fp64_bit_exact(kind, frac):
    cfg, st = clustered(kind, frac=frac)
    _compare(cfg, st, 1e-12)


def test_equalize_mixed_bit_exact_positions():
    cfg, st = clustered("chem")
    cfg.precision = PT_PREC_MIXED
    _compare(cfg, st, 1e-8)


def test_equalize_twice_uses_new_draws():
    cfg, st = clustered("chem")
    o = oracle_for(cfg, st)
    e = eng.Engine(cfg)
    e.upload(st)
    for _ in range(2):
        assert e.equalize() == o.equalize()
        assert np.array_equal(e.get(eng.F_TRACER_R), o.get(20))
    e.close()


def test_step_with_equalize_matches_oracle():
    cfg, st = clustered("chem")
    o = oracle_for(cfg, st)
    e = eng.Engine(cfg)
    e.upload(st)
    e.solve_psi()
    o.solve_psi()
    dt, _ = e.step()
    o.step()
    assert dt == o.scalar("dt")
    for fid, oid in ((eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22)):
        assert rel_err(e.get(fid), o.get(oid)) <= 1e-10, fid
    assert np.array_equal(e.get(eng.F_TRACER_TYPE), o.get(24))
    e.close()


def test_equalize_config_checks():
    cfg, st = clustered("chem")
    cfg.discrete_types = 0
    with pytest.raises(eng.PtError) as ex:
        eng.Engine(cfg)
    assert "equalize" in str(ex.value)


def test_rkc2_step_with_equalize_matches_oracle():
    """The RKC2 stepper equalises first too (Chebyshev.f90:131-137)."""
    cfg, st = clustered("chem")
    cfg.chebyshev, cfg.nstage = 1, 3
    o = oracle_for(cfg, st)
    e = eng.Engine(cfg)
    e.upload(st)
    e.solve_psi()
    o.solve_psi()
    dt, _ = e.step()
    o.step()
    assert dt == o.scalar("dt")
    for fid, oid in ((eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22)):
        assert rel_err(e.get(fid), o.get(oid)) <= 1e-10, fid
    assert np.array_equal(e.get(eng.F_TRACER_TYPE), o.get(24))
    e.close()
