"""The RKC2 Chebyshev energy stepper on the GPU (Chebyshev=1: energy_time_Chebyshev,
Chebyshev.f90:113-243, the shipped run's nstage=3, damping=100, aRK2=0.5) against the oracle's
restatement through the C ABI: the RK2 time step, and after three steps the tracers, T, C and psi
to 1e-10 with tracer counts bit-exact, in the FP64 path with the reference's rounding."""
import numpy as np
import pytest

from oracle.ptref import Oracle
from projectracer_gb300 import engine as eng
from projectracer_gb300.config import PT_PREC_MIXED
from tests.helpers import rel_err, small_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["iso", "chem"])
def test_rkc2_steps_match_oracle(kind):
    cfg, st = small_case(kind)
    cfg.chebyshev, cfg.nstage, cfg.damping, cfg.aRK2 = 1, 3, 100.0, 0.5
    cfg.reference_rounding = 1
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    e = eng.Engine(cfg)
    e.upload(st)
    for n in range(3):
        i0 = e.solve_psi()
        o.solve_psi()
        assert i0["cycles"] == int(o.scalar("cycles")), n
        dt, info = e.step()
        o.step()
        assert dt == o.scalar("dt"), n
    for fid, oid in ((eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22), (eng.F_T, 0), (eng.F_SF, 7)):
        assert rel_err(e.get(fid), o.get(oid)) < 1e-10, fid
    if cfg.comp:
        assert rel_err(e.get(eng.F_CNEW), o.get(4)) < 1e-10
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    assert e.time()[0] == pytest.approx(o.scalar("time"), rel=1e-15)
    e.close()


def test_rkc2_is_fp64_only():
    cfg, _ = small_case("iso")
    cfg.chebyshev = 1
    cfg.precision = PT_PREC_MIXED
    with pytest.raises(eng.PtError) as ex:
        eng.Engine(cfg)
    assert ex.value.code == -1
