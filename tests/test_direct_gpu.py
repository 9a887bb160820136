"""The direct banded psi solve on the GPU (iterate=0, the reference's shipped default:
build_SF_matrix / solve_SF_equation, momentum.f90:319-653) against the reference's own shipped run
and against the oracle's restatement, through the C ABI.

The shipped run is 100x100 with 612,060 tracers: n = 10,201 unknowns, band widths 303/303.  The GPU
assembles the same matrix, equilibrates its rows and factors it with the unblocked band LU in the
reference's operation order (no fused multiply-adds), then solves with the banded substitutions.
So psi follows the oracle's to its last bits (within 1e-13 relative), and the t=0 statistics
through the solve (v_rms, mobility, strain_max) match stats.dat to 1e-10, as the oracle does
(tests/test_oracle_golden.py); that bound is the LAPACK implementation's rounding at a condition
number of about 1e8.
"""
import numpy as np
import pytest

from oracle.ptref import Oracle
from projectracer_gb300 import engine as eng
from tests.helpers import golden_t0, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def direct_t0(golden):
    cfg, st, start, o = golden_t0(golden, direct=1)
    e = eng.Engine(cfg)
    e.upload(st)
    for f, v in start.items():
        e.set(f, v)
    info = e.solve_psi()
    out = {"stats": e.stats(), "info": info,
           "fields": {f: e.get(f) for f in (eng.F_SF, eng.F_U, eng.F_W)}}
    e.close()
    o.solve_psi()
    out["oracle"] = {7: o.get(7), 8: o.get(8), 9: o.get(9), "stats": o.stats()}
    return cfg, out


def test_direct_config_is_the_shipped_solver(direct_t0):
    cfg, _ = direct_t0
    assert cfg.direct == 1 and cfg.nx == 100 and cfg.ivis == 0


def test_direct_psi_matches_oracle(direct_t0):
    _, out = direct_t0
    for fid, oid in ((eng.F_SF, 7), (eng.F_U, 8), (eng.F_W, 9)):
        assert rel_err(out["fields"][fid], out["oracle"][oid]) < 1e-13, fid


def test_direct_stats_t0_match_the_shipped_run(golden, direct_t0):
    _, out = direct_t0
    st, ref = out["stats"], golden["stats"][0]
    for k in ("vrms", "mobility", "strain_max"):
        assert st[k] == pytest.approx(ref[k], rel=1e-10), k
    for k in ("Tavg", "Nu", "Nu_bot", "RaT_avg", "q1", "q2", "q3", "q4", "Cavg", "entrainment"):
        assert st[k] == pytest.approx(ref[k], rel=2e-14, abs=1e-15), k
    for k in ("empty_cells", "tracer_min", "tracer_max"):
        assert st[k] == ref[k], k


def test_direct_steps_match_oracle(golden):
    """Two RK4 steps with the direct solve from the restart state (the factorisation is built once
    and reused, as in the reference): dt, tracers, T and psi against the oracle's direct path."""
    cfg, st, _, _ = golden_t0(golden, direct=1)
    o = Oracle(cfg, iterate=0, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    e = eng.Engine(cfg)
    e.upload(st)
    for _ in range(2):
        e.solve_psi()
        o.solve_psi()
        dt, _ = e.step()
        o.step()
        assert dt == o.scalar("dt")
    e.solve_psi()
    o.solve_psi()
    for fid, oid in ((eng.F_SF, 7), (eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22), (eng.F_T, 0)):
        assert rel_err(e.get(fid), o.get(oid)) < 1e-10, fid
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    e.close()


def test_direct_rejects_variable_viscosity(golden):
    cfg, st, _, _ = golden_t0(golden, direct=1)
    cfg.ivis = 1
    with pytest.raises(eng.PtError) as ex:
        eng.Engine(cfg)
    assert ex.value.code == -1


@pytest.mark.parametrize("nx,nz", [(128, 128), (152, 152), (256, 128)])
def test_direct_solve_matches_oracle_on_larger_grids(nx, nz):
    """The substitution kernel keeps b in global memory and the band window the column steps
    touch in shared memory, so the grid is bounded by the band width only: psi bit-identical to
    the oracle's direct solve up to 256x128, the size the survey of the reference rates the direct
    path feasible at (33,153 unknowns, band 387/387)."""
    from projectracer_gb300.config import PT_PREC_FP64, workload
    from projectracer_gb300.inputs import make_state

    cfg, _ = workload("C1", 1.0, PT_PREC_FP64)
    cfg.nx, cfg.nz, cfg.aspect = nx, nz, nx / nz
    cfg.direct, cfg.ntr = 1, nx * nz * 4
    st = make_state(cfg, 3)
    e = eng.Engine(cfg)
    e.upload(st)
    e.solve_psi()
    e.solve_psi()  # the second solve substitutes with the factors of the first
    sf = e.get(eng.F_SF)
    e.close()
    o = Oracle(cfg, iterate=0, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    o.solve_psi()
    assert np.array_equal(sf.view(np.int64), o.get(7).view(np.int64))
