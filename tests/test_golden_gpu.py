"""The GPU engine against the reference's own shipped run, through the C ABI.

The shipped run (100x100, 612,060 tracers, 2 OpenMP threads) wrote its t=0 statistics row to
stats.dat (basics.f90:427-428) and its t=0 snapshot to T10000 (main.f90:396-397); both are
fixtures in tests/golden.  The t=0 state is rebuilt by the oracle's restatement of the start-up
(initial T, mzran tracer seeding split over 2 threads, composition.f90:776-858), pinned by
tests/test_oracle_golden.py, and uploaded into the engine as a restart (pt_upload_state): the
engine projects the tracers itself (counts, Cnew).  The reference's fresh start-up builds T_vis
and T_buoy differently from its restart read (main.f90:168-230 against grid.f90:93-95 with
main.f90:204-210), so the start-up's T, T_vis, T_buoy, C_vis and C_buoy are then set through
pt_set_field, as a driver that starts fresh would.  The engine then solves for psi and computes
the velocities and the statistics.

These cases solve for psi by multigrid; tests/test_direct_gpu.py runs the shipped run's own direct
banded solve.  The grid spacing 0.01 is not a power of two, so these cases run the general branches of the
projection and the RK stage (cell index by llround(x/h), the FP64 division in the shape
functions, floor(x/h) in the fixed-point projection) that the power-of-two test grids skip.

Tolerances:
  * tracer counts and every column that depends only on T, the projection and the stats sums:
    bit-exact counts, 2e-14 relative (stats.dat prints 15 digits);
  * the columns through the psi solve (v_rms, mobility, strain_max): the reference used the
    direct banded solve, the engine multigrid to a relative residual of 1e-12; the two agree to
    1e-9 (the oracle's multigrid at the same tolerance is 2.5e-10 from the printed values);
  * T10000 columns: the 5 printed digits.
"""
import os

import numpy as np
import pytest

from oracle.ptref import Oracle
from projectracer_gb300 import engine as eng
from projectracer_gb300.config import PT_PREC_MIXED
from tests.helpers import golden_t0

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden_state(golden):
    cfg, st, start, _ = golden_t0(golden, direct=0)
    return cfg, st, start


@pytest.fixture(scope="module")
def engine_t0(golden_state):
    cfg, st, start = golden_state
    e = eng.Engine(cfg)
    e.upload(st)
    projected = {f: e.get(f) for f in (eng.F_NEMPTY, eng.F_TRATIO, eng.F_CNEW, eng.F_TVIS)}
    for f, v in start.items():
        e.set(f, v)
    before = e.stats()
    info = e.solve_psi()
    after = e.stats()
    fields = {f: e.get(f) for f in (eng.F_T, eng.F_SF, eng.F_U, eng.F_W, eng.F_NEMPTY, eng.F_CNEW)}
    e.close()
    return before, after, info, fields, projected


def test_golden_state_is_the_shipped_run(golden, golden_state):
    cfg, st, _ = golden_state
    assert cfg.nx == 100 and cfg.nz == 100 and len(st["rtr"]) == golden["stdout"]["ntr"] == 612060
    assert cfg.aspect / cfg.nx == 0.01


def test_stats_t0_without_psi(golden, engine_t0):
    """Columns that need no psi solve, straight after the restart upload."""
    st = engine_t0[0]
    ref = golden["stats"][0]
    for k in ("empty_cells", "tracer_min", "tracer_max"):
        assert st[k] == ref[k], k
    for k in ("time", "Tavg", "Nu", "Nu_bot", "q1", "q2", "q3", "q4", "Cavg", "entrainment"):
        assert st[k] == pytest.approx(ref[k], rel=2e-14, abs=1e-15), k


def test_stats_t0_through_psi_solve(golden, engine_t0):
    _, st, info, _, _ = engine_t0
    ref = golden["stats"][0]
    assert info["resid_ratio"] <= 1e-12
    for k in ("vrms", "mobility", "strain_max"):
        assert st[k] == pytest.approx(ref[k], rel=1e-9), k
    assert st["RaT_avg"] == pytest.approx(ref["RaT_avg"], rel=2e-14)  # needs the viscosity of the solve
    for k in ("empty_cells", "tracer_min", "tracer_max"):
        assert st[k] == ref[k], k


def test_snapshot_t0_fields(engine_t0):
    """T10000 (x, z, T, SF, u, w, stress, vis, Tvis, nempty, Cnew, Cvis; 5 printed digits)."""
    f = engine_t0[3]
    d = np.load(os.path.join(HERE, "golden", "T10000_subset.npz"))
    i, k, cols = d["i"], d["k"], d["cols"]
    mine = {2: f[eng.F_T][k + 3, i + 3], 3: f[eng.F_SF][k + 3, i + 3], 4: f[eng.F_U][k + 3, i + 3],
            5: f[eng.F_W][k + 3, i + 3], 9: f[eng.F_NEMPTY][k, i], 10: f[eng.F_CNEW][k + 5, i + 5]}
    assert np.array_equal(mine[9], cols[:, 9].astype(np.int32))
    for col, v in mine.items():
        ref = cols[:, col]
        assert np.all(np.abs(v - ref) <= 5.01e-5 * np.abs(ref) + 1e-300), col


def test_projection_bit_exact_at_non_power_of_two_spacing(golden_state, engine_t0):
    """The FP64 projection of the shipped run's tracers (dr = ds = 0.01) against the oracle in
    the engine's canonical summation order: counts, Tratio, Cnew and the smoothed Tvis bit for
    bit."""
    cfg, st, _ = golden_state
    f = engine_t0[4]  # straight after the upload's projection and smoothing
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    assert np.array_equal(f[eng.F_NEMPTY], o.get(11))
    assert np.array_equal(f[eng.F_TRATIO][1:-1, 1:-1], o.get(1)[1:-1, 1:-1])
    assert np.array_equal(f[eng.F_CNEW], o.get(4))
    assert np.array_equal(f[eng.F_TVIS][1:-1, 1:-1], o.get(2)[1:-1, 1:-1])


def test_mixed_projection_at_non_power_of_two_spacing(golden_state):
    """The fixed-point projection's general branch (cell and fraction from floor(x / h)) against
    its integer restatement, bit for bit, on the shipped run's tracers."""
    from oracle.project_fx import project_fx, ratios

    cfg, st, _ = golden_state
    c = cfg.copy()
    c.precision = PT_PREC_MIXED
    e = eng.Engine(c)
    e.upload(st)
    TS, CS, S, cnt = project_fx(c.nx, c.nz, c.aspect, st["rtr"], st["str"], st["Ttr"], st["Ctr"])
    assert np.array_equal(e.get(eng.F_NEMPTY), cnt)
    Tg = e.get(eng.F_TRATIO)[3:-3, 3:-3]
    Cg = e.get(eng.F_CNEW)[5:-5, 5:-5]
    Tr, Cr = ratios(TS, CS, S, Tg, Cg)
    assert np.array_equal(Tg[1:-1, 1:-1], Tr[1:-1, 1:-1])
    assert np.array_equal(Cg[1:-1, 1:-1], Cr[1:-1, 1:-1])
    e.close()


def test_step_at_non_power_of_two_spacing(golden_state):
    """One RK4 step from the shipped run's t=0 state (isoviscous, multigrid at 1e-12), engine
    against oracle: dt, tracers and T to 1e-10, counts bit-exact."""
    cfg, st, _ = golden_state
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    e = eng.Engine(cfg)
    e.upload(st)
    i0 = e.solve_psi()
    o.solve_psi()
    assert i0["cycles"] == int(o.scalar("cycles"))
    dt, _ = e.step()
    o.step()
    assert dt == o.scalar("dt")
    for fid, oid in ((eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22)):
        a, b = e.get(fid), o.get(oid)
        assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b)), fid
    a, b = e.get(eng.F_T), o.get(0)
    assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b))
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    e.close()
