"""Pins the CPU oracle to the reference's own shipped run (tests/golden, made by make_golden.py).

The shipped run (100x100, 612,060 tracers, direct banded psi solve, 2 OpenMP threads) printed
known-answer values to stdout and the t=0 statistics row to stats.dat.  Reproducing that row
needs the restated start-up (initial T, mzran tracer seeding split over 2 threads), the
projection, the direct solve with LAPACK-style band LU, velocities and stats.
"""
import numpy as np
import pytest

from oracle.ptref import Oracle
from projectracer_gb300.config import PtConfig


@pytest.fixture(scope="module")
def golden_run(golden):
    cfg = PtConfig.from_groups(golden["namelist"])
    cfg.iheattype = 0  # interior H is never evaluated before the first stats row
    o = Oracle(cfg, iterate=0, nparts=golden["stdout"]["Nthreads"])
    inp = golden["namelist"]["inputs"]
    o.init_reference(int(inp["tpc"]), golden["stdout"]["Nthreads"], float(inp["klayer"]),
                     float(inp["dlayer"]), 1)
    o.solve_psi()
    return o, o.stats()


def test_known_answers(golden, golden_run):
    o, _ = golden_run
    kat = golden["stdout"]
    assert o.scalar("RKC1_stability") == pytest.approx(kat["RKC1_stability"], rel=1e-15)
    assert o.scalar("Tbot_iso") == kat["Tbot_iso"]
    assert o.scalar("Ttop_iso") == kat["Ttop_iso"]
    assert int(o.scalar("subD")) == kat["subD"] and int(o.scalar("supD")) == kat["supD"]
    assert o.cfg.ntr == kat["ntr"]
    assert int(o.scalar("kent")) == kat["kent"]
    assert o.scalar("delta_T") == kat["T_smoothing"] and o.scalar("delta_C") == kat["C_smoothing"]


def test_stats_row_t0(golden, golden_run):
    _, st = golden_run
    ref = golden["stats"][0]
    # integer columns: bit-exact tracer counts of the projection
    for k in ("empty_cells", "tracer_min", "tracer_max"):
        assert st[k] == ref[k], k
    # columns that depend only on T, the projection and the tracer seeding: printed digits
    for k in ("time", "Tavg", "Nu", "Nu_bot", "RaT_avg", "q1", "q2", "q3", "q4", "Cavg", "entrainment"):
        assert st[k] == pytest.approx(ref[k], rel=2e-14, abs=1e-15), k
    # columns through the direct psi solve (condition ~1e8): LAPACK-implementation rounding
    for k in ("vrms", "mobility", "strain_max"):
        assert st[k] == pytest.approx(ref[k], rel=1e-10), k


def test_snapshot_t0_fields(golden_run):
    import os
    o, _ = golden_run
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "T10000_subset.npz"))
    i, k, cols = d["i"], d["k"], d["cols"]
    fields = {2: o.get(0)[k + 3, i + 3], 3: o.get(7)[k + 3, i + 3], 4: o.get(8)[k + 3, i + 3],
              5: o.get(9)[k + 3, i + 3], 9: o.get(11)[k, i], 10: o.get(4)[k + 5, i + 5]}
    for col, mine in fields.items():
        ref = cols[:, col]
        # 5 significant digits printed (g14.5E3)
        assert np.all(np.abs(mine - ref) <= 5.01e-5 * np.abs(ref) + 1e-300), col


def test_lateral_profile_t0(golden, golden_run):
    o, _ = golden_run
    T = o.get(0)
    nx = o.nx
    dr = o.cfg.aspect / nx
    prof = np.array(golden["P10000_z_Tlat"])
    for kk, (z, tlat) in enumerate(prof):
        row = T[kk + 3, 3:nx + 4]
        fint = 0.0
        for ii in range(nx):
            fint = fint + 0.5 * (row[ii] * 1.0 + row[ii + 1] * 1.0) * dr
        assert fint / o.cfg.aspect == pytest.approx(tlat, rel=5.01e-5, abs=1e-300)
