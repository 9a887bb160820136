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


def _g14_5e3(x: float) -> str:
    """Fortran g14.5E3 as gfortran prints it (F form for 0.1 <= |x| < 1e5, else E form)."""
    if x == 0.0:
        return "%9.4f     " % x  # '-0.0000' for a negative zero
    k = int(("%.4e" % x).split("e")[1]) + 1
    if 0 <= k <= 5:
        return "%9.*f     " % (5 - k, x)
    m = "%.4e" % abs(x)
    return "%14s" % ("%s0.%s%sE%s%03d" % ("-" if x < 0 else "", m[0], m[2:6], "-" if k < 0 else "+", abs(k)))


def test_snapshot_t0_text(golden_run):
    """The sampled lines of the shipped T10000 as printed, every column but the stress one: T, psi
    (with the sign of its zeros: -0 on the non-corner wall nodes), u, w, vis, Tvis, nempty, Cnew,
    Cvis."""
    import json
    import os
    o, _ = golden_run
    with open(os.path.join(os.path.dirname(__file__), "golden", "snapshot_t0_lines.json")) as fh:
        ref = json.load(fh)["T10000"]
    nz = o.cfg.nz
    f3 = [o.get(q) for q in (0, 7, 8, 9, 10, 2)]
    ne, C, Cv = o.get(11), o.get(4), o.get(5)
    checked = 0
    for n, line in ref:
        i, k = divmod(n, nz + 2)
        if k > nz:
            continue
        cols = [line[14 * j:14 * (j + 1)] for j in (2, 3, 4, 5, 7, 8)]
        assert [_g14_5e3(f[k + 3, i + 3]) for f in f3] == cols, n
        assert "%6d" % ne[k, i] == line[126:132], n
        assert _g14_5e3(C[k + 5, i + 5]) + _g14_5e3(Cv[k + 5, i + 5]) == line[132:160], n
        checked += 1
    assert checked > 250
