"""The plain FP64 GPU path against the oracle on the full-size stated configurations, over many
steps, through the C ABI.

  C1  128x128, isoviscous, Ra_T = 1e5, 20 tracers per cell (327,680), Courant 0.5: all 100 steps
  C2  256x128, thermochemical, eta = exp(-ln(1e3) T), Ra_T = 1e6, Ra_C = 5e5, 30 tracers per cell
      (983,040), velocity-limited time step, the reference's cycle on 4 levels: 20 steps

Both sides start from the same seeded restart state and run the same sequence as the reference's
time loop (main.f90:245-300): psi solve, stats, energy_time.  The engine runs its FP64 path with
reference_rounding = 1 (the reference's FP64 stencil operations in its order, no fused
multiply-adds, banded substitution on the coarsest grid).  Required: the time step equal every
step (within 1e-10 when it is velocity-limited), integer tracer counts bit-exact, and T, C, psi,
the tracers, Nu and v_rms within 1e-10 relative to each field's largest magnitude after the last
step.

The default FP64 path forms the stencil sums exactly in integer arithmetic: it differs from the
reference's FP64 rounding, and hence from the oracle, by a fraction of the solve tolerance (about
1e-9 relative in psi at 128x128 and 256x128 after one solve, residual tolerance 1e-8); the last
test bounds that difference.
"""
import numpy as np
import pytest

from oracle.ptref import Oracle
from projectracer_gb300 import engine as eng
from projectracer_gb300.config import workload
from projectracer_gb300.inputs import make_state

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-300)


@pytest.mark.parametrize("name,steps", [("C1", 100), ("C2", 20)])
def test_config_fp64_matches_oracle_over_steps(name, steps):
    cfg, w = workload(name)
    cfg.reference_rounding = 1
    st = make_state(cfg, 1, noise=0.0 if name == "C1" else 1e-3)
    assert cfg.ntr == cfg.nx * cfg.nz * w["tpc"]
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    e = eng.Engine(cfg)
    e.upload(st)
    worst = 0.0
    for n in range(steps):
        ie = e.solve_psi()
        o.solve_psi()
        assert ie["cycles"] == int(o.scalar("cycles")), n
        if n % 10 == 0:
            se, so = e.stats(), o.stats()
            for k in ("empty_cells", "tracer_min", "tracer_max"):
                assert se[k] == so[k], (n, k)
            for k in ("Nu", "vrms", "Tavg"):
                worst = max(worst, abs(se[k] - so[k]) / abs(so[k]))
        dt, _ = e.step()
        o.step()
        if cfg.CFL:  # velocity-limited: dt carries the velocity's rounding
            assert abs(dt - o.scalar("dt")) <= TOL * o.scalar("dt"), n
        else:
            assert dt == o.scalar("dt"), n
    e.solve_psi()
    o.solve_psi()
    se, so = e.stats(), o.stats()
    for k in ("empty_cells", "tracer_min", "tracer_max"):
        assert se[k] == so[k], k
    for k in ("Nu", "vrms", "Tavg", "Nu_bot") + (("Cavg", "entrainment") if cfg.comp else ()):
        assert se[k] == pytest.approx(so[k], rel=TOL), k
    assert worst < TOL
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    for fid, oid in ((eng.F_T, 0), (eng.F_SF, 7), (eng.F_U, 8), (eng.F_W, 9), (eng.F_TRACER_R, 20),
                     (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22)):
        assert rel(e.get(fid), o.get(oid)) < TOL, fid
    if cfg.comp:
        assert rel(e.get(eng.F_CNEW), o.get(4)) < TOL
    t_e, _ = e.time()
    assert t_e == pytest.approx(o.scalar("time"), rel=1e-15)
    e.close()


def test_fp64_rounding_modes_agree_to_the_solve_tolerance():
    """The default FP64 path (exact stencil sums) against reference_rounding = 1 on C2 over two
    steps: psi and the velocities within 10 x the residual tolerance, the tracers and T far
    closer (they integrate the velocities over one step), counts equal."""
    cfg, w = workload("C2")
    cfg.ntr = cfg.nx * cfg.nz * 4
    st = make_state(cfg, 1, noise=1e-3)
    out = []
    for rounding in (0, 1):
        c = cfg.copy()
        c.reference_rounding = rounding
        e = eng.Engine(c)
        e.upload(st)
        for _ in range(2):
            e.solve_psi()
            e.step()
        e.solve_psi()
        out.append({f: e.get(f) for f in (eng.F_SF, eng.F_U, eng.F_W, eng.F_T, eng.F_TRACER_R, eng.F_NEMPTY)})
        e.close()
    a, b = out
    for f in (eng.F_SF, eng.F_U, eng.F_W):
        assert rel(a[f], b[f]) < 10 * cfg.tolerance, f
    for f in (eng.F_T, eng.F_TRACER_R):
        assert rel(a[f], b[f]) < 1e-10, f
    assert np.array_equal(a[eng.F_NEMPTY], b[eng.F_NEMPTY])
