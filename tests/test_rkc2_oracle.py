"""The RKC2 Chebyshev energy stepper (Chebyshev=1, energy_time_Chebyshev, Chebyshev.f90:113-243) in
the oracle, on the CPU: at the same time step it integrates the same tracer equations as the RK4
stepper (energy_time), so after the same number of steps the two agree closely, and more closely
at half the time step.  (RKC2 takes its step from the RK2 stability bound, 2/eigD against RK4's
2.8/eigD, so a Courant number 1.4 times larger gives both the same dt.)"""
import numpy as np

from oracle.ptref import Oracle
from tests.helpers import small_case


def _run(cfg, st, cheb, courant, steps):
    c = cfg.copy()
    c.chebyshev, c.nstage, c.damping, c.aRK2 = cheb, 3, 100.0, 0.5
    c.courant = courant * (1.4 if cheb else 1.0)
    o = Oracle(c, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    for _ in range(steps):
        o.solve_psi()
        o.step()
    return o.scalar("time"), o.get(20), o.get(22)


def test_rkc2_and_rk4_integrate_the_same_equations():
    cfg, st = small_case("iso", nx=32, nz=32, tpc=4)
    diffs = []
    for courant, steps in ((0.05, 4), (0.025, 8)):
        t4, r4, T4 = _run(cfg, st, 0, courant, steps)
        t2, r2, T2 = _run(cfg, st, 1, courant, steps)
        assert t2 == np.float64(t4) or abs(t2 - t4) <= 1e-15 * t4
        disp = np.abs(r4 - st["rtr"]).max()
        assert disp > 1e-4  # the tracers moved
        dr = np.abs(r2 - r4).max()
        assert dr < 1e-3 * disp
        diffs.append(np.abs(T2 - T4).max())
    assert diffs[0] < 1e-4
    assert diffs[1] < 0.6 * diffs[0]
