"""Why the 1024x512 and 256x128 workloads do not run the reference's multigrid cycle unchanged,
shown on the CPU with the oracle (no GPU).

The reference never resets the coarse corrections error(:,:,2:grids) between cycles (zeroed once,
main.f90:229), so every coarse visit starts from the previous cycle's correction.  At the
1024x512 workload's physics (Ra_T = 1e7, Ra_C = 2e6, viscosity contrast 1e5 in T and 10 in depth)
that stale-correction cycle on 6 levels diverges on the first solve at 256x128 and stops with the
reference's "Abnormally High Residual" (iterative_solver.f90:438-447), and so does the 256x128
thermochemical workload on 6 levels.  The correction scheme (each descent from zero;
PT_MG_CORRECTION) converges on the same states, and so does the reference's own cycle on 4 levels.
"""
import pytest

from oracle.ptref import Oracle
from projectracer_gb300.config import PT_MG_CORRECTION, PT_MG_REFERENCE, workload
from projectracer_gb300.inputs import make_state
from tests.helpers import small_case


def _oracle(cfg, st):
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    return o


def test_stale_correction_diverges_at_workload_physics():
    cfg, st = small_case("c3", nx=256, nz=128, tpc=4)
    cfg.grids = 6
    cfg.max_cycles = 60  # bounded: the failure comes as the divergence stop or the cycle cap
    cfg.mg_scheme = PT_MG_REFERENCE
    with pytest.raises(RuntimeError, match="oracle error -(3|4)"):
        _oracle(cfg, st).solve_psi()
    cfg.mg_scheme = PT_MG_CORRECTION
    o = _oracle(cfg, st)
    o.solve_psi()
    assert o.scalar("resid_ratio") <= cfg.tolerance
    assert o.scalar("cycles") <= 30


def test_thermochemical_workload_levels():
    cfg, w = workload("C2")
    cfg.ntr = cfg.nx * cfg.nz * 4  # the solve does not depend on the tracer density
    st = make_state(cfg, 1, noise=1e-3)
    assert cfg.grids == 4 and cfg.mg_scheme == PT_MG_REFERENCE and cfg.CFL == 1
    o = _oracle(cfg, st)
    o.solve_psi()
    assert o.scalar("resid_ratio") <= cfg.tolerance and o.scalar("cycles") <= 20
    cfg.grids = 6
    cfg.max_cycles = 60
    with pytest.raises(RuntimeError, match="oracle error -(3|4)"):
        _oracle(cfg, st).solve_psi()
