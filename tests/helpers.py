"""Shared set-up for parity tests: one configuration, one seeded state, oracle and engine."""
from __future__ import annotations

import numpy as np

from projectracer_gb300.config import PtConfig, workload
from projectracer_gb300.inputs import make_state


def small_case(kind: str = "iso", nx: int = 64, nz: int = 64, tpc: int = 8, seed: int = 3) -> tuple[PtConfig, dict]:
    """CPU-sized parity cases on the hot path's code branches.
    iso:   isoviscous thermal convection (comp=0, ivis=0), the C1 physics
    chem:  thermochemical, eta(T), composition layer (comp=1, ivis=1), C2-like at lower Ra
    depth: eta(T,z) with internal heating (ivis=1, visP>1, H>0), C3/C5-like at lower Ra
    c3:    the 1024x512 workload's physics (Ra_T=1e7, Ra_C=2e6, eta contrast 1e5 x depth 10) on a
           small grid, with velocity-limited time steps (CFL=1) and the correction-scheme cycle
    """
    if kind == "iso":
        c, _ = workload("C1")
        c.nx, c.nz = nx, nz
    elif kind == "chem":
        c, _ = workload("C2")
        c.nx, c.nz = nx, nz
        c.RaT, c.RaC, c.visT = 1e5, 5e4, 1e3
        c.courant = 0.1
        c.CFL, c.grids = 0, 6  # diffusive time step and the reference's level count at this low Ra
    elif kind == "depth":
        c, _ = workload("C3")
        c.nx, c.nz = nx, nz
        c.RaT, c.RaC, c.visT, c.visP, c.H = 1e5, 2e4, 1e3, 10.0, 1.0
        c.courant = 0.05
        c.CFL = 0
        c.mg_scheme = 0
    elif kind == "c3":
        from projectracer_gb300.config import PT_MG_CORRECTION

        c, _ = workload("C3")
        c.nx, c.nz = nx, nz
        c.grids = 4
        c.CFL = 1
        c.courant = 0.5
        c.mg_scheme = PT_MG_CORRECTION
        c.mg_cycle = 0  # the reference's schedule in both precisions (parity cases)
    else:
        raise ValueError(kind)
    c.ntr = nx * nz * tpc
    st = make_state(c, seed, noise=1e-3 if kind != "iso" else 0.0)
    return c, st


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


def walls(cfg, st):
    """A copy of st with a few tracers on the walls and corners (x = 0 or aspect, z = 0 or 1)."""
    st = dict(st)
    r, s = st["rtr"].copy(), st["str"].copy()
    r[:4], s[:4] = [0.0, cfg.aspect, 0.0, cfg.aspect], [0.0, 1.0, 1.0, 0.0]
    r[-3:], s[-2:] = cfg.aspect, 1.0
    st["rtr"], st["str"] = r, s
    return st


def golden_t0(golden: dict, direct: int = 0):
    """The reference's shipped run (100x100, 612,060 tracers) at t=0, rebuilt by the oracle's
    restatement of its start-up: (cfg, restart arrays, start-up fields by field id, oracle).
    direct=1 keeps the run's own psi solver (iterate=0, the banded direct solve); direct=0 uses
    multigrid at a relative residual of 1e-12."""
    from oracle.ptref import Oracle
    from projectracer_gb300 import engine as eng
    from projectracer_gb300.inputs import grid_coords

    cfg = PtConfig.from_groups(golden["namelist"])
    cfg.iheattype = 0  # interior H is never evaluated before the first stats row
    cfg.direct = direct
    cfg.tolerance = 1e-12
    inp = golden["namelist"]["inputs"]
    o = Oracle(cfg, iterate=0 if direct else 1, nparts=golden["stdout"]["Nthreads"])
    o.init_reference(int(inp["tpc"]), golden["stdout"]["Nthreads"], float(inp["klayer"]), float(inp["dlayer"]), 1)
    cfg.Tbot_iso, cfg.Ttop_iso = o.scalar("Tbot_iso"), o.scalar("Ttop_iso")  # set by initial_temperature
    xg, zg = grid_coords(cfg)
    st = dict(xg=xg, zg=zg, T=o.get(0), Cnew=o.get(4), SF=o.get(7), rtr=o.get(20), str=o.get(21), Ttr=o.get(22),
              Ctr=o.get(23))
    start = {eng.F_T: o.get(0), eng.F_TVIS: o.get(2), eng.F_TBUOY: o.get(3), eng.F_CVIS: o.get(5),
             eng.F_CBUOY: o.get(6)}
    return cfg, st, start, o
