"""Run configuration: the ``pt_config`` struct of include/ptgpu.h as a ctypes mirror.

``PtConfig.from_namelist`` maps the reference's namelist (basics.f90:54-66) onto the struct;
``workload(name)`` builds the five benchmark configurations (grid, Rayleigh numbers, viscosity
law, tracer density) with the reference's shipped solver settings (inputs.nml) where the
configuration does not say otherwise.
"""

from __future__ import annotations

import ctypes
import math

from .namelist import read_namelist

PT_PREC_FP64 = 0
PT_PREC_MIXED = 1
PT_GUESS_PREVIOUS = 0
PT_GUESS_ZERO = 1
PT_GUESS_UNET = 2
PT_GUESS_EXTRAPOLATE = 3
PT_MG_REFERENCE = 0
PT_MG_CORRECTION = 1
PT_CYCLE_REFERENCE = 0
PT_CYCLE_V = 1


class PtConfig(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32),
        ("nz", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("grids", ctypes.c_int32),
        ("mingrid", ctypes.c_int32),
        ("Nmulti", ctypes.c_int32),
        ("vis_iter", ctypes.c_int32),
        ("max_cycles", ctypes.c_int32),
        ("nstageS", ctypes.c_int32),
        ("comp", ctypes.c_int32),
        ("Tbot", ctypes.c_int32),
        ("Vbc", ctypes.c_int32),
        ("ivis", ctypes.c_int32),
        ("iheattype", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("guess_mode", ctypes.c_int32),
        ("ntr", ctypes.c_int64),
        ("aspect", ctypes.c_double),
        ("tolerance", ctypes.c_double),
        ("eig_ratio", ctypes.c_double),
        ("dampingS", ctypes.c_double),
        ("c_2", ctypes.c_double),
        ("c_1", ctypes.c_double),
        ("courant", ctypes.c_double),
        ("courantT", ctypes.c_double),
        ("courantC", ctypes.c_double),
        ("courant_stream", ctypes.c_double),
        ("RaT", ctypes.c_double),
        ("RaC", ctypes.c_double),
        ("H", ctypes.c_double),
        ("Htype", ctypes.c_double),
        ("conduct_factor", ctypes.c_double),
        ("visP", ctypes.c_double),
        ("visT", ctypes.c_double),
        ("delta_visT", ctypes.c_double),
        ("eig_ratio_min", ctypes.c_double),
        ("visC", ctypes.c_double),
        ("delta_visC", ctypes.c_double),
        ("Tbot_iso", ctypes.c_double),
        ("Ttop_iso", ctypes.c_double),
        ("dent", ctypes.c_double),
        ("mg_scheme", ctypes.c_int32),
        ("CFL", ctypes.c_int32),
        ("mg_cycle", ctypes.c_int32),
        ("nstageC", ctypes.c_int32),
        ("discrete_types", ctypes.c_int32),
        ("reference_rounding", ctypes.c_int32),
        ("direct", ctypes.c_int32),
        ("chebyshev", ctypes.c_int32),
        ("nstage", ctypes.c_int32),
        ("damping", ctypes.c_double),
        ("aRK2", ctypes.c_double),
        ("krylov", ctypes.c_int32),
        ("equalize", ctypes.c_int32),
        ("tpc", ctypes.c_int32),
        ("pad2_", ctypes.c_int32),
        ("dist_factor", ctypes.c_double),
        ("Cinit", ctypes.c_double),
        ("eq_seed", ctypes.c_uint64),
    ]

    @staticmethod
    def defaults() -> "PtConfig":
        """Solver settings of the reference's shipped inputs.nml (velocity-solver block)."""
        c = PtConfig()
        c.order = 4
        c.grids = 6
        c.mingrid = 4
        c.Nmulti = 1
        c.vis_iter = 12
        c.max_cycles = 1000
        c.nstageS = 35
        c.comp = 1
        c.Tbot = 0
        c.Vbc = 0
        c.ivis = 0
        c.iheattype = 0
        c.precision = PT_PREC_FP64
        c.guess_mode = PT_GUESS_PREVIOUS
        c.aspect = 1.0
        c.tolerance = 1e-3
        c.eig_ratio = 1.0
        c.dampingS = 1000.0
        c.c_2 = 0.95
        c.c_1 = 0.9
        c.courant = 0.99
        c.courantT = 0.99
        c.courantC = 0.99
        c.courant_stream = 0.99
        c.RaT = 1e5
        c.RaC = 0.0
        c.H = 0.0
        c.Htype = 0.0
        c.conduct_factor = 1.0
        c.visP = 1.0
        c.visT = 1.0
        c.delta_visT = 2.0
        c.eig_ratio_min = 2.0
        c.visC = 1.0
        c.delta_visC = 1.0
        c.Tbot_iso = 1.0
        c.Ttop_iso = 0.0
        c.dent = 0.5
        c.mg_scheme = PT_MG_REFERENCE
        c.nstage = 3
        c.damping = 100.0
        c.aRK2 = 0.5
        c.dist_factor = 1e-4
        c.Cinit = -1.0
        c.eq_seed = 1
        return c

    @staticmethod
    def from_namelist(path: str, ntr: int | None = None) -> "PtConfig":
        return PtConfig.from_groups(read_namelist(path), ntr)

    @staticmethod
    def from_groups(g: dict, ntr: int | None = None) -> "PtConfig":
        c = PtConfig.defaults()
        inp = g.get("inputs", {})
        for key in ("nx", "nz", "order", "grids", "mingrid", "Nmulti", "vis_iter", "max_cycles",
                    "nstageS", "comp", "Tbot", "Vbc", "CFL"):
            if key.lower() in inp:
                setattr(c, key, int(inp[key.lower()]))
        for key in ("nstage", "chebyshev", "equalize", "tpc"):
            if key in inp:
                setattr(c, key, int(inp[key]))
        for key in ("damping", "aRK2", "dist_factor"):
            if key.lower() in inp:
                setattr(c, key, float(inp[key.lower()]))
        for key in ("aspect", "tolerance", "eig_ratio", "dampingS", "c_2", "c_1", "courant",
                    "courantT", "courantC", "courant_stream", "dent"):
            if key.lower() in inp:
                setattr(c, key, float(inp[key.lower()]))
        ray = g.get("rayleigh_numbers", {})
        c.RaT = float(ray.get("rat", c.RaT))
        c.RaC = float(ray.get("rac(1)", c.RaC))
        heat = g.get("heating_conductivity", {})
        c.iheattype = int(heat.get("iheattype", 0))
        c.H = float(heat.get("h", 0.0))
        c.conduct_factor = float(heat.get("conduct_factor(1)", 1.0))
        c.Htype = float(heat.get("htype(1)", 0.0))
        vis = g.get("viscosity", {})
        c.ivis = int(vis.get("ivis", 0))
        for key in ("visP", "visT", "delta_visT", "eig_ratio_min"):
            if key.lower() in vis:
                setattr(c, key, float(vis[key.lower()]))
        c.visC = float(vis.get("visc(1)", 1.0))
        c.delta_visC = float(vis.get("delta_visc(1)", 1.0))
        gpu = g.get("gpu", {})
        c.precision = int(gpu.get("precision", c.precision))
        c.guess_mode = int(gpu.get("guess_mode", c.guess_mode))
        c.discrete_types = 1 if int(inp.get("ic_continuous", 1)) == 0 else 0
        c.direct = 1 if int(inp.get("iterate", 1)) == 0 else 0
        c.mg_scheme = int(gpu.get("mg_scheme", PT_MG_REFERENCE))
        c.mg_cycle = int(gpu.get("mg_cycle", PT_CYCLE_REFERENCE))
        c.krylov = int(gpu.get("krylov", 0))
        tpc = int(inp.get("tpc", 0))
        c.tpc = tpc
        c.ntr = ntr if ntr is not None else (c.nx + 1) * (c.nz + 1) * tpc
        return c

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}

    def copy(self) -> "PtConfig":
        c = PtConfig()
        ctypes.pointer(c)[0] = self
        return c


WORKLOADS = {
    # 128x128, isoviscous, Ra_T=1e5, Ra_C=0, H=0, 20 tracers per cell, Courant 0.5, 100 steps
    # (mixed precision: the 1024x512 method's V-cycle and smoother, GCR with 8 directions around
    # it, which at 1e-8 needs 5.9 instead of 9.3 cycles per solve; the FP64 path keeps the
    # reference's solver)
    "C1": dict(nx=128, nz=128, aspect=1.0, RaT=1e5, RaC=0.0, comp=0, ivis=0, visT=1.0, visP=1.0,
               tpc=20, courant=0.5, tolerance=1e-8, steps=100,
               mg_cycle=PT_CYCLE_V, mixed_nstageS=10, mixed_nstageC=8, mixed_dampingS=30.0,
               mixed_guess=PT_GUESS_EXTRAPOLATE, mixed_krylov=8),
    # 256x128, thermochemical, eta = exp(-ln(1e3) T), 30 tracers per cell, 500 steps.  As at
    # 1024x512, Ra_C=5e5 on the projected composition interface moves tracers out of the domain
    # within two steps of the diffusive time step (CFL=0), so the run uses the reference's
    # velocity-limited step (CFL=1); the reference's 6-level stale-correction cycle diverges on the
    # first solve (oracle), so the run keeps the reference's cycle on 4 levels (grids=4, a
    # namelist option), which converges in 8-12 cycles.
    "C2": dict(nx=256, nz=128, aspect=2.0, RaT=1e6, RaC=5e5, comp=1, ivis=1, visT=1e3, visP=1.0,
               tpc=30, courant=0.5, tolerance=1e-8, steps=500, CFL=1, grids=4,
               mg_cycle=PT_CYCLE_V, mixed_nstageS=10, mixed_nstageC=8, mixed_dampingS=30.0,
               mixed_guess=PT_GUESS_EXTRAPOLATE, mixed_krylov=8),
    # 1024x512, eta = exp(-ln(1e5) T + ln(10)(1-z)), 32 tracers per cell, 200 steps, 1e-8
    # The projected composition interface and Ra_C=2e6 drive velocities of order 1e5 from the
    # first step: the run needs the reference's velocity-limited time step (CFL=1) to keep tracers
    # inside the domain, and the correction-scheme cycle (mg_scheme=1) to converge with 6 levels.
    # 1e-8 is below the FP64 round-off floor of the reference's residual at this size: the
    # plain FP64 solve levels off at 2.0e-8 (first solve) and 1.6e-7 (the RK-stage solves of
    # the first step), a floor set by rounding psi itself to FP64.  Timings therefore use
    # bench_tolerance = 1e-6 for every arm.  The mixed-precision solve runs a V-cycle (mg_cycle):
    # more cycles than the reference's W-type schedule but far less coarse-level work per cycle,
    # and an 8-stage RKC1 smoother (damping 50) instead of 35 stages (damping 1000): 9.0 instead of
    # 7.4 cycles per solve, 27% less time per step (measured on GB300).  The FP64 comparison keeps
    # the reference's smoother.
    "C3": dict(nx=1024, nz=512, aspect=2.0, RaT=1e7, RaC=2e6, comp=1, ivis=1, visT=1e5, visP=10.0,
               tpc=32, courant=0.5, tolerance=1e-8, steps=200, CFL=1, mg_scheme=1, bench_tolerance=1e-6,
               mg_cycle=PT_CYCLE_V, mixed_nstageS=10, mixed_nstageC=8, mixed_dampingS=30.0,
               mixed_guess=PT_GUESS_EXTRAPOLATE),
    # 512x256 learned-guess configuration (Ra_T and contrast sampled per run)
    "C4": dict(nx=512, nz=256, aspect=2.0, RaT=1e6, RaC=2e5, comp=1, ivis=1, visT=1e2, visP=1.0,
               tpc=16, courant=0.5, tolerance=1e-8, steps=1),
    # 2048x1024, Ra_T=1e8, Ra_C=2e7, contrast 1e6, 30 tracers per cell, H=5, 100 steps
    # (timed, like 1024x512, at bench_tolerance with the mixed method's V-cycle settings)
    "C5": dict(nx=2048, nz=1024, aspect=2.0, RaT=1e8, RaC=2e7, comp=1, ivis=1, visT=1e5, visP=10.0,
               tpc=30, courant=0.5, tolerance=1e-8, steps=100, H=5.0, CFL=1, mg_scheme=1, bench_tolerance=1e-6,
               mg_cycle=PT_CYCLE_V, mixed_nstageS=10, mixed_nstageC=8, mixed_dampingS=30.0,
               mixed_guess=PT_GUESS_EXTRAPOLATE),
}


def workload(name: str, scale: float = 1.0, precision: int = PT_PREC_FP64) -> tuple[PtConfig, dict]:
    """Configuration for a named workload; ``scale`` < 1 shrinks the grid by powers of two
    (used for CPU-sized parity cases of the same physics)."""
    w = dict(WORKLOADS[name])
    c = PtConfig.defaults()
    div = 1
    if scale < 1.0:
        div = 2 ** int(round(-math.log2(scale)))
    c.nx = w["nx"] // div
    c.nz = w["nz"] // div
    c.aspect = w["aspect"]
    c.RaT = w["RaT"]
    c.RaC = w["RaC"]
    c.comp = w["comp"]
    c.ivis = w["ivis"]
    c.visT = w["visT"]
    c.visP = w["visP"]
    c.courant = w["courant"]
    c.tolerance = w["tolerance"]
    c.H = w.get("H", 0.0)
    c.CFL = w.get("CFL", 0)
    c.grids = w.get("grids", c.grids)
    c.mg_scheme = w.get("mg_scheme", PT_MG_REFERENCE)
    # schedule, smoother and guess of the mixed-precision method; FP64 keeps the reference's
    c.mg_cycle = w.get("mg_cycle", PT_CYCLE_REFERENCE) if precision == PT_PREC_MIXED else PT_CYCLE_REFERENCE
    if precision == PT_PREC_MIXED and "mixed_nstageS" in w:
        c.nstageS = w["mixed_nstageS"]
        c.nstageC = w.get("mixed_nstageC", 0)
        c.dampingS = w["mixed_dampingS"]
    if precision == PT_PREC_MIXED and "mixed_guess" in w:
        c.guess_mode = w["mixed_guess"]
    if precision == PT_PREC_MIXED:
        c.krylov = w.get("mixed_krylov", 0)
    c.precision = precision
    c.ntr = c.nx * c.nz * w["tpc"]
    c.tpc = w["tpc"]
    return c, w
