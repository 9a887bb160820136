"""Benchmark: time steps per second of the tracer-convection hot path on GB300.

One "step" is one time step of the reference's loop (main.f90:245-300): the psi solve at the top
of the step (pt_solve_psi) and energy_time (pt_step: RK4 over all tracers with three more psi
solves and four tracer->grid projections).  Inputs are seeded synthetic restart files of the
workload (no dataset is involved); every step works on 1.7 GB of tracer state, far above the
129 MB L2, so no cache flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload C3] [--precision mixed|fp64]
  python bench.py --impl reference ...   (CPU restatement of the reference on the host cores)

Multi-GPU: the path does not shard (no domain decomposition in the reference), so N ranks run N
independent replicas ("replicas only"); value = N * steps / max-over-ranks time.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "timesteps/s @1024x512,16M tracers; \u03c8-solve ms at 1e-8 resid vs plain FP64 GPU"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Host-side barrier / max over ranks (gloo); the data path has no collective."""

    def __init__(self, world: int):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as tdist

            tdist.init_process_group("gloo")
            self.tdist = tdist

    def barrier(self):
        if self.world > 1:
            self.tdist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.tdist.all_reduce(t, op=self.tdist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.tdist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        mhz, maxm, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                mhz.append(float(p[1]))
                maxm = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        mhz.sort()
        med = mhz[len(mhz) // 2] if mhz else None
        return {"sm_mhz": med, "sm_max_mhz": maxm, "reasons": sorted(reasons), "samples": len(mhz)}


def bench_config(workload: str, precision: str):
    from projectracer_gb300.config import PT_PREC_FP64, PT_PREC_MIXED, workload as wl

    prec = PT_PREC_MIXED if precision == "mixed" else PT_PREC_FP64
    cfg, w = wl(workload, 1.0, prec)
    return cfg, w


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def cpu_baseline(workload: str, steps: int = 1) -> dict:
    """The oracle (plain-C restatement of the reference, OpenMP over all host cores) on the
    full-size workload: one untimed psi solve, then `steps` timed steps (psi solve + energy_time),
    each about 20-40 s of CPU work on 8-16 cores."""
    from oracle.ptref import Oracle, build
    from projectracer_gb300.inputs import make_state

    build()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    cfg, w = bench_config(workload, "fp64")
    apply_bench_solver(cfg, w)
    st = make_state(cfg, 3, noise=w.get("noise", 1e-3))
    o = Oracle(cfg, iterate=1, nparts=cores)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    o.solve_psi()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.solve_psi()
        o.step()
    dt = (time.perf_counter() - t0) / steps
    return {"value": 1.0 / dt, "unit": "timesteps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full-size step(s) ({cfg.nx}x{cfg.nz}, {cfg.ntr} tracers, tolerance {cfg.tolerance:g}) "
                      f"after one untimed psi solve: {dt:.2f} s per step",
            "sample_seconds_per_step": dt}


def apply_bench_solver(cfg, w, scale=1.0):
    """Timed tolerance of the workload: the 1024x512 workload's 1e-8 lies below the FP64
    round-off floor of the reference's residual at that size, so every arm runs at
    bench_tolerance.  A reduced-scale sample keeps the coarsest grid of the full-size run."""
    cfg.tolerance = w.get("bench_tolerance", cfg.tolerance)
    if scale < 1.0:
        cfg.grids = max(2, cfg.grids - int(round(-math.log2(scale))))


def run_reference(args, rank: int, world: int):
    """The reference's algorithm on the host cores (the oracle port: no Fortran compiler here),
    same workload, metric and tolerance; at most 3 timed steps so the run stays within minutes."""
    if rank != 0:
        return
    steps = max(1, min(3, args.steps))
    r = cpu_baseline(args.workload, steps=steps)
    value = r["value"]
    cfg, w = bench_config(args.workload, "fp64")
    apply_bench_solver(cfg, w)
    line = {"metric": METRIC, "value": value, "unit": "timesteps/s", "n_gpus": world, "steps": steps,
            "warmup": 1, "ms_per_step": r["sample_seconds_per_step"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{args.workload} {cfg.nx}x{cfg.nz} {cfg.ntr} tracers",
                       "tolerance": cfg.tolerance, "l2_flush": "inputs larger than L2"},
            "cpu_baseline": {"value": value, "unit": "timesteps/s", "cores": r["cores"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": value, "unit": "timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="C3")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="only the headline workload (no error, residual-floor, 1e-8 and per-configuration sections)")
    ap.add_argument("--krylov", type=int, default=-1,
                    help="GCR directions of the mixed solve (default: the workload's setting; 0 = defect correction)")
    ap.add_argument("--tpc", type=int, default=0,
                    help="tracers per cell override (profiling captures of a smaller tracer state only)")
    ap.add_argument("--rows", nargs="*", default=None, choices=list(ROW_NAMES),
                    help="also time the follow-on rows (all, or the ones named) on the GPU with the oracle beside "
                         "them (extended_rows): f-1 file writers, f-2 direct solve, f-3 equalisation, f-4 RKC2 "
                         "stepper, A9 discrete types")
    ap.add_argument("--only-rows", action="store_true", help="with --rows: print only the rows' JSON object")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.only_rows:
        from projectracer_gb300 import engine as eng

        if rank == 0:
            print(json.dumps({"extended_rows": extended_rows(eng, args.rows or list(ROW_NAMES))}), flush=True)
        return
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np

    from projectracer_gb300 import engine as eng
    from projectracer_gb300.inputs import make_state

    dist = Dist(world)
    cfg, w = bench_config(args.workload, args.precision)
    apply_bench_solver(cfg, w)
    if args.tpc > 0:
        cfg.ntr = cfg.nx * cfg.nz * args.tpc
    if args.krylov >= 0 and args.precision == "mixed":
        cfg.krylov = args.krylov
    st = make_state(cfg, 3 + rank, noise=w.get("noise", 1e-3))
    e = eng.Engine(cfg)
    e.upload(st)
    W = max(3, args.warmup)
    for _ in range(W):
        e.solve_psi()
        e.step()
    # timed region: device-resident inputs
    sampler = ClockSampler(local)
    sampler.start()
    e.prof_enable(True)  # live kernel timing: event pairs inside the captured graphs, no extra syncs
    e.prof_reset()
    ph0 = e.phase_times()
    dist.barrier()
    e.region_begin()  # CUDA event on the library's stream (the calls below return synchronised)
    t0 = time.perf_counter()
    cycles, solve_ms, nsolve = 0, 0.0, 0
    for _ in range(args.steps):
        i0 = e.solve_psi()
        dt, i1 = e.step()
        cycles += i0["cycles"] + i1["cycles"]
        solve_ms += i0["ms"] + i1["ms"]
        nsolve += 4
    dev_s = e.region_end() * 1e-3
    host_s = time.perf_counter() - t0
    ph1 = e.phase_times()
    kinds = {kid: e.prof_kernel(kid) for kid in range(4)}
    e.prof_enable(False)
    dist.barrier()
    elapsed = dist.max(dev_s)
    clocks = sampler.stop()
    launches = e.launches()
    grids = int(e.L.pt_grids())
    value = world * args.steps / elapsed
    # end to end through the C ABI with host buffers: per step the driver pushes its tracer
    # arrays (pinned host memory) and reads back the restart records
    e2e = end_to_end(e, eng, cfg, st, max(1, min(3, args.steps)), dist, world)
    roof = roofline(kinds, cfg)
    phase_names = ("tracer_rk_stages", "projections", "psi_solves", "mg_setup", "mg_level1", "mg_coarse_levels",
                   "grid_work", "coarse_factor")
    phases = {nm: (ph1[q] - ph0[q]) / args.steps for q, nm in enumerate(phase_names)}
    # the plain FP64 GPU path from the same state: psi-solve ms at the same tolerance
    fp64 = None
    extra = {}
    if args.precision == "mixed" and not args.no_fp64_compare:
        snap = snapshot(e, eng, st)
        e.close()
        e = None
        fp64 = fp64_comparison(eng, cfg, snap)
        fp64_same = fp64_comparison(eng, cfg, snap, same_schedule=True)
        if not args.quick:
            extra["mixed_error_vs_fp64"] = mixed_error_vs_fp64(eng, cfg, snap)
            extra[f"psi_residual_floor_{cfg.nx}x{cfg.nz}"] = residual_floor(eng, cfg, snap)
        del snap
    if not args.quick and rank == 0:
        if e is not None:
            e.close()
            e = None
        extra["psi_solve_at_1e-8"] = psi_at_1e8(eng)
        extra["per_config"] = per_config(eng)
    if args.rows is not None and rank == 0:
        if e is not None:
            e.close()
            e = None
        extra["extended_rows"] = extended_rows(eng, args.rows or list(ROW_NAMES))
    line = {"metric": METRIC, "value": value, "unit": "timesteps/s", "n_gpus": world, "steps": args.steps,
            "warmup": W, "ms_per_step": elapsed / args.steps * 1e3, "host_ms_per_step": host_s / args.steps * 1e3,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
            "data": "synthetic",
            "config": dict({"workload": f"{args.workload} {cfg.nx}x{cfg.nz} {cfg.ntr} tracers",
                            "precision": args.precision, "replicas": world, "l2_flush": "inputs larger than L2"},
                           **solver_keys(cfg, grids)),
            "psi_solve_ms": solve_ms / max(1, nsolve), "mg_cycles_per_solve": cycles / max(1, nsolve),
            "tracers_per_s": value * cfg.ntr, "gpu_launches": launches, "clocks": clocks, "e2e": e2e,
            "roofline": roof, "phase_ms_per_step": phases}
    if fp64 is not None:
        line["fp64_path"] = fp64
        line["psi_solve_speedup_vs_fp64"] = fp64["psi_solve_ms"] / max(1e-9, line["psi_solve_ms"])
        line["fp64_same_schedule"] = fp64_same
        line["psi_solve_speedup_vs_fp64_same_schedule"] = fp64_same["psi_solve_ms"] / max(1e-9, line["psi_solve_ms"])
    line.update(extra)
    if rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = {k: v for k, v in cpu_baseline(args.workload).items()
                                    if k != "sample_seconds_per_step"}
        except Exception as ex:  # the baseline is reported, not required for the GPU number
            line["cpu_baseline"] = {"value": None, "unit": "timesteps/s", "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"failed: {ex}"}
    if e is not None:
        e.close()
    dist.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


GUESS_NAMES = {0: "previous psi", 1: "zero", 2: "learned", 3: "time-extrapolated"}


def solver_keys(cfg, grids=None) -> dict:
    """The solver settings that define the timed method (the workload text fixes the physics; these
    say where the timed run differs from the reference's shipped settings)."""
    from projectracer_gb300.config import PT_CYCLE_V, PT_MG_CORRECTION, PT_PREC_MIXED

    mixed = cfg.precision == PT_PREC_MIXED
    return {"tolerance": cfg.tolerance, "grids": grids if grids is not None else cfg.grids, "courant": cfg.courant,
            "CFL": cfg.CFL, "mg_scheme": "correction" if cfg.mg_scheme == PT_MG_CORRECTION else "reference",
            "mg_cycle": "V" if (mixed and cfg.mg_cycle == PT_CYCLE_V) else "reference W-type",
            "nstageS": cfg.nstageS, "nstageC": (cfg.nstageC or cfg.nstageS) if mixed else cfg.nstageS,
            "dampingS": cfg.dampingS, "guess": GUESS_NAMES[cfg.guess_mode],
            "coarse_solve": "FP64 explicit inverse of the FP64 banded LU",
            "outer": f"GCR({cfg.krylov}) with the cycle as preconditioner" if (mixed and cfg.krylov > 0)
            else "defect correction (x += cycle correction)"}


def fp64_reference_method(cfg):
    """The plain FP64 GPU path with the reference's solver (W-type schedule, 35-stage RKC1 smoother
    with damping 1000, previous-psi start) on cfg's physics, grid and tolerance."""
    from projectracer_gb300.config import PT_CYCLE_REFERENCE, PT_PREC_FP64, PtConfig

    c = cfg.copy()
    c.precision = PT_PREC_FP64
    c.krylov = 0
    ref = PtConfig.defaults()
    c.nstageS, c.dampingS, c.nstageC = ref.nstageS, ref.dampingS, 0
    c.guess_mode = ref.guess_mode
    c.mg_cycle = PT_CYCLE_REFERENCE
    return c


def _rel(a, b) -> float:
    import numpy as np

    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-300)


def mixed_error_vs_fp64(eng, cfg, snap) -> dict:
    """The mixed path's error against the plain FP64 GPU path from the same state: in each
    precision one psi solve, one step (three more solves, four projections) and the psi solve of
    the next step, at the same tolerance; then the largest difference of each result relative to
    the FP64 field's largest magnitude."""
    out = {}
    for tag, c in (("mixed", cfg.copy()), ("fp64", fp64_reference_method(cfg))):
        e = eng.Engine(c)
        e.upload(snap)
        e.solve_psi()
        dt, _ = e.step()
        info = e.solve_psi()
        out[tag] = {"dt": dt, "resid_ratio": info["resid_ratio"], "stats": e.stats(),
                    "fields": {nm: e.get(fid) for nm, fid in (("psi", eng.F_SF), ("u", eng.F_U), ("w", eng.F_W),
                                                              ("T", eng.F_T), ("C", eng.F_CNEW),
                                                              ("tracer_r", eng.F_TRACER_R),
                                                              ("tracer_s", eng.F_TRACER_S),
                                                              ("tracer_T", eng.F_TRACER_T),
                                                              ("tracer_C", eng.F_TRACER_C))}}
        e.close()
    m, f = out["mixed"], out["fp64"]
    err = {nm: _rel(m["fields"][nm], f["fields"][nm]) for nm in f["fields"]}
    for k in ("Nu", "vrms", "Tavg", "Cavg"):
        err[k] = abs(m["stats"][k] - f["stats"][k]) / max(abs(f["stats"][k]), 1e-300)
    err["dt"] = abs(m["dt"] - f["dt"]) / f["dt"]
    err["nempty_equal"] = bool((m["stats"]["empty_cells"], m["stats"]["tracer_min"], m["stats"]["tracer_max"]) ==
                               (f["stats"]["empty_cells"], f["stats"]["tracer_min"], f["stats"]["tracer_max"]))
    return {"relative_error": err, "tolerance": cfg.tolerance,
            "resid_ratio": {"mixed": m["resid_ratio"], "fp64": f["resid_ratio"]},
            "how": "from the same state: psi solve + one RK4 step + the next psi solve in each precision; "
                   "max |mixed - fp64| / max |fp64| per field (the FP64 path runs the reference's solver)"}


def residual_floor(eng, cfg, snap, cycles: int = 40) -> dict:
    """The lowest relative residual a top-of-step psi solve reaches within `cycles` cycles at a
    tolerance it cannot meet (1e-14), for the FP64 path (reference solver) and the mixed path."""
    out = {}
    for tag, c in (("fp64", fp64_reference_method(cfg)), ("mixed", cfg.copy())):
        c.tolerance, c.max_cycles = 1e-14, cycles
        e = eng.Engine(c)
        e.upload(snap)
        try:
            e.solve_psi()
            status = "converged"
        except eng.PtError as ex:
            status = {-4: "cycle cap", -3: "diverged"}.get(ex.code, str(ex))
        h = e.residuals()
        e.close()
        if not h:
            out[tag] = {"status": status}
            continue
        q = min(range(len(h)), key=lambda j: h[j])
        out[tag] = {"min_resid_ratio": h[q], "at_test": q + 1, "tests": len(h), "last": h[-1], "status": status,
                    "reaches_1e-8": bool(h[q] <= 1e-8)}
    return out


def timed_steps(eng, cfg, st, steps: int, warmup: int) -> dict:
    """Device-timed steps (psi solve + energy_time) of one configuration from a fresh upload (at
    most 100 cycles per solve: a solve that cannot reach the tolerance fails instead of running on)."""
    cfg = cfg.copy()
    cfg.max_cycles = min(cfg.max_cycles, 100)
    e = eng.Engine(cfg)
    e.upload(st)
    for _ in range(warmup):
        e.solve_psi()
        e.step()
    e.region_begin()
    cyc, ms, ns, worst = 0, 0.0, 0, 0.0
    for _ in range(steps):
        i0 = e.solve_psi()
        _, i1 = e.step()
        cyc += i0["cycles"] + i1["cycles"]
        ms += i0["ms"] + i1["ms"]
        ns += 4
        worst = max(worst, i0["resid_ratio"], i1["resid_ratio"])
    el = e.region_end() * 1e-3
    e.close()
    return {"timesteps_per_s": steps / el, "ms_per_step": el / steps * 1e3, "tracers_per_s": steps / el * cfg.ntr,
            "psi_solve_ms": ms / ns, "mg_cycles_per_solve": cyc / ns, "max_resid_ratio": worst, "steps": steps}


def per_config(eng, steps: int = 3) -> dict:
    """Throughput of the other stated configurations on one GPU (device-timed, after 2 warm-up
    steps), each in plain FP64 (the reference's solver) and in mixed precision (C1, C2: GCR around
    the mixed cycle at the configuration's 1e-8); the CPU restatement beside C1 (the configuration
    the CPU can run in full)."""
    from projectracer_gb300.config import PT_PREC_FP64, PT_PREC_MIXED, workload
    from projectracer_gb300.inputs import make_state

    res = {}
    for name, precs in (("C1", (PT_PREC_FP64, PT_PREC_MIXED)), ("C2", (PT_PREC_FP64, PT_PREC_MIXED)),
                        ("C5", (PT_PREC_MIXED, PT_PREC_FP64))):
        cfg0, w = workload(name)
        st = make_state(cfg0, 1, noise=0.0 if name == "C1" else 1e-3)
        entry = {"grid": f"{cfg0.nx}x{cfg0.nz}", "tracers": int(cfg0.ntr)}
        for prec in precs:
            cfg, w = workload(name, 1.0, prec)
            apply_bench_solver(cfg, w)
            if prec == PT_PREC_FP64:
                cfg = fp64_reference_method(cfg)
            tag = "mixed" if prec == PT_PREC_MIXED else "fp64"
            try:
                r = timed_steps(eng, cfg, st, steps if name != "C5" else 2, 2)
                r["config"] = solver_keys(cfg)
            except Exception as ex:  # a configuration that fails is reported, not fatal
                r = {"failed": str(ex)}
            entry[tag] = r
        res[name] = entry
        del st
    try:
        cb = cpu_baseline("C1", steps=3)
        res["C1"]["cpu_baseline"] = {k: v for k, v in cb.items() if k != "sample_seconds_per_step"}
    except Exception as ex:
        res["C1"]["cpu_baseline"] = {"failed": str(ex)}
    return res


def psi_at_1e8(eng, steps: int = 2) -> dict:
    """psi-solve time at the metric's 1e-8 relative residual where the FP64 path reaches it: the
    1024x512 workload's physics on a 512x256 grid (six levels down to 16x8), and the 256x128
    thermochemical workload; plain FP64 (reference solver) against mixed precision from the same
    seeded state, 2 warm-up steps then `steps` timed steps (4 solves each).  The mixed arm runs
    GCR with 8 directions around its cycle (near 1e-8 the plain defect correction slows down);
    the plain mixed cycle is reported beside it."""
    from projectracer_gb300.config import PT_PREC_MIXED, workload
    from projectracer_gb300.inputs import make_state

    res = {}
    for name, scale in (("C3", 0.5), ("C2", 1.0)):
        cfg, w = workload(name, scale, PT_PREC_MIXED)
        cfg.tolerance = 1e-8
        if name == "C3":
            cfg.ntr = cfg.nx * cfg.nz * 8
            cfg.grids = 6
        st = make_state(cfg, 2, noise=1e-3)
        entry = {"grid": f"{cfg.nx}x{cfg.nz}", "tolerance": 1e-8}
        gcr = cfg.copy()
        gcr.krylov = 8
        dc = cfg.copy()
        dc.krylov = 0
        for tag, c in (("fp64", fp64_reference_method(cfg)), ("mixed", gcr), ("mixed_defect_correction", dc)):
            try:
                r = timed_steps(eng, c, st, steps, 2)
                r["reached"] = bool(r["max_resid_ratio"] <= 1e-8)
                r["outer"] = solver_keys(c)["outer"]
                entry[tag] = r
            except Exception as ex:
                entry[tag] = {"failed": str(ex)}
        if "psi_solve_ms" in entry.get("fp64", {}) and "psi_solve_ms" in entry.get("mixed", {}):
            entry["psi_solve_speedup"] = entry["fp64"]["psi_solve_ms"] / entry["mixed"]["psi_solve_ms"]
            entry["step_speedup"] = entry["fp64"]["ms_per_step"] / entry["mixed"]["ms_per_step"]
        res[f"{name} physics {cfg.nx}x{cfg.nz}"] = entry
    return res


ROW_NAMES = ("f-1", "f-2", "f-3", "f-4", "A9")


def extended_rows(eng, which) -> dict:
    """The follow-on rows named in `which` on the GPU, each with the oracle timed beside it on all
    host cores (the file writer against the package's numpy writer of the same records).  GPU
    times are host-timed around calls that return synchronised (the writers: until pt_io_wait
    returns)."""
    import shutil
    import tempfile

    import numpy as np

    from oracle.ptref import Oracle, build
    from projectracer_gb300.config import PT_PREC_FP64, PT_PREC_MIXED, workload
    from projectracer_gb300.inputs import make_state, write_restart

    build()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    clock = time.perf_counter

    def oracle_for(cfg, st, iterate=1, types=None):
        o = Oracle(cfg, iterate=iterate, nparts=cores)
        if types is not None:
            o.set_types(types)
        o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
        return o

    def timed(fn, reps=1):
        t0 = clock()
        for _ in range(reps):
            fn()
        return (clock() - t0) / reps * 1e3

    def one_step(x):
        x.solve_psi()
        x.step()

    def f2():
        """the banded direct psi solve (iterate=0) on the 128x128 isoviscous grid; the first solve
        of a run assembles, equilibrates and factors, later ones substitute"""
        cfg, _ = workload("C1", 1.0, PT_PREC_FP64)
        cfg.direct, cfg.ntr = 1, 128 * 128 * 20
        st = make_state(cfg, 3)
        e = eng.Engine(cfg)
        e.upload(st)
        g_first = timed(e.solve_psi)
        g_solve = timed(e.solve_psi, 5)
        e.close()
        o = oracle_for(cfg, st, iterate=0)
        c_first = timed(o.solve_psi)
        o.step()
        c_solve = timed(o.solve_psi)
        n = (cfg.nx + 1) * (cfg.nz + 1)
        return "f-2 direct banded psi solve", {
            "case": f"128x128 isoviscous, {n} unknowns, band widths {3 * (cfg.nz + 1)}/{3 * (cfg.nz + 1)}",
            "gpu_ms": {"factor_and_solve": g_first, "solve": g_solve},
            "cpu_ms": {"factor_and_solve": c_first, "solve": c_solve}, "cpu_cores": cores,
            "cpu_note": "the oracle's band factorisation and substitutions are serial"}

    def f3():
        """tracer equalisation after 5% of the tracers gathered into a small box (512x512, 20 per
        cell, 5.2M tracers)"""
        cfg, _ = workload("C1", 1.0, PT_PREC_FP64)
        cfg.nx = cfg.nz = 512
        cfg.ntr = 512 * 512 * 20
        cfg.equalize, cfg.tpc = 1, 20
        st = make_state(cfg, 3)
        rng = np.random.default_rng(5)
        idx = rng.choice(cfg.ntr, cfg.ntr // 20, replace=False)
        st["rtr"][idx] = 0.3 + 0.05 * rng.random(len(idx))
        st["str"][idx] = 0.5 + 0.05 * rng.random(len(idx))
        e = eng.Engine(cfg)
        e.upload(st)
        e.equalize()  # first call: allocations
        e.upload(st)
        info = {}
        g_eq = timed(lambda: info.update(e.equalize()))
        e.close()
        o = oracle_for(cfg, st)
        c_eq = timed(o.equalize)
        return "f-3 tracer equalisation", {
            "case": f"512x512, {cfg.ntr} tracers, 5% gathered into a 0.05 x 0.05 box", "moved": int(info.get("moved", 0)),
            "gpu_ms": g_eq, "cpu_ms": c_eq, "cpu_cores": cores, "cpu_note": "the oracle's equalisation is serial"}

    def f4():
        """the RKC2 energy stepper (Chebyshev=1, 3 stages) on the 128x128 isoviscous grid, FP64"""
        cfg, _ = workload("C1", 1.0, PT_PREC_FP64)
        cfg.ntr = 128 * 128 * 20
        cfg.chebyshev, cfg.nstage, cfg.damping, cfg.aRK2 = 1, 3, 100.0, 0.5
        st = make_state(cfg, 3)
        e = eng.Engine(cfg)
        e.upload(st)
        one_step(e)
        g_step = timed(lambda: one_step(e), 3)
        e.close()
        o = oracle_for(cfg, st)
        one_step(o)
        c_step = timed(lambda: one_step(o))
        return "f-4 RKC2 energy stepper", {
            "case": "128x128 isoviscous, 327,680 tracers, nstage 3, tolerance 1e-8", "gpu_ms_per_step": g_step,
            "cpu_ms_per_step": c_step, "cpu_cores": cores}

    def a9():
        """discrete tracer types (projection by type counts) in the FP64 step, 256x128
        thermochemical"""
        cfg, w = workload("C2", 1.0, PT_PREC_FP64)
        cfg.ntr = 256 * 128 * 30
        cfg.discrete_types = 1
        st = make_state(cfg, 3, noise=w.get("noise", 1e-3))
        types = (st["Ctr"] > 0.5).astype(np.int32)
        e = eng.Engine(cfg)
        e.upload(dict(st, Ttype=types))
        one_step(e)
        g_step = timed(lambda: one_step(e), 3)
        e.close()
        o = oracle_for(cfg, st, types=types)
        one_step(o)
        c_step = timed(lambda: one_step(o))
        return "A9 discrete tracer types", {
            "case": "256x128 thermochemical, 983,040 tracers, FP64 step (4 projections)", "gpu_ms_per_step": g_step,
            "cpu_ms_per_step": c_step, "cpu_cores": cores}

    def f1():
        """snapshot (T/P text) and restart (gfortran records) files of the 1024x512 state"""
        cfg, w = workload("C3", 1.0, PT_PREC_MIXED)
        st = make_state(cfg, 3, noise=w.get("noise", 1e-3))
        d1, d2 = tempfile.mkdtemp(), tempfile.mkdtemp()
        try:
            e = eng.Engine(cfg)
            e.upload(st)
            g_snap = timed(lambda: (e.write_snapshot(d1, 0), e.io_wait()))
            g_rst = timed(lambda: (e.write_restart(d1), e.io_wait()))
            e.close()
            sizes = {f: os.path.getsize(os.path.join(d1, f)) for f in sorted(os.listdir(d1))}
            c_rst = timed(lambda: write_restart(d2, st, cfg.comp))
        finally:
            shutil.rmtree(d1, ignore_errors=True)
            shutil.rmtree(d2, ignore_errors=True)
        rst_bytes = sizes.get("Trestart", 0) + sizes.get("restart_tracers", 0)
        return "f-1 snapshot and restart files", {
            "case": f"1024x512, {cfg.ntr} tracers", "bytes": sizes, "gpu_ms": {"snapshot": g_snap, "restart": g_rst},
            "gpu_restart_gbs": rst_bytes / (g_rst * 1e-3) / 1e9, "cpu_ms": {"restart_numpy_writer": c_rst},
            "cpu_note": "the package's numpy writer of the same restart records from host arrays "
                        "(no Fortran compiler here for the reference's own writer)"}

    rows = {"f-1": f1, "f-2": f2, "f-3": f3, "f-4": f4, "A9": a9}
    out = {}
    for name in ROW_NAMES:
        if name in which:
            key, val = rows[name]()
            out[key] = val
    return out


def snapshot(e, eng, st) -> dict:
    """Current restart state of the engine (grid T, C, psi and the tracer arrays)."""
    snap = dict(st)
    for key, fid in (("T", eng.F_T), ("Cnew", eng.F_CNEW), ("SF", eng.F_SF), ("rtr", eng.F_TRACER_R),
                     ("str", eng.F_TRACER_S), ("Ctr", eng.F_TRACER_C), ("Ttr", eng.F_TRACER_T)):
        snap[key] = e.get(fid)
    return snap


def fp64_comparison(eng, cfg, snap, steps: int = 2, same_schedule: bool = False) -> dict:
    """The plain FP64 GPU path from the mixed run's state at the same tolerance: one untimed step,
    then `steps` timed steps.  Default: the reference's algorithm (its W-type schedule, 35-stage
    RKC1 smoother, previous-psi start).  same_schedule: FP64 with the mixed run's schedule,
    smoother and initial guess, so that only the precision differs."""
    from projectracer_gb300.config import PT_CYCLE_REFERENCE, PT_PREC_FP64, PtConfig

    c = cfg.copy()
    c.precision = PT_PREC_FP64
    c.krylov = 0  # the FP64 path is the plain cycle
    if not same_schedule:
        ref = PtConfig.defaults()  # the reference's smoother (35 stages, damping 1000), warm start
        c.nstageS, c.dampingS = ref.nstageS, ref.dampingS
        c.guess_mode = ref.guess_mode
        c.mg_cycle = PT_CYCLE_REFERENCE
    e = eng.Engine(c)
    e.upload(snap)
    e.solve_psi()
    e.step()
    t0 = time.perf_counter()
    cycles, solve_ms, nsolve = 0, 0.0, 0
    for _ in range(steps):
        i0 = e.solve_psi()
        _, i1 = e.step()
        cycles += i0["cycles"] + i1["cycles"]
        solve_ms += i0["ms"] + i1["ms"]
        nsolve += 4
    el = time.perf_counter() - t0
    e.close()
    return {"timesteps_per_s": steps / el, "ms_per_step": el / steps * 1e3, "psi_solve_ms": solve_ms / nsolve,
            "mg_cycles_per_solve": cycles / nsolve, "steps": steps, "tolerance": c.tolerance,
            "schedule": "V-cycle" if c.mg_cycle else "reference W-type", "rkc_stages": c.nstageS,
            "guess": {0: "previous psi", 1: "zero", 2: "learned", 3: "time-extrapolated"}[c.guess_mode]}


def end_to_end(e, eng, cfg, st, steps, dist, world):
    import numpy as np

    try:
        import torch

        def pinned(a):
            return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    except Exception:  # pinned buffers are an optimisation of the host side only
        def pinned(a):
            return np.ascontiguousarray(a)
    n = int(cfg.ntr)
    h_r, h_s, h_T, h_C = (pinned(np.empty(n)) for _ in range(4))
    h_r[:] = e.get(eng.F_TRACER_R)
    h_s[:] = e.get(eng.F_TRACER_S)
    h_T[:] = e.get(eng.F_TRACER_T)
    h_C[:] = e.get(eng.F_TRACER_C)
    lx, hx, lz, hz, _ = e.extent(eng.F_T)
    grid_T = pinned(np.empty((hz - lz + 1, hx - lx + 1)))
    grid_S = pinned(np.empty_like(grid_T))
    lx, hx, lz, hz, _ = e.extent(eng.F_CNEW)
    grid_C = pinned(np.empty((hz - lz + 1, hx - lx + 1)))
    ptr = lambda a: a.ctypes.data_as(__import__("ctypes").c_void_p)  # noqa: E731
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        for fid, a in ((eng.F_TRACER_R, h_r), (eng.F_TRACER_S, h_s), (eng.F_TRACER_T, h_T), (eng.F_TRACER_C, h_C)):
            e._check(e.L.pt_set_field(fid, ptr(a)))
        e.solve_psi()
        e.step()
        e._check(e.L.pt_download_state(ptr(grid_T), ptr(grid_C), ptr(grid_S), ptr(h_r), ptr(h_s), ptr(h_C), ptr(h_T), None))
    dist.barrier()
    el = dist.max(time.perf_counter() - t0)
    h2d = 4 * n * 8
    d2h = 4 * n * 8 + (grid_T.size + grid_S.size + grid_C.size) * 8
    return {"value": world * steps / el, "unit": "timesteps/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": steps,
            "note": "per step: tracer arrays host->device through pt_set_field, pt_solve_psi + pt_step, "
                    "restart records device->host through pt_download_state"}


KERNEL_NAMES = {0: "RKC1 stage, FP64, finest level", 1: "RKC1 stage, FP32, finest level",
                2: "RK4 tracer stage (3 interpolations + update)", 3: "tracer->grid projection"}


def algorithmic_bytes(kid: int, cfg) -> float:
    """Bytes a launch must move at minimum (each array touched once):
    FP64 stage: S_j-1 stencil, S_j-2, S_0, dtst, rhs, 5 coefficient fields, out = 11 x 8 B per node;
    FP32 stage (increment form): D_j-1 stencil, D_j-2, F0, dtst, 5 coefficient fields, out = 10 x 4 B
    per node (+4 B for Y0 on the last stage, not counted);
    RK tracer stage, FP64 path: 2 stage positions, 3 step-start values, 3 accumulators read +
    written, 3 next positions written = 14 x 8 B per tracer, + the derivative tables, 12 x 8 B per
    node; mixed path: the positions, step-start values and results in FP64, the 3 slope sums in
    FP32 (read + written in stages 2-3, one way in stages 1 and 4): 82 B per tracer averaged over
    the four stages, + the FP32 tables, 3 x 16 B per node;
    projection: position pair + T (+C) per tracer, and the per-node sums: 32 B per tracer + 28 B
    per node."""
    nx, nz = cfg.nx, cfg.nz
    interior = (nx - 1) * (nz - 1)
    nodes = (nx + 1) * (nz + 1)
    n = float(cfg.ntr)
    from projectracer_gb300.config import PT_PREC_MIXED

    mixed = cfg.precision == PT_PREC_MIXED
    rk = 82.0 * n + 48.0 * nodes if mixed else 112.0 * n + 96.0 * nodes
    return {0: 88.0 * interior, 1: 40.0 * interior, 2: rk, 3: 32.0 * n + 28.0 * nodes}[kid]


# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu capture of
# each kernel class on the 1024x512 grid (the commands, tracer counts and figures are in the
# profiles/ summaries named here).  Grid kernels are captured at full size; the tracer
# kernels' traffic grows with the tracer count and is scaled by it.  Cold-cache figures: ncu
# flushes the caches before each pass, so for the L2-resident stage kernel this is an upper bound.
NCU_TRAFFIC = {
    1: ("per launch", 17.09e6, "profiles/k_rkc_stage_f2_C3_1024x512.md"),
    2: ("per tracer", 109.9e6 / 2097152, "profiles/k_rk_stage_f_C3_1024x512.md"),
    3: ("per tracer", (554.03e6 + 16.40e6) / 16777216, "profiles/k_project_fx_C3_1024x512.md"),
}


def ncu_traffic(kid: int, cfg):
    """(bytes per launch, source) for kernel class kid at this workload, or (None, None)."""
    if kid not in NCU_TRAFFIC or cfg.nx != 1024 or cfg.nz != 512:
        return None, None
    kind, v, src = NCU_TRAFFIC[kid]
    return (v if kind == "per launch" else v * float(cfg.ntr)), src


def roofline(kinds: dict, cfg) -> dict | None:
    """Roofline of the kernel class with the largest share of the timed region, from the live
    event timings (launch-averaged), and the same figures for every timed kernel class."""
    peaks = measured_peaks()
    from projectracer_gb300.config import PT_PREC_MIXED

    per_kernel = {}
    for k, (c, ms) in kinds.items():
        if not c:
            continue
        avg_s = ms / c * 1e-3
        per = algorithmic_bytes(k, cfg)
        achieved = per / avg_s / 1e9
        traffic, src = ncu_traffic(k, cfg) if cfg.precision == PT_PREC_MIXED else (None, None)  # mixed-path kernels
        per_kernel[k] = {"launches": c, "total_ms": ms, "avg_ms": avg_s * 1e3, "algorithmic_bytes_per_launch": per,
                         "achieved_gbs": achieved, "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                         "traffic_source": src}
    if not per_kernel:
        return None
    kid = max(per_kernel, key=lambda k: per_kernel[k]["total_ms"])
    d = per_kernel[kid]
    return {"bound": "hbm", "kernel": KERNEL_NAMES[kid], "achieved": d["achieved_gbs"], "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": d["frac"], "peak_source": peaks["source"] + " (burst copy)",
            "traffic": d["traffic"], "traffic_source": d["traffic_source"],
            "algorithmic_bytes_per_launch": d["algorithmic_bytes_per_launch"], "avg_launch_ms": d["avg_ms"],
            "timed_kernels": {KERNEL_NAMES[k]: v for k, v in per_kernel.items()}}


if __name__ == "__main__":
    main()
