"""GPU engine vs the CPU oracle on identical seeded inputs, through the C ABI.

Integer work (cell indices, tracer counts) and the projection / boundary-condition / smoother
kernels are compared bit for bit (the oracle runs the projection in the engine's canonical
summation order).  Floating-point results that pass through the FMA-contracted kernels (psi
solve, tracer interpolation) are compared at the required tolerance of 1e-10 relative to the
field's maximum (per single solve / step, typically 1e-13).
"""
import numpy as np
import pytest

from oracle.ptref import Oracle
from projectracer_gb300 import engine as eng
from tests.helpers import rel_err, small_case, walls

pytestmark = pytest.mark.gpu

TOL = 1e-10


def pair(kind, **kw):
    cfg, st = small_case(kind, **kw)
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    e = eng.Engine(cfg)
    e.upload(st)
    return cfg, o, e


# (kind, nx, nz): the power-of-two grids of the physics cases, and 96x48 (spacing 1/48, not a power
# of two: the general branches of the cell index, the shape functions and the multigrid constants)
GRIDS = [("iso", 64, 64), ("chem", 64, 64), ("depth", 64, 64), ("chem", 96, 48), ("depth", 96, 48)]
GRID_IDS = [f"{k}-{nx}x{nz}" for k, nx, nz in GRIDS]


@pytest.mark.parametrize("kind,nx,nz", GRIDS, ids=GRID_IDS)
def test_upload_projection_bit_exact(kind, nx, nz):
    cfg, o, e = pair(kind, nx=nx, nz=nz)
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    for fid in (eng.F_TRATIO, eng.F_TVIS, eng.F_TBUOY, eng.F_T):
        g, r = e.get(fid), o.get(fid)
        assert np.array_equal(g[1:-1, 1:-1] if fid != eng.F_T else g, r[1:-1, 1:-1] if fid != eng.F_T else r), fid
    if cfg.comp:
        assert np.array_equal(e.get(eng.F_CNEW), o.get(4))
    e.close()


@pytest.mark.parametrize("kind,nx,nz", [("iso", 64, 64), ("chem", 64, 64), ("c3", 64, 64), ("chem", 96, 48)],
                         ids=["iso", "chem", "c3", "chem-96x48"])
def test_mixed_projection_bit_exact(kind, nx, nz):
    """The one-pass fixed-point projection of the mixed-precision path equals its integer
    restatement bit for bit (counts, Tratio and Cnew on every node with tracers), tracers on the
    walls and corners included."""
    from oracle.project_fx import project_fx, ratios
    from projectracer_gb300.config import PT_PREC_MIXED

    cfg, st = small_case(kind, nx=nx, nz=nz)
    st = walls(cfg, st)
    cfg.precision = PT_PREC_MIXED
    e = eng.Engine(cfg)
    e.upload(st)
    TS, CS, S, cnt = project_fx(cfg.nx, cfg.nz, cfg.aspect, st["rtr"], st["str"], st["Ttr"],
                                st["Ctr"] if cfg.comp else None)
    assert np.array_equal(e.get(eng.F_NEMPTY), cnt)
    Tg = e.get(eng.F_TRATIO)[3:-3, 3:-3]
    Cg = e.get(eng.F_CNEW)[5:-5, 5:-5] if cfg.comp else None
    Tr, Cr = ratios(TS, CS, S, Tg, Cg)
    # interior nodes (the wall nodes take boundary values afterwards)
    assert np.array_equal(Tg[1:-1, 1:-1], Tr[1:-1, 1:-1])
    if cfg.comp:
        assert np.array_equal(Cg[1:-1, 1:-1], Cr[1:-1, 1:-1])
    e.close()


def test_mixed_projection_independent_of_tracer_order():
    """Integer sums: permuting the tracers leaves the mixed-precision projection bit-identical."""
    from projectracer_gb300.config import PT_PREC_MIXED

    cfg, st = small_case("chem")
    cfg.precision = PT_PREC_MIXED
    perm = np.random.default_rng(7).permutation(len(st["rtr"]))
    st2 = dict(st)
    for f in ("rtr", "str", "Ctr", "Ttr"):
        st2[f] = st[f][perm]
    out = []
    for state in (st, st2):
        e = eng.Engine(cfg)
        e.upload(state)
        out.append([e.get(f) for f in (eng.F_NEMPTY, eng.F_TRATIO, eng.F_CNEW, eng.F_T)])
        e.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_mixed_steps_independent_of_tracer_order():
    """Mixed precision re-sorts its tracers by cell when the order loses locality.  The caller
    still sees its own order: three steps from a shuffled upload give, after un-shuffling, the
    same tracers and grid fields bit for bit as from the seeding order; set/get of a tracer field
    after the re-sort round-trips in the caller's order."""
    from projectracer_gb300.config import PT_PREC_MIXED

    cfg, st = small_case("chem")
    cfg.precision = PT_PREC_MIXED
    perm = np.random.default_rng(11).permutation(len(st["rtr"]))
    st2 = dict(st)
    for f in ("rtr", "str", "Ctr", "Ttr"):
        st2[f] = st[f][perm]
    tr = (eng.F_TRACER_R, eng.F_TRACER_S, eng.F_TRACER_T, eng.F_TRACER_C)
    out, sorts = [], []
    for state in (st, st2):
        e = eng.Engine(cfg)
        e.upload(state)
        for _ in range(3):
            e.step()
        out.append([e.get(f) for f in (eng.F_T, eng.F_CNEW, eng.F_SF, eng.F_NEMPTY)] + [e.get(f) for f in tr])
        sorts.append(e.resorts())
        if state is st2:
            v = np.random.default_rng(5).random(len(perm))
            e.set(eng.F_TRACER_T, v)
            assert np.array_equal(e.get(eng.F_TRACER_T), v)
            e.set(eng.F_TRACER_T, out[1][6])
            e.step()  # the re-sorted state keeps stepping
            assert np.all(np.isfinite(e.get(eng.F_TRACER_R)))
        e.close()
    assert sorts[1] >= 1, "a shuffled tracer order must trigger a re-sort"
    for a, b in zip(out[0][:4], out[1][:4]):
        assert np.array_equal(a, b)
    for a, b in zip(out[0][4:], out[1][4:]):
        assert np.array_equal(a[perm], b)


@pytest.mark.parametrize("kind,nx,nz", GRIDS, ids=GRID_IDS)
def test_solve_psi_matches_oracle(kind, nx, nz):
    cfg, o, e = pair(kind, nx=nx, nz=nz)
    info = e.solve_psi()
    o.solve_psi()
    assert info["cycles"] == int(o.scalar("cycles"))
    assert rel_err(e.get(eng.F_SF), o.get(7)) < TOL
    assert rel_err(e.get(eng.F_U), o.get(8)) < TOL
    assert rel_err(e.get(eng.F_W), o.get(9)) < TOL
    assert rel_err(e.get(eng.F_VIS)[3:-3, 3:-3], o.get(10)[3:-3, 3:-3]) < 1e-12
    assert info["n_eta"] == int(o.scalar("n_eta"))
    e.close()


@pytest.mark.parametrize("kind,nx,nz", GRIDS, ids=GRID_IDS)
def test_step_matches_oracle(kind, nx, nz):
    cfg, o, e = pair(kind, nx=nx, nz=nz)
    e.solve_psi()
    o.solve_psi()
    dt, info = e.step()
    o.step()
    assert dt == o.scalar("dt")
    for fid, oid in ((eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22)):
        assert rel_err(e.get(fid), o.get(oid)) < TOL, fid
    assert rel_err(e.get(eng.F_T), o.get(0)) < TOL
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    if cfg.comp:
        assert rel_err(e.get(eng.F_CNEW), o.get(4)) < TOL
    e.close()


def test_stats_match_oracle():
    cfg, o, e = pair("chem")
    e.solve_psi()
    o.solve_psi()
    sg, so = e.stats(), o.stats()
    for k in ("empty_cells", "tracer_min", "tracer_max"):
        assert sg[k] == so[k]
    for k in ("Tavg", "Nu", "Nu_bot", "q1", "q2", "q3", "q4", "Cavg", "entrainment"):
        assert sg[k] == pytest.approx(so[k], rel=1e-13, abs=1e-300), k
    for k in ("vrms", "mobility", "strain_max", "RaT_avg"):
        assert sg[k] == pytest.approx(so[k], rel=TOL), k
    e.close()


def test_three_steps_stay_close():
    cfg, o, e = pair("chem")
    for _ in range(3):
        e.solve_psi()
        o.solve_psi()
        e.step()
        o.step()
    sg, so = e.stats(), o.stats()
    for k in ("Tavg", "vrms", "Nu", "Cavg"):
        assert sg[k] == pytest.approx(so[k], rel=TOL), k
    assert rel_err(e.get(eng.F_TRACER_R), o.get(20)) < TOL
    e.close()


@pytest.mark.parametrize("kind", ["iso", "chem", "depth"])
def test_mixed_precision_solve_meets_tolerance_and_matches_fp64(kind):
    """Mixed precision (FP32 cycles, FP64 residual/defect correction) reaches the same relative
    residual as the plain FP64 GPU solve; its psi is compared against the FP64 GPU psi."""
    from projectracer_gb300.config import PT_PREC_MIXED

    cfg, st = small_case(kind)
    e64 = eng.Engine(cfg)
    e64.upload(st)
    i64 = e64.solve_psi()
    sf64 = e64.get(eng.F_SF)
    e64.close()
    cfg.precision = PT_PREC_MIXED
    em = eng.Engine(cfg)
    em.upload(st)
    im = em.solve_psi()
    sfm = em.get(eng.F_SF)
    em.close()
    assert i64["resid_ratio"] <= cfg.tolerance and im["resid_ratio"] <= cfg.tolerance
    # both solutions satisfy |r|/|RHS| <= 1e-8; they agree to the solve tolerance times the
    # operator's conditioning, far below the discretisation error
    assert rel_err(sfm, sf64) < 1e-6


@pytest.mark.parametrize("kind", ["iso", "chem"])
def test_correction_scheme_solve_matches_oracle(kind):
    """mg_scheme = PT_MG_CORRECTION (coarse corrections restart from zero at each descent)."""
    from projectracer_gb300.config import PT_MG_CORRECTION

    cfg, st = small_case(kind)
    cfg.mg_scheme = PT_MG_CORRECTION
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    e = eng.Engine(cfg)
    e.upload(st)
    info = e.solve_psi()
    o.solve_psi()
    assert info["cycles"] == int(o.scalar("cycles"))
    assert rel_err(e.get(eng.F_SF), o.get(7)) < TOL
    e.close()


def test_cfl_steps_match_oracle():
    """The 1024x512 workload's physics on a 128x64 grid with velocity-limited time steps (CFL=1,
    energy.f90:809 and 859-866): dt, tracers and T after two full steps."""
    cfg, o, e = pair("c3", nx=128, nz=64)
    for _ in range(2):
        i0 = e.solve_psi()
        o.solve_psi()
        assert i0["cycles"] == int(o.scalar("cycles"))
        dt, _ = e.step()
        o.step()
        assert abs(dt - o.scalar("dt")) <= TOL * o.scalar("dt")
    for fid, oid in ((eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22)):
        assert rel_err(e.get(fid), o.get(oid)) < TOL, fid
    assert rel_err(e.get(eng.F_T), o.get(0)) < TOL
    assert rel_err(e.get(eng.F_SF), o.get(7)) < TOL
    e.close()


def test_mixed_precision_on_workload_physics():
    """Mixed precision on the 1024x512 workload's physics (viscosity contrast 1e5 x 10 in depth):
    same tolerance, same number of cycles as the FP64 correction-scheme solve, psi within 1e-6."""
    from projectracer_gb300.config import PT_PREC_MIXED

    cfg, st = small_case("c3", nx=128, nz=64)
    e = eng.Engine(cfg)
    e.upload(st)
    i64 = e.solve_psi()
    sf64 = e.get(eng.F_SF)
    e.close()
    cfg.precision = PT_PREC_MIXED
    e = eng.Engine(cfg)
    e.upload(st)
    im = e.solve_psi()
    assert im["resid_ratio"] <= cfg.tolerance
    assert abs(im["cycles"] - i64["cycles"]) <= 1
    assert rel_err(e.get(eng.F_SF), sf64) < 1e-6
    e.close()


def test_mixed_v_cycle_meets_tolerance():
    """The V-cycle schedule of the mixed-precision solve reaches the same FP64 residual test."""
    from projectracer_gb300.config import PT_CYCLE_V, PT_PREC_MIXED

    cfg, st = small_case("c3", nx=128, nz=64)
    e = eng.Engine(cfg)
    e.upload(st)
    e.solve_psi()
    sf64 = e.get(eng.F_SF)
    e.close()
    cfg.precision = PT_PREC_MIXED
    cfg.mg_cycle = PT_CYCLE_V
    e = eng.Engine(cfg)
    e.upload(st)
    im = e.solve_psi()
    assert im["resid_ratio"] <= cfg.tolerance
    assert rel_err(e.get(eng.F_SF), sf64) < 1e-6
    e.close()


def test_mixed_step_close_to_fp64():
    """A full mixed-precision step (FP32 multigrid inside FP64 defect correction, FP32 Taylor
    interpolation, FP64 positions) against the plain FP64 step from the same state: the tracers
    and T agree to the psi solve tolerance times the step's displacement."""
    from projectracer_gb300.config import PT_PREC_MIXED

    cfg, st = small_case("c3", nx=128, nz=64)
    out = {}
    for prec in (cfg.precision, PT_PREC_MIXED):
        c = cfg.copy()
        c.precision = prec
        e = eng.Engine(c)
        e.upload(st)
        e.solve_psi()
        dt, _ = e.step()
        out[prec] = {f: e.get(f) for f in (eng.F_TRACER_R, eng.F_TRACER_S, eng.F_TRACER_T, eng.F_T)}
        out[prec]["dt"] = dt
        e.close()
    a, b = out[cfg.precision], out[PT_PREC_MIXED]
    assert abs(a["dt"] - b["dt"]) <= 1e-6 * a["dt"]
    for f in (eng.F_TRACER_R, eng.F_TRACER_S):
        assert rel_err(b[f], a[f]) < 1e-7, f
    assert rel_err(b[eng.F_TRACER_T], a[eng.F_TRACER_T]) < 1e-6
    assert rel_err(b[eng.F_T], a[eng.F_T]) < 1e-6


def test_extrapolated_guess_steps_close_to_previous_guess():
    """PT_GUESS_EXTRAPOLATE (psi extrapolated in time between the solves of a step) only changes
    where each solve starts: after two full steps the tracers agree with the previous-psi run to
    the solve tolerance, and the extrapolated run needs no more cycles."""
    from projectracer_gb300.config import PT_GUESS_EXTRAPOLATE, PT_GUESS_PREVIOUS, PT_PREC_MIXED

    cfg, st = small_case("c3", nx=128, nz=64)
    cfg.precision = PT_PREC_MIXED
    out, cycles = {}, {}
    for mode in (PT_GUESS_PREVIOUS, PT_GUESS_EXTRAPOLATE):
        c = cfg.copy()
        c.guess_mode = mode
        e = eng.Engine(c)
        e.upload(st)
        n = 0
        for _ in range(3):
            n += e.solve_psi()["cycles"]
            n += e.step()[1]["cycles"]
        out[mode] = (e.get(eng.F_TRACER_R), e.get(eng.F_TRACER_S), e.get(eng.F_T))
        cycles[mode] = n
        e.close()
    for a, b in zip(out[PT_GUESS_PREVIOUS], out[PT_GUESS_EXTRAPOLATE]):
        assert rel_err(b, a) < 1e-6
    assert cycles[PT_GUESS_EXTRAPOLATE] <= cycles[PT_GUESS_PREVIOUS]


def test_mixed_tables_match_fp64_stencils():
    """The mixed RK stage's FP32 tables (value and x-derivatives 1..3 of u and w, built from exact
    integer stencil sums) against the same stencils in FP64 on the downloaded velocities: the
    values to FP32 rounding, the derivatives to 1e-6 of their largest magnitude."""
    from projectracer_gb300.config import PT_PREC_MIXED

    cfg, st = small_case("c3")
    cfg.precision = PT_PREC_MIXED
    e = eng.Engine(cfg)
    e.upload(st)
    e.solve_psi()
    e.step()
    nx, nz = cfg.nx, cfg.nz
    dr = cfg.aspect / nx
    taps = {1: ([1, -8, 0, 8, -1], 12.0, 2), 2: ([-1, 16, -30, 16, -1], 12.0, 2),
            3: ([1, -8, 13, 0, -13, 8, -1], 8.0, 3)}
    for which, field in ((0, eng.F_U), (1, eng.F_W)):
        f = e.get(field)  # rows k = -3..nz+3, columns i = -3..nx+3
        tab = e.table(which).astype(np.float64)
        assert np.array_equal(tab[..., 0], f[:, 3:nx + 4].astype(np.float32).astype(np.float64))
        for m, (w, den, half) in taps.items():
            ref = np.zeros((nz + 7, nx + 1))
            for j, c in enumerate(w):
                off = j - half
                ref += c * f[:, 3 + off:3 + off + nx + 1]
            ref /= den * dr ** m
            scale = np.abs(ref).max()
            assert scale > 0
            assert np.abs(tab[..., m] - ref).max() <= 1e-6 * scale, (which, m)
    e.close()
