"""Discrete tracer types (iC_continuous=0, ntype=1: tracers_to_corners_OG, composition.f90:1090-1276)
on the GPU, through the C ABI, against the oracle's restatement.

FP64: the projection sums T*S and the per-type shape sums in the canonical order, nempty_real =
count_type_real(0) + count_type_real(1), C = count_type_real(1) / nempty_real, T = T1 / nempty_real:
node values, tracer counts and per-type counts bit for bit; one step to 1e-10.  Mixed precision:
the fixed-point projection of the type (0 or 1) as C, bit for bit against its integer
restatement (the per-type shape sums of integer weights add exactly), per-type counts exact.  The
types cross the ABI as int32 in the caller's order, also after the mixed path re-sorts its
tracers.
"""
import numpy as np
import pytest

from oracle.ptref import Oracle
from projectracer_gb300 import engine as eng
from projectracer_gb300.config import PT_PREC_MIXED
from tests.helpers import rel_err, small_case

pytestmark = pytest.mark.gpu


def _case(nx=64, nz=64, seed=5):
    cfg, st = small_case("chem", nx=nx, nz=nz)
    cfg.discrete_types = 1
    ty = (st["Ctr"] > 0.5).astype(np.int32)
    flip = np.random.default_rng(seed).random(len(ty)) < 0.1
    ty[flip] = 1 - ty[flip]
    st = dict(st)
    st["Ttype"] = ty
    return cfg, st


def _oracle(cfg, st):
    o = Oracle(cfg, iterate=1, nparts=0)
    o.set_types(st["Ttype"])
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    return o


@pytest.mark.parametrize("nx,nz", [(64, 64), (96, 48)])
def test_discrete_projection_bit_exact(nx, nz):
    cfg, st = _case(nx, nz)
    o = _oracle(cfg, st)
    e = eng.Engine(cfg)
    e.upload(st)
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    assert np.array_equal(e.get(eng.F_COUNT_TYPE), o.get(13))
    assert np.array_equal(e.get(eng.F_CNEW), o.get(4))
    for fid in (eng.F_TRATIO, eng.F_TVIS, eng.F_TBUOY):
        assert np.array_equal(e.get(fid)[1:-1, 1:-1], o.get(fid)[1:-1, 1:-1]), fid
    assert np.array_equal(e.get(eng.F_TRACER_TYPE), st["Ttype"])
    e.close()


def test_discrete_step_matches_oracle():
    cfg, st = _case()
    o = _oracle(cfg, st)
    e = eng.Engine(cfg)
    e.upload(st)
    for _ in range(2):
        i0 = e.solve_psi()
        o.solve_psi()
        assert i0["cycles"] == int(o.scalar("cycles"))
        dt, _ = e.step()
        o.step()
        assert dt == o.scalar("dt")
    for fid, oid in ((eng.F_TRACER_R, 20), (eng.F_TRACER_S, 21), (eng.F_TRACER_T, 22), (eng.F_T, 0), (eng.F_CNEW, 4),
                     (eng.F_SF, 7)):
        assert rel_err(e.get(fid), o.get(oid)) < 1e-10, fid
    assert np.array_equal(e.get(eng.F_NEMPTY), o.get(11))
    assert np.array_equal(e.get(eng.F_COUNT_TYPE), o.get(13))
    ty = np.empty(cfg.ntr, dtype=np.int32)
    e._check(e.L.pt_download_state(None, None, None, None, None, None, None, ty.ctypes.data))
    assert np.array_equal(ty, st["Ttype"])
    e.close()


def test_discrete_mixed_projection_and_resort():
    from oracle.project_fx import project_fx, ratios

    cfg, st = _case()
    cfg.precision = PT_PREC_MIXED
    perm = np.random.default_rng(3).permutation(cfg.ntr)  # a shuffled order: the mixed path re-sorts
    st2 = dict(st)
    for f in ("rtr", "str", "Ctr", "Ttr", "Ttype"):
        st2[f] = st[f][perm]
    e = eng.Engine(cfg)
    e.upload(st2)
    TS, CS, S, cnt = project_fx(cfg.nx, cfg.nz, cfg.aspect, st2["rtr"], st2["str"], st2["Ttr"],
                                st2["Ttype"].astype(float))
    assert np.array_equal(e.get(eng.F_NEMPTY), cnt)
    Tg = e.get(eng.F_TRATIO)[3:-3, 3:-3]
    Cg = e.get(eng.F_CNEW)[5:-5, 5:-5]
    Tr, Cr = ratios(TS, CS, S, Tg, Cg)
    assert np.array_equal(Tg[1:-1, 1:-1], Tr[1:-1, 1:-1])
    assert np.array_equal(Cg[1:-1, 1:-1], Cr[1:-1, 1:-1])
    o = _oracle(cfg.copy(), st)  # per-type counts do not depend on the order
    assert np.array_equal(e.get(eng.F_COUNT_TYPE), o.get(13))
    for _ in range(3):
        e.solve_psi()
        e.step()
    assert e.resorts() >= 1
    assert np.array_equal(e.get(eng.F_TRACER_TYPE), st2["Ttype"])  # the caller's order
    flipped = st2["Ttype"].copy()
    flipped[:100] = 1 - flipped[:100]
    e.set(eng.F_TRACER_TYPE, flipped)
    assert np.array_equal(e.get(eng.F_TRACER_TYPE), flipped)
    assert np.array_equal(e.get(eng.F_TRACER_C), flipped.astype(float))
    e.close()


def test_discrete_types_argument_checks():
    cfg, st = _case()
    e = eng.Engine(cfg)
    bad = dict(st)
    bad["Ttype"] = st["Ttype"].copy()
    bad["Ttype"][7] = 2
    with pytest.raises(eng.PtError) as ex:
        e.upload(bad)
    assert ex.value.code == -9
    e.upload(st)
    with pytest.raises(eng.PtError) as ex:
        e.set(eng.F_TRACER_C, st["Ctr"])
    assert ex.value.code == -9
    e.close()
    c2 = cfg.copy()
    c2.discrete_types = 0
    e = eng.Engine(c2)
    with pytest.raises(eng.PtError):
        e.get(eng.F_COUNT_TYPE) if False else e.extent(eng.F_TRACER_TYPE)
    e.close()
