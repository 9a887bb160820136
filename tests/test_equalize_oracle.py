"""Tracer equalisation (equalize_tracers, composition.f90:266-763) in the oracle, on the CPU.

The reference's own result depends on its OpenMP thread count (one mzran stream per thread); the
restatement follows its rules with counter-based random numbers.  What the reference's rules fix is
checked here:
  * donors come only from nodes above their type's target, receivers are nodes below it, and a
    node receives at most as many tracers as it lacked;
  * tracers are conserved, stay in the domain, and moved tracers take their node's majority type;
  * the poorest level is filled first: after the moves no node lacks more than before, and the
    deficit shrinks by the number moved;
  * same seed, same result; another seed moves other tracers.
"""
import numpy as np
import pytest

from oracle.ptref import Oracle
from tests.helpers import small_case


def clustered(kind="chem", nx=64, nz=32, tpc=8, frac=0.05, seed=5):
    """A state whose tracers have drifted: `frac` of them gathered into a small box."""
    cfg, st = small_case(kind, nx=nx, nz=nz, tpc=tpc)
    rng = np.random.default_rng(seed)
    n = len(st["rtr"])
    idx = rng.choice(n, int(frac * n), replace=False)
    st = dict(st)
    st["rtr"] = st["rtr"].copy()
    st["str"] = st["str"].copy()
    st["rtr"][idx] = 0.3 * cfg.aspect + 0.05 * rng.random(len(idx))
    st["str"][idx] = 0.5 + 0.05 * rng.random(len(idx))
    cfg.equalize = 1
    cfg.tpc = tpc
    cfg.Cinit = 0.2
    if cfg.comp:
        cfg.discrete_types = 1
        st["Ttype"] = (st["Ctr"] > 0.5).astype(np.int32)
    return cfg, st


def oracle_for(cfg, st):
    o = Oracle(cfg, iterate=1, nparts=0)
    if cfg.comp:
        o.set_types(st["Ttype"])
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    return o


def node_counts(cfg, r, s):
    i = np.rint(r / (cfg.aspect / cfg.nx)).astype(int)
    k = np.rint(s / (1.0 / cfg.nz)).astype(int)
    return np.bincount(i + (cfg.nx + 1) * k, minlength=(cfg.nx + 1) * (cfg.nz + 1))


@pytest.mark.parametrize("kind", ["chem", "iso"])
def test_equalize_rules(kind):
    cfg, st = clustered(kind)
    o = oracle_for(cfg, st)
    r0, s0 = o.get(20).copy(), o.get(21).copy()
    ty0 = o.get(24).copy() if cfg.comp else None
    before = node_counts(cfg, r0, s0)
    info = o.equalize()
    r1, s1 = o.get(20), o.get(21)
    after = node_counts(cfg, r1, s1)
    moved = (r1 != r0) | (s1 != s0)
    assert info["nfree"] > 0 and 0 < info["moved"] <= info["nfree"]
    assert moved.sum() == info["moved"]
    assert after.sum() == before.sum() == len(r0)
    assert np.all((r1 >= 0) & (r1 <= cfg.aspect) & (s1 >= 0) & (s1 <= 1))
    # donors left rich nodes; receivers were poor and gained at most their deficit
    node_from = (np.rint(r0[moved] / (cfg.aspect / cfg.nx)) + (cfg.nx + 1) * np.rint(s0[moved] * cfg.nz)).astype(int)
    node_to = (np.rint(r1[moved] / (cfg.aspect / cfg.nx)) + (cfg.nx + 1) * np.rint(s1[moved] * cfg.nz)).astype(int)
    gained = np.bincount(node_to, minlength=len(before))
    target = info["tpc_type"][0] if cfg.comp == 0 else max(info["tpc_type"])
    assert np.all(before[node_from] > min(info["tpc_type"][: 1 + cfg.comp]))
    assert np.all(gained[gained > 0] <= np.maximum(target - before[gained > 0], 0) + 0)
    # the poorest nodes gained first: the least count among receiving nodes did not fall
    recv = np.unique(node_to)
    assert after[recv].min() >= before[recv].min()
    if cfg.comp:
        ty1 = o.get(24)
        assert np.array_equal(ty1[~moved], ty0[~moved])
        assert info["count_type"][0] + info["count_type"][1] == len(r0)


def test_equalize_deterministic_and_seeded():
    cfg, st = clustered()
    runs = []
    for seed in (1, 1, 2):
        c = cfg.copy()
        c.eq_seed = seed
        o = oracle_for(c, st)
        info = o.equalize()
        runs.append((o.get(20).copy(), o.get(21).copy(), o.get(22).copy(), o.get(24).copy(), info))
    a, b, c = runs
    for x, y in zip(a[:4], b[:4]):
        assert np.array_equal(x, y)
    assert a[4] == b[4]
    assert not np.array_equal(a[0], c[0])
    assert a[4]["moved"] == c[4]["moved"]  # how many move does not depend on the draws


def test_equalize_nothing_to_do():
    cfg, st = small_case("iso", nx=32, nz=32, tpc=4)
    cfg.equalize, cfg.tpc = 1, 1 << 20  # every node is below target, none above: no donors
    o = oracle_for(cfg, st)
    r0 = o.get(20).copy()
    info = o.equalize()
    assert info["moved"] == 0 and info["nfree"] == 0
    assert np.array_equal(o.get(20), r0)


def test_step_runs_equalize_first():
    cfg, st = clustered()
    o = oracle_for(cfg, st)
    r0 = o.get(20).copy()
    o.solve_psi()
    o.step()
    c = cfg.copy()
    c.equalize = 0
    o2 = oracle_for(c, st)
    o2.solve_psi()
    o2.step()
    assert not np.array_equal(o.get(20), o2.get(20))
    assert np.all(np.isfinite(o.get(20))) and len(o.get(20)) == len(r0)
