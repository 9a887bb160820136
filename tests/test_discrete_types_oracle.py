"""The oracle's restatement of the discrete-type projection (tracers_to_corners_OG,
composition.f90:1090-1276, ntype=1, bilinear shape function) on the CPU: per-type counts add up,
and the node values agree with the continuous projection of the same tracers with C = type to the
last bits (the two differ only in how the shape sums are grouped: nempty_real is the sum of the
per-type shape sums, composition.f90:1221)."""
import numpy as np

from oracle.ptref import Oracle
from tests.helpers import small_case


def _types(st, seed=5):
    ty = (st["Ctr"] > 0.5).astype(np.int32)
    flip = np.random.default_rng(seed).random(len(ty)) < 0.1
    ty[flip] = 1 - ty[flip]
    return ty


def test_discrete_projection_counts_and_values():
    cfg, st = small_case("chem")
    cfg.discrete_types = 1
    ty = _types(st)
    for nparts in (0, 2):  # canonical order and the reference's two-thread order
        o = Oracle(cfg, iterate=1, nparts=nparts)
        o.set_types(ty)
        o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
        n, n1 = o.get(11), o.get(13)
        assert n.sum() == len(ty) and n1.sum() == ty.sum()
        assert np.all((n1 >= 0) & (n1 <= n))
        C = o.get(4)[5:-5, 5:-5]
        assert C.min() >= 0.0 and C.max() <= 1.0
        assert np.array_equal(o.get(24), ty)
    c2 = cfg.copy()
    c2.discrete_types = 0
    cont = Oracle(c2, iterate=1, nparts=0)
    cont.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], ty.astype(float),
                      st["Ttr"])
    og = Oracle(cfg, iterate=1, nparts=0)
    og.set_types(ty)
    og.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    assert np.max(np.abs(cont.get(4) - og.get(4))) <= 4 * np.finfo(float).eps
    assert np.max(np.abs(cont.get(1) - og.get(1))) <= 4 * np.finfo(float).eps
    assert np.array_equal(cont.get(11), og.get(11))
