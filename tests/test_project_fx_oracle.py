"""The fixed-point restatement of the mixed-precision projection (oracle/project_fx.py) against
the FP64 restatement of the reference's projection (oracle/ptref, composition.f90:942-1087):
counts identical, projected fields within the fixed-point resolution.  CPU only."""
import numpy as np
import pytest

from oracle.project_fx import ONE, fix28, floor_fix, project_fx, ratios
from oracle.ptref import Oracle
from projectracer_gb300 import engine as eng
from tests.helpers import rel_err, small_case, walls


def test_fix28_rounds_half_away_from_zero():
    q = 2.0 ** -28
    v = np.array([0.0, 0.5 * q, -0.5 * q, 1.5 * q, -1.5 * q, 0.49999 * q, 1.0, -1.0, 3.999999])
    assert fix28(v).tolist() == [0, 1, -1, 2, -2, 0, ONE, -ONE, int(np.floor(3.999999 * ONE + 0.5))]
    with pytest.raises(ValueError):
        fix28(np.array([4.0]))


def test_floor_fix_on_nodes_and_walls():
    i0, f = floor_fix(np.array([0.0, 0.25, 0.375, 2.0]), 0.125)
    assert i0.tolist() == [0, 2, 3, 16] and f.tolist() == [0, 0, 0, 0]
    i0, f = floor_fix(np.array([0.125 * (5 + 0.75)]), 0.125)
    assert i0.tolist() == [5] and f.tolist() == [3 * ONE // 4]


@pytest.mark.parametrize("kind", ["iso", "chem", "c3"])
def test_fixed_point_projection_matches_reference_order(kind):
    cfg, st = small_case(kind)
    st = walls(cfg, st)
    o = Oracle(cfg, iterate=1, nparts=0)
    o.load_restart(st["xg"], st["zg"], st["T"], st["Cnew"], st["SF"], st["rtr"], st["str"], st["Ctr"], st["Ttr"])
    TS, CS, S, cnt = project_fx(cfg.nx, cfg.nz, cfg.aspect, st["rtr"], st["str"], st["Ttr"],
                                st["Ctr"] if cfg.comp else None)
    assert np.array_equal(cnt, o.get(11))
    g = 3  # ghost width of the T fields
    ref_T = o.get(eng.F_TRATIO)[g:-g, g:-g]
    Tr, Cr = ratios(TS, CS, S, ref_T, o.get(4)[5:-5, 5:-5] if cfg.comp else None)
    assert rel_err(Tr[1:-1, 1:-1], ref_T[1:-1, 1:-1]) < 1e-7
    if cfg.comp:
        assert rel_err(Cr, o.get(4)[5:-5, 5:-5]) < 1e-7


def test_fixed_point_projection_independent_of_order():
    cfg, st = small_case("chem")
    p = np.random.default_rng(5).permutation(len(st["rtr"]))
    a = project_fx(cfg.nx, cfg.nz, cfg.aspect, st["rtr"], st["str"], st["Ttr"], st["Ctr"])
    b = project_fx(cfg.nx, cfg.nz, cfg.aspect, st["rtr"][p], st["str"][p], st["Ttr"][p], st["Ctr"][p])
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
