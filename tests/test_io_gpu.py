"""The snapshot and restart files written from the device state (snapshots, main.f90:377-424;
print_restart, main.f90:457-496) and the restart read (grid.f90:55-104), through the C ABI.

  * restart records: what the library writes is read back by the Python reader of the same
    gfortran record form bit for bit, equals the state the engine holds, and a fresh engine that
    reads the files continues exactly as the original; also in mixed precision after the tracers
    were re-sorted (the records keep the caller's order), with discrete tracer types (an integer*4
    Ttype record), and with records split into sub-records (byte-identical to the Python writer's
    split);
  * the writes are asynchronous: a step started right after the call does not change what is
    written;
  * the t=0 snapshot of the shipped run (direct solve) reproduces the reference's own T10000 and
    P10000 text, line for line, in the sampled lines.
"""
import os

import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from projectracer_gb300 import inputs
from projectracer_gb300.config import PT_PREC_MIXED
from tests.helpers import golden_t0, small_case

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GRID = (("T", eng.F_T), ("Cnew", eng.F_CNEW), ("SF", eng.F_SF))
TRACERS = (("rtr", eng.F_TRACER_R), ("str", eng.F_TRACER_S), ("Ctr", eng.F_TRACER_C), ("Ttr", eng.F_TRACER_T))


def _state(e):
    return {k: e.get(f) for k, f in GRID + TRACERS}


def _same(a, b):
    for k in a:
        if k in b:
            assert np.array_equal(np.asarray(a[k]).reshape(-1), np.asarray(b[k]).reshape(-1)), k


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_restart_round_trip(tmp_path, precision):
    cfg, st = small_case("chem")
    cfg.precision = precision
    if precision == PT_PREC_MIXED:  # a shuffled upload: the mixed path re-sorts its tracers
        perm = np.random.default_rng(2).permutation(cfg.ntr)
        st = dict(st)
        for f in ("rtr", "str", "Ctr", "Ttr"):
            st[f] = st[f][perm]
    e = eng.Engine(cfg)
    e.upload(st)
    for _ in range(3):
        e.solve_psi()
        e.step()
    if precision == PT_PREC_MIXED:
        assert e.resorts() >= 1
    held = _state(e)
    e.write_restart(str(tmp_path))
    e.step()  # queued after the copies: does not change what is written
    e.io_wait()
    _same(held, inputs.read_restart(str(tmp_path), cfg))
    # continue from the original and from a fresh engine that reads the files
    e2 = eng.Engine(cfg)
    e2.read_restart(str(tmp_path))
    e.close()
    e = eng.Engine(cfg)
    e.upload(held | {"xg": st["xg"], "zg": st["zg"]})
    for x in (e, e2):
        x.solve_psi()
        x.step()
    _same(_state(e), _state(e2))
    e.close()
    e2.close()


def test_restart_sub_records_and_types(tmp_path):
    cfg, st = small_case("chem")
    cfg.discrete_types = 1
    st = dict(st)
    st["Ttype"] = (st["Ctr"] > 0.5).astype(np.int32)
    e = eng.Engine(cfg)
    e.upload(st)
    e.solve_psi()
    e.step()
    e._check(e.L.pt_prof_record_limit(4096))
    e.write_restart(str(tmp_path))
    e.io_wait()
    back = inputs.read_restart(str(tmp_path), cfg)
    assert np.array_equal(back["Ttype"], st["Ttype"])
    assert np.array_equal(back["rtr"], e.get(eng.F_TRACER_R))
    # the Python writer with the same split writes the same bytes
    old = inputs._MAXREC
    try:
        inputs._MAXREC = 4096
        ref = tmp_path / "py"
        ref.mkdir()
        grid = [back["xg"], back["zg"], back["T"], back["Cnew"], back["SF"]]
        with open(ref / "Trestart", "wb") as fh:
            inputs._write_record(fh, b"".join(np.ascontiguousarray(x, dtype="<f8").tobytes() for x in grid))
        trc = [back["rtr"].tobytes(), back["str"].tobytes(), back["Ttype"].astype("<i4").tobytes(), back["Ttr"].tobytes()]
        with open(ref / "restart_tracers", "wb") as fh:
            inputs._write_record(fh, b"".join(trc))
    finally:
        inputs._MAXREC = old
    for name in ("Trestart", "restart_tracers"):
        assert (tmp_path / name).read_bytes() == (ref / name).read_bytes(), name
    assert (tmp_path / "restart_tracers").stat().st_size > 3 * 4096  # really split
    e2 = eng.Engine(cfg)
    e2.read_restart(str(tmp_path))
    assert np.array_equal(e2.get(eng.F_TRACER_TYPE), st["Ttype"])
    e2.close()
    e.close()


def test_snapshot_t0_is_the_reference_text(tmp_path, golden):
    import json

    cfg, st, start, _ = golden_t0(golden, direct=1)
    e = eng.Engine(cfg)
    e.upload(st)
    for f, v in start.items():
        e.set(f, v)
    e.solve_psi()
    e.write_snapshot(str(tmp_path), 0)
    e.io_wait()
    e.close()
    with open(os.path.join(HERE, "golden", "snapshot_t0_lines.json")) as fh:
        ref = json.load(fh)
    mine_t = (tmp_path / "T10000").read_text().split("\n")
    mine_p = [ln for ln in (tmp_path / "P10000").read_text().split("\n") if ln]
    assert len(mine_t) == (cfg.nx + 1) * (cfg.nz + 2) + 1
    bad = [(n, line, mine_t[n]) for n, line in ref["T10000"] if mine_t[n] != line]
    assert not bad, bad[:3]
    assert mine_p == ref["P10000"]
