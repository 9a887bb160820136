"""Training pairs of a time-evolved run (pt_pair_capture / pt_pair_take): every converged solve of
a step -- the top-of-step solve and the three RK-stage solves -- records the pair that
pt_training_pair writes for the current state, and the pairs round-trip through .npy shards."""
import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from projectracer_gb300 import learned
from tests.helpers import small_case

pytestmark = pytest.mark.gpu


def test_pairs_of_every_solve(tmp_path):
    cfg, st = small_case("chem", nx=128, nz=64)
    e = eng.Engine(cfg)
    e.upload(st)
    learned.pair_capture(16)
    e.solve_psi()
    x_top, y_top = learned.training_pair(e)
    e.step()
    e.solve_psi()
    e.step()
    X, Y = learned.pair_take(e, 16)
    assert X.shape == (8, 4, 64, 128) and Y.shape == (8, 64, 128)
    assert np.array_equal(X[0], x_top) and np.array_equal(Y[0], y_top)
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(Y))
    assert np.allclose(np.abs(Y).reshape(8, -1).max(axis=1), 1.0)  # psi / max|psi|
    assert not np.array_equal(Y[1], Y[0]) and not np.array_equal(X[4], X[0])
    X2, _ = learned.pair_take(e, 16)
    assert len(X2) == 0  # taken pairs leave the buffer
    learned.pair_capture(2)  # capacity bounds what is recorded
    e.solve_psi()
    e.step()
    X3, _ = learned.pair_take(e, 16)
    assert len(X3) == 2
    learned.pair_capture(0)
    e.close()
    names = learned.write_shards(X, Y, str(tmp_path), shard=3)
    assert names == ["00000", "00001", "00002"]
    Xr, Yr = learned.read_shards(str(tmp_path))
    assert np.array_equal(Xr, X) and np.array_equal(Yr, Y)
