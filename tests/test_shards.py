"""Training-pair shards (the learned guess's data set): write_shards splits the (input, psi) pairs
into numbered .npy files of at most `shard` pairs, read_shards concatenates every shard of a
directory in order; a second run appends with `start` and the order is kept."""
import numpy as np

from projectracer_gb300.learned import read_shards, write_shards


def test_shards_round_trip_in_order(tmp_path):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((600, 4, 8, 16)).astype(np.float32)
    Y = (2.0 * X[:, 0] - X[:, 3]).astype(np.float32)
    names = write_shards(X[:400], Y[:400], str(tmp_path), shard=256)
    names += write_shards(X[400:], Y[400:], str(tmp_path), shard=256, start=len(names))
    assert names == ["00000", "00001", "00002"]
    X2, Y2 = read_shards(str(tmp_path))
    assert X2.dtype == np.float32 and np.array_equal(X2, X) and np.array_equal(Y2, Y)


def test_read_shards_of_an_empty_directory(tmp_path):
    X, Y = read_shards(str(tmp_path))
    assert len(X) == 0 and len(Y) == 0
