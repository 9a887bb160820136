"""The learned psi guess end to end: training pairs written by the FP64 solver, the network trained
on them with its own tensor-core kernels, and what the trained network gains over the solve
without it (the zero guess) on held-out states."""
import os

import numpy as np
import pytest

from projectracer_gb300 import engine as eng
from projectracer_gb300 import learned as ln
from projectracer_gb300.config import PT_GUESS_UNET, PT_GUESS_ZERO
from projectracer_gb300.inputs import make_state

pytestmark = pytest.mark.gpu

NX, NZ = 64, 32


def _scaled_error(guess, psi):
    """Relative L2 error of the best multiple of the guess (interior nodes)."""
    g, p = guess[1:, 1:].ravel().astype(np.float64), psi[1:, 1:].ravel().astype(np.float64)
    a = float(g @ p) / max(float(g @ g), 1e-300)
    return float(np.linalg.norm(a * g - p) / np.linalg.norm(p))


def test_trained_guess_beats_untrained_and_keeps_cycles_bounded(tmp_path):
    rng = np.random.default_rng(21)
    X, Y = ln.solver_pairs(rng, 48, NX, NZ)
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(Y))
    assert np.allclose(np.max(np.abs(Y), axis=(1, 2)), 1.0)  # psi / max|psi|
    untrained = ln.UNet(NZ, NX, 8, seed=5)
    net = ln.UNet(NZ, NX, 8, seed=5)
    hist = ln.train(net, X, Y, epochs=20, batch=8, lr=1e-3)
    assert hist[-1] < 0.1 * hist[0]
    path = str(tmp_path / "unet.bin")
    net.save(path)
    Xe, Ye = ln.solver_pairs(np.random.default_rng(77), 4, NX, NZ)
    err_trained = [_scaled_error(g, p) for g, p in zip(net.forward(Xe), Ye)]
    err_untrained = [_scaled_error(g, p) for g, p in zip(untrained.forward(Xe), Ye)]
    # the trained network's starting point is far closer to the converged psi than an untrained one
    assert np.mean(err_trained) < 0.5 * np.mean(err_untrained)
    assert np.mean(err_trained) < 0.3
    # in the solver: same tolerance, at most one cycle more than from zero (the fallback bound)
    ev = np.random.default_rng(78)
    for _ in range(2):
        cfg = ln.sample_config(ev, NX, NZ)
        st = make_state(cfg, int(ev.integers(1 << 30)), noise=1e-3)
        cyc = {}
        for mode in (PT_GUESS_ZERO, PT_GUESS_UNET):
            e = eng.Engine(cfg)
            e.upload(st)
            e.set_guess_mode(mode, path if mode == PT_GUESS_UNET else None)
            info = e.solve_psi()
            assert info["resid_ratio"] <= cfg.tolerance
            cyc[mode] = info["cycles"]
            e.close()
        assert cyc[PT_GUESS_UNET] <= cyc[PT_GUESS_ZERO] + 1
    net.close()
    untrained.close()
    os.remove(path)
