"""The learned psi guess from Python: the network handle (include/ptgpu_unet.h), training pairs
written out by the FP64 solver, and training with the network's own tensor-core kernels.

    net = UNet(nz, nx, max_batch=8, seed=1)
    X, Y = solver_pairs(configs_and_states)      # FP64 solves -> (inputs, psi) pairs
    train(net, X, Y, epochs=20, batch=8, lr=1e-3)
    net.save("unet.bin"); engine.set_guess_mode(PT_GUESS_UNET, "unet.bin")
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import engine as eng
from .config import PT_GUESS_PREVIOUS, PT_GUESS_UNET, PT_GUESS_ZERO, PT_PREC_FP64, PtConfig, workload
from .inputs import make_state

_c = ctypes


def _bind(L):
    if getattr(L, "_unet_bound", False):
        return L
    vp, i32, f32p = _c.c_void_p, _c.c_int, _c.POINTER(_c.c_float)
    L.pt_unet_create.argtypes = [i32, i32, i32, _c.c_uint64, _c.POINTER(vp)]
    L.pt_unet_destroy.argtypes = [vp]
    L.pt_unet_num_params.argtypes = [vp, _c.POINTER(_c.c_int64)]
    L.pt_unet_get_params.argtypes = [vp, vp]
    L.pt_unet_set_params.argtypes = [vp, vp]
    L.pt_unet_forward.argtypes = [vp, vp, i32, vp]
    L.pt_unet_gradients.argtypes = [vp, vp, vp, i32, vp, f32p]
    L.pt_unet_train_step.argtypes = [vp, vp, vp, i32, _c.c_float, f32p]
    L.pt_unet_save.argtypes = [vp, _c.c_char_p]
    L.pt_unet_load.argtypes = [_c.c_char_p, i32, i32, i32, _c.POINTER(vp)]
    L.pt_training_pair.argtypes = [vp, vp]
    L.pt_unet_guess_info.argtypes = [_c.POINTER(i32), _c.POINTER(_c.c_double), _c.POINTER(_c.c_double)]
    L.pt_tc_gemm_check.argtypes = [vp, vp, vp, i32, i32, i32]
    L.pt_unet_profile_forward.argtypes = [vp, vp, i32, vp]
    L.pt_pair_capture.argtypes = [i32]
    L.pt_pair_take.argtypes = [vp, vp, i32, _c.POINTER(i32)]
    L._unet_bound = True
    return L


def library():
    return _bind(eng.load_library())


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class UNet:
    """A network on the nz x nx node grid (both multiples of 8)."""

    def __init__(self, nz: int, nx: int, max_batch: int = 8, seed: int = 1, handle=None):
        self.L = library()
        self.nz, self.nx, self.max_batch = nz, nx, max_batch
        self.h = _c.c_void_p()
        if handle is not None:
            self.h = handle
        else:
            self._ok(self.L.pt_unet_create(nz, nx, max_batch, seed, _c.byref(self.h)))

    @classmethod
    def load(cls, path: str, nz: int, nx: int, max_batch: int = 8) -> "UNet":
        L = library()
        h = _c.c_void_p()
        rc = L.pt_unet_load(path.encode(), nz, nx, max_batch, _c.byref(h))
        if rc:
            raise eng.PtError(rc, L.pt_last_error().decode())
        return cls(nz, nx, max_batch, handle=h)

    def _ok(self, rc):
        if rc:
            raise eng.PtError(rc, self.L.pt_last_error().decode())

    def num_params(self) -> int:
        n = _c.c_int64()
        self._ok(self.L.pt_unet_num_params(self.h, _c.byref(n)))
        return n.value

    def params(self) -> np.ndarray:
        p = np.zeros(self.num_params(), dtype=np.float32)
        self._ok(self.L.pt_unet_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p: np.ndarray):
        p = _f32(p)
        self._ok(self.L.pt_unet_set_params(self.h, p.ctypes.data))

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = _f32(x)
        y = np.zeros((x.shape[0], self.nz, self.nx), dtype=np.float32)
        self._ok(self.L.pt_unet_forward(self.h, x.ctypes.data, x.shape[0], y.ctypes.data))
        return y

    def gradients(self, x: np.ndarray, t: np.ndarray):
        x, t = _f32(x), _f32(t)
        g = np.zeros(self.num_params(), dtype=np.float32)
        loss = _c.c_float()
        self._ok(self.L.pt_unet_gradients(self.h, x.ctypes.data, t.ctypes.data, x.shape[0], g.ctypes.data,
                                          _c.byref(loss)))
        return loss.value, g

    def train_step(self, x: np.ndarray, t: np.ndarray, lr: float) -> float:
        x, t = _f32(x), _f32(t)
        loss = _c.c_float()
        self._ok(self.L.pt_unet_train_step(self.h, x.ctypes.data, t.ctypes.data, x.shape[0], lr, _c.byref(loss)))
        return loss.value

    def profile_forward(self, x: np.ndarray) -> np.ndarray:
        """Device ms of each convolution GEMM of one forward pass (pt_unet_profile_forward)."""
        x = _f32(x)
        ms = np.zeros(14, dtype=np.float32)
        self._ok(self.L.pt_unet_profile_forward(self.h, x.ctypes.data, x.shape[0], ms.ctypes.data))
        return ms

    def save(self, path: str):
        self._ok(self.L.pt_unet_save(self.h, path.encode()))

    def close(self):
        if self.h:
            self.L.pt_unet_destroy(self.h)
            self.h = _c.c_void_p()


def training_pair(e: eng.Engine):
    """(x [4][nz][nx], psi [nz][nx]) of the engine's current state, after a solve."""
    L = library()
    x = np.zeros((4, e.nz, e.nx), dtype=np.float32)
    y = np.zeros((e.nz, e.nx), dtype=np.float32)
    rc = L.pt_training_pair(x.ctypes.data, y.ctypes.data)
    if rc:
        raise eng.PtError(rc, L.pt_last_error().decode())
    return x, y


def pair_capture(capacity: int):
    """Record the training pair of every converged solve of the current engine (pt_pair_capture)."""
    L = library()
    rc = L.pt_pair_capture(int(capacity))
    if rc:
        raise eng.PtError(rc, L.pt_last_error().decode())


def pair_take(e: eng.Engine, max_pairs: int):
    """The pairs recorded since the last call: (X [n][4][nz][nx], Y [n][nz][nx]) float32."""
    L = library()
    X = np.zeros((max_pairs, 4, e.nz, e.nx), dtype=np.float32)
    Y = np.zeros((max_pairs, e.nz, e.nx), dtype=np.float32)
    n = _c.c_int(0)
    rc = L.pt_pair_take(X.ctypes.data, Y.ctypes.data, int(max_pairs), _c.byref(n))
    if rc:
        raise eng.PtError(rc, L.pt_last_error().decode())
    return X[: n.value], Y[: n.value]


def run_pairs(cfg: PtConfig, st: dict, steps: int, warmup: int = 0):
    """Training pairs of a time-evolved run: `warmup` unrecorded steps, then every converged solve of
    `steps` steps (the top-of-step solve and the three RK-stage solves of each) -> (X, Y).  A solve
    that fails to converge ends the run; the pairs of the solves before it are kept."""
    e = eng.Engine(cfg)
    try:
        e.upload(st)
        try:
            for _ in range(warmup):
                e.solve_psi()
                e.step()
        except eng.PtError:
            return (np.zeros((0, 4, cfg.nz, cfg.nx), np.float32), np.zeros((0, cfg.nz, cfg.nx), np.float32))
        pair_capture(4 * steps + 4)
        try:
            for _ in range(steps):
                e.solve_psi()
                e.step()
        except eng.PtError:
            pass
        X, Y = pair_take(e, 4 * steps + 4)
        pair_capture(0)
    finally:
        e.close()
    return X, Y


def write_shards(X: np.ndarray, Y: np.ndarray, out_dir: str, shard: int = 256, start: int = 0) -> list[str]:
    """Pairs as .npy shards: x_<n>.npy ([m][4][nz][nx]) and y_<n>.npy ([m][nz][nx]), m <= shard."""
    import os

    os.makedirs(out_dir, exist_ok=True)
    names = []
    for q, a in enumerate(range(0, len(X), shard)):
        tag = f"{start + q:05d}"
        np.save(os.path.join(out_dir, f"x_{tag}.npy"), X[a:a + shard])
        np.save(os.path.join(out_dir, f"y_{tag}.npy"), Y[a:a + shard])
        names.append(tag)
    return names


def read_shards(in_dir: str):
    """All shards of a directory written by write_shards, in order."""
    import glob
    import os

    xs = sorted(glob.glob(os.path.join(in_dir, "x_*.npy")))
    X = np.concatenate([np.load(f) for f in xs]) if xs else np.zeros((0,), np.float32)
    Y = np.concatenate([np.load(f.replace(os.sep + "x_", os.sep + "y_")) for f in xs]) if xs else np.zeros((0,), np.float32)
    return X, Y


def guess_info():
    L = library()
    used, rp, rn = _c.c_int(), _c.c_double(), _c.c_double()
    L.pt_unet_guess_info(_c.byref(used), _c.byref(rp), _c.byref(rn))
    return {"used": bool(used.value), "resid_prev": rp.value, "resid_net": rn.value}


def sample_config(rng: np.random.Generator, nx: int, nz: int, tpc: int = 4) -> PtConfig:
    """A thermochemical configuration with Ra_T in [1e5, 1e7] and a temperature viscosity contrast in
    [1e2, 1e5], both log-uniform (the learned-guess workload's sampling, on an nx x nz grid)."""
    c, _ = workload("C4")
    c.nx, c.nz = nx, nz
    c.RaT = float(10.0 ** rng.uniform(5.0, 7.0))
    c.RaC = 0.2 * c.RaT
    c.visT = float(10.0 ** rng.uniform(2.0, 5.0))
    c.visP = 1.0
    c.precision = PT_PREC_FP64
    c.mg_scheme = 1
    c.CFL = 1
    c.grids = max(2, min(6, int(round(math.log2(min(nx, nz) / 8))) + 1))
    c.tolerance = 1e-8
    c.max_cycles = 200
    c.ntr = nx * nz * tpc
    return c


def solver_pairs(rng: np.random.Generator, n: int, nx: int, nz: int, tpc: int = 4):
    """n training pairs from FP64 solves of sampled configurations and seeded states."""
    X = np.zeros((n, 4, nz, nx), dtype=np.float32)
    Y = np.zeros((n, nz, nx), dtype=np.float32)
    for q in range(n):
        cfg = sample_config(rng, nx, nz, tpc)
        st = make_state(cfg, int(rng.integers(1 << 30)), noise=1e-3)
        e = eng.Engine(cfg)
        try:
            e.upload(st)
            e.set_guess_mode(PT_GUESS_ZERO)
            e.solve_psi()
            X[q], Y[q] = training_pair(e)
        finally:
            e.close()
    return X, Y


def train(net: UNet, X: np.ndarray, Y: np.ndarray, epochs: int, batch: int, lr: float = 1e-3, seed: int = 0):
    """Adam over shuffled minibatches; returns the mean loss of each epoch."""
    rng = np.random.default_rng(seed)
    hist = []
    for _ in range(epochs):
        order = rng.permutation(len(X))
        losses = []
        for s in range(0, len(X) - batch + 1, batch):
            idx = order[s:s + batch]
            losses.append(net.train_step(X[idx], Y[idx], lr))
        hist.append(float(np.mean(losses)))
    return hist


def c4_study(out_dir: str, n_train: int = 1000, n_test: int = 200, steps_per_run: int = 10, warmup: int = 2,
             epochs: int = 10, batch: int = 8, lr: float = 1e-3, seed: int = 7, nx: int = 512, nz: int = 256,
             tpc: int = 16, log=print) -> dict:
    """The learned-guess evaluation of the 512x256 configuration.

    Training pairs come from time-evolved FP64 runs of sampled physics (sample_config: Ra_T in
    [1e5, 1e7], viscosity contrast in [1e2, 1e5]; `warmup` unrecorded steps, then every converged
    solve of `steps_per_run` steps) and are written as .npy shards under out_dir/train.  The network
    (4 levels, width 32) is trained on n_train of them.  Held-out: new runs of the same sampling; at
    each top-of-step solve the FP64 solve to 1e-8 is run three times from the same state -- from
    zero, from the previous step's psi (the reference's warm start) and from the network's guess
    (with its fallback to the previous psi after one cycle) -- and a fourth time from the network's
    guess with psi zeroed first (a cold start: the fallback then compares against the zero guess);
    the V-cycles are recorded, with the network's error on psi / max|psi| against the zero
    guess's."""
    import os
    import time

    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    Xs, Ys, runs = [], [], 0
    while sum(len(x) for x in Xs) < n_train:
        if runs > n_train:
            raise RuntimeError("c4_study: too few converging runs for the training pairs")
        cfg = sample_config(rng, nx, nz, tpc)
        st = make_state(cfg, int(rng.integers(1 << 30)), noise=1e-3)
        x, y = run_pairs(cfg, st, steps_per_run, warmup)
        Xs.append(x)
        Ys.append(y)
        runs += 1
    X = np.concatenate(Xs)[:n_train]
    Y = np.concatenate(Ys)[:n_train]
    del Xs, Ys
    shards = write_shards(X, Y, os.path.join(out_dir, "train"))
    t_pairs = time.perf_counter() - t0
    log(f"pairs: {len(X)} from {runs} runs in {t_pairs:.1f} s, {len(shards)} shards")
    net = UNet(nz, nx, max_batch=batch, seed=seed)
    t0 = time.perf_counter()
    hist = train(net, X, Y, epochs, batch, lr, seed)
    t_train = time.perf_counter() - t0
    log(f"training: {epochs} epochs in {t_train:.1f} s, loss {hist[0]:.4g} -> {hist[-1]:.4g}")
    wpath = os.path.join(out_dir, "unet_c4.bin")
    net.save(wpath)
    cyc = {"zero": [], "previous": [], "learned": [], "learned_cold": []}
    used, used_cold, mse_net, mse_zero = [], [], [], []
    test_runs, skipped = 0, 0
    while len(cyc["zero"]) < n_test:
        if test_runs > n_test + 50:
            break
        cfg = sample_config(rng, nx, nz, tpc)
        st = make_state(cfg, int(rng.integers(1 << 30)), noise=1e-3)
        e = eng.Engine(cfg)
        try:
            e.upload(st)
            for _ in range(warmup):
                e.solve_psi()
                e.step()
            for _ in range(steps_per_run):
                if len(cyc["zero"]) >= n_test:
                    break
                prev = e.get(eng.F_SF)
                e.set_guess_mode(PT_GUESS_ZERO)
                cz = e.solve_psi()["cycles"]
                xt, yt = training_pair(e)
                pred = net.forward(xt[None])[0]
                e.set(eng.F_SF, np.zeros_like(prev))  # cold start: the network against zero
                e.set_guess_mode(PT_GUESS_UNET, wpath)
                cc = e.solve_psi()["cycles"]
                uc = guess_info()["used"]
                e.set(eng.F_SF, prev)
                cl = e.solve_psi()["cycles"]
                ul = guess_info()["used"]
                e.set(eng.F_SF, prev)
                e.set_guess_mode(PT_GUESS_PREVIOUS)
                cp = e.solve_psi()["cycles"]
                cyc["zero"].append(cz)
                cyc["learned"].append(cl)
                cyc["learned_cold"].append(cc)
                cyc["previous"].append(cp)
                used.append(ul)
                used_cold.append(uc)
                mse_net.append(float(np.mean((pred - yt) ** 2)))
                mse_zero.append(float(np.mean(yt ** 2)))
                e.step()
        except eng.PtError:
            skipped += 1  # a solve of this run did not converge (the rest of the run is dropped)
        finally:
            e.close()
        test_runs += 1
    net.close()
    out = {"grid": f"{nx}x{nz}", "tracers_per_cell": tpc, "tolerance": 1e-8, "train_pairs": int(len(X)),
           "train_runs": runs, "test_solves": len(cyc["zero"]), "test_runs": test_runs,
           "test_runs_ended_by_a_failed_solve": skipped, "epochs": epochs,
           "batch": batch, "lr": lr, "loss_history": hist, "seconds_pairs": t_pairs, "seconds_training": t_train,
           "cycles_mean": {k: float(np.mean(v)) for k, v in cyc.items()},
           "cycles_median": {k: float(np.median(v)) for k, v in cyc.items()},
           "cycles_max": {k: int(np.max(v)) for k, v in cyc.items()},
           "learned_guess_kept": float(np.mean(used)), "learned_cold_guess_kept": float(np.mean(used_cold)),
           "heldout_mse_network": float(np.mean(mse_net)), "heldout_mse_zero_guess": float(np.mean(mse_zero))}
    with open(os.path.join(out_dir, "c4_study.json"), "w") as fh:
        import json

        json.dump(out, fh, indent=1)
    return out


def profile(nz: int = 256, nx: int = 512, batch: int = 8, reps: int = 5) -> dict:
    """Speed of the network's tensor-core GEMMs: per-layer device time of the forward convolutions
    (CUDA events, pt_unet_profile_forward) with their TFLOP/s, and the host time of whole forward
    passes and training steps on random inputs."""
    import time

    net = UNet(nz, nx, max_batch=batch, seed=1)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((batch, 4, nz, nx)).astype(np.float32)
    Y = (0.1 * rng.standard_normal((batch, nz, nx))).astype(np.float32)
    ms = net.profile_forward(X)
    fl = conv_flops(nz, nx, batch)
    layers = [{"cin": LAYERS[q][0], "cout": LAYERS[q][1], "level": LAYERS[q][2], "ms": float(ms[q]),
               "tflops": float(fl[q] / (ms[q] * 1e-3) / 1e12)} for q in range(len(LAYERS))]
    net.forward(X)
    net.train_step(X, Y, 1e-4)
    t0 = time.perf_counter()
    for _ in range(reps):
        net.forward(X)
    tf = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        net.train_step(X, Y, 1e-4)
    tt = (time.perf_counter() - t0) / reps
    net.close()
    return {"grid": f"{nx}x{nz}", "batch": batch, "layers": layers, "forward_gemm_ms": float(ms.sum()),
            "forward_gemm_tflops": float(sum(fl) / (ms.sum() * 1e-3) / 1e12), "forward_ms": tf * 1e3,
            "train_step_ms": tt * 1e3, "train_step_tflops": 3 * sum(fl) / tt / 1e12}


# (cin, cout, level) of the 14 convolutions, as built by the library (4 levels, width 32)
LAYERS = [(4, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 128, 2), (128, 128, 2), (128, 256, 3),
          (256, 256, 3), (384, 128, 2), (128, 128, 2), (192, 64, 1), (64, 64, 1), (96, 32, 0), (32, 32, 0)]


def conv_flops(nz: int, nx: int, batch: int) -> list[float]:
    """FLOPs of each convolution GEMM of one forward pass (2 per multiply-add)."""
    return [18.0 * ci * co * batch * nz * nx / 4 ** lv for ci, co, lv in LAYERS]


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="learned-guess study at 512x256 (c4_study) or GEMM profile")
    ap.add_argument("out_dir", nargs="?", default=None)
    ap.add_argument("--train", type=int, default=1000)
    ap.add_argument("--test", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--profile", action="store_true", help="time the network's GEMMs instead")
    a = ap.parse_args()
    if a.profile:
        print(json.dumps(profile()))
    else:
        print(json.dumps(c4_study(a.out_dir, n_train=a.train, n_test=a.test, epochs=a.epochs)))

