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
from .config import PT_GUESS_ZERO, PT_PREC_FP64, PtConfig, workload
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
