"""Seeded synthetic inputs: the contents of the reference's restart files for a workload.

The reference restarts from two unformatted files (print_restart, main.f90:457-496): Trestart
with xg, zg, T, Cnew, SF and restart_tracers with rtr, str, Ctr, Ttr.  ``make_state`` builds
those arrays for a configuration so that the CPU oracle and the GPU engine start from identical
bits; ``write_restart``/``read_restart`` store them in the Fortran sequential-unformatted layout
(4-byte record markers; gfortran splits records above 2 GiB into sub-records with negative
continuation markers).

Initial conditions (no public dataset is involved; the workloads define them):
  T   = 1 - z + 0.01 cos(pi x / aspect) sin(pi z)  [+ uniform noise of amplitude ``noise``]
  C   = 1 where z < layer (dense bottom layer), else 0
  psi = 0
  tracers: exactly ntr/(nx*nz) per grid cell, laid out as an a x b sub-lattice of the cell with
  each tracer at a uniform-random position inside its sub-cell (jittered stratified sampling,
  seeded), carrying T and C of their position.  Cells are visited in
  the reference's seeding order (i outer, k inner), so tracer IDs are spatially grouped as in
  initialize_tracers (composition.f90:807-846).
"""

from __future__ import annotations

import os
import struct

import numpy as np

from .config import PtConfig


def grid_coords(cfg: PtConfig):
    """xg(-6:nx+6), zg(-6:nz+6) of the uniform grid (grid.f90:46-54, 105-116)."""
    nx, nz, a = cfg.nx, cfg.nz, cfg.aspect
    dr, ds = a / nx, 1.0 / nz
    xg = np.zeros(nx + 13)
    zg = np.zeros(nz + 13)
    xg[6:nx + 7] = dr * np.arange(nx + 1)
    zg[6:nz + 7] = ds * np.arange(nz + 1)
    for i in range(1, 7):
        xg[6 - i] = -xg[6 + i]
        xg[6 + nx + i] = a - xg[6 + nx - i] + a
        zg[6 - i] = -zg[6 + i]
        zg[6 + nz + i] = 1.0 - zg[6 + nz - i] + 1.0
    xg[6], zg[6], xg[6 + nx], zg[6 + nz] = 0.0, 0.0, a, 1.0
    return xg, zg


def initial_T(x, z, aspect, rng=None, noise=0.0):
    t = (1.0 - z) + 0.01 * np.cos(np.pi * x / aspect) * np.sin(np.pi * z)
    if noise > 0.0 and rng is not None:
        t = t + noise * (2.0 * rng.random(np.shape(t)) - 1.0)
    return t


def make_state(cfg: PtConfig, seed: int, noise: float = 0.0, layer: float = 0.2) -> dict:
    nx, nz, a = cfg.nx, cfg.nz, cfg.aspect
    rng = np.random.default_rng(seed)
    xg, zg = grid_coords(cfg)
    X, Z = np.meshgrid(xg[3:nx + 10], zg[3:nz + 10])  # (-3:nx+3) x (-3:nz+3)
    T = initial_T(X, Z, a, rng, noise)
    T[:, :] = np.where((Z < 0) | (Z > 1), 0.0, T)
    X5, Z5 = np.meshgrid(xg[1:nx + 12], zg[1:nz + 12])  # (-5:nx+5)
    C = np.where(Z5 < layer, 1.0, 0.0) if cfg.comp else np.zeros_like(X5)
    SF = np.zeros((nz + 7, nx + 7))
    n = int(cfg.ntr)
    per = n // (nx * nz)
    if per * nx * nz != n:
        raise ValueError("ntr must be a multiple of nx*nz")
    sa = int(np.floor(np.sqrt(per)))
    while per % sa:
        sa -= 1
    sb = per // sa  # sub-lattice sa (x) by sb (z)
    ci = np.repeat(np.arange(nx), nz * per)
    ck = np.tile(np.repeat(np.arange(nz), per), nx)
    sub = np.tile(np.arange(per), nx * nz)
    sx, sz = sub % sa, sub // sa
    r = (ci + (sx + rng.random(n)) / sa) * (a / nx)
    s = (ck + (sz + rng.random(n)) / sb) * (1.0 / nz)
    Ttr = initial_T(r, s, a, rng, noise)
    Ctr = np.where(s < layer, 1.0, 0.0) if cfg.comp else np.zeros(n)
    return dict(xg=xg, zg=zg, T=T, Cnew=C, SF=SF, rtr=r, str=s, Ctr=Ctr, Ttr=Ttr)


_MAXREC = 2**31 - 9  # gfortran sub-record payload limit


def _write_record(fh, payload: bytes):
    n = len(payload)
    if n <= _MAXREC:
        fh.write(struct.pack("<i", n))
        fh.write(payload)
        fh.write(struct.pack("<i", n))
        return
    off = 0
    first = True
    while off < n:
        chunk = payload[off:off + _MAXREC]
        last = off + len(chunk) >= n
        head = len(chunk) if (first and last) else (-len(chunk) if not last else len(chunk))
        tail = -len(chunk) if not first else len(chunk)
        if first and not last:
            head, tail = -len(chunk), len(chunk)
        elif not first and not last:
            head, tail = -len(chunk), -len(chunk)
        elif not first and last:
            head, tail = len(chunk), -len(chunk)
        fh.write(struct.pack("<i", head))
        fh.write(chunk)
        fh.write(struct.pack("<i", tail))
        off += len(chunk)
        first = False


def _read_record(fh) -> bytes:
    parts = []
    while True:
        (head,) = struct.unpack("<i", fh.read(4))
        data = fh.read(abs(head))
        fh.read(4)
        parts.append(data)
        if head >= 0:
            break
    return b"".join(parts)


def write_restart(directory: str, state: dict, comp: int = 1):
    """Trestart (xg,zg,T,[Cnew],SF) and restart_tracers (rtr,str,[Ctr],Ttr), main.f90:462-494."""
    grid = [state["xg"], state["zg"], state["T"]] + ([state["Cnew"]] if comp else []) + [state["SF"]]
    with open(os.path.join(directory, "Trestart"), "wb") as fh:
        _write_record(fh, b"".join(np.ascontiguousarray(x, dtype="<f8").tobytes() for x in grid))
    trc = [state["rtr"], state["str"]] + ([state["Ctr"]] if comp else []) + [state["Ttr"]]
    with open(os.path.join(directory, "restart_tracers"), "wb") as fh:
        _write_record(fh, b"".join(np.ascontiguousarray(x, dtype="<f8").tobytes() for x in trc))


def read_restart(directory: str, cfg: PtConfig) -> dict:
    nx, nz, comp, n = cfg.nx, cfg.nz, cfg.comp, int(cfg.ntr)
    with open(os.path.join(directory, "Trestart"), "rb") as fh:
        buf = np.frombuffer(_read_record(fh), dtype="<f8")
    sizes = [("xg", nx + 13), ("zg", nz + 13), ("T", (nz + 7) * (nx + 7))]
    if comp:
        sizes.append(("Cnew", (nz + 11) * (nx + 11)))
    sizes.append(("SF", (nz + 7) * (nx + 7)))
    out, off = {}, 0
    for name, m in sizes:
        out[name] = buf[off:off + m].copy()
        off += m
    out["T"] = out["T"].reshape(nz + 7, nx + 7)
    out["SF"] = out["SF"].reshape(nz + 7, nx + 7)
    out["Cnew"] = out["Cnew"].reshape(nz + 11, nx + 11) if comp else np.zeros((nz + 11, nx + 11))
    with open(os.path.join(directory, "restart_tracers"), "rb") as fh:
        raw = _read_record(fh)
    if comp and getattr(cfg, "discrete_types", 0):  # rtr, str, Ttype (integer*4), Ttr
        out["rtr"] = np.frombuffer(raw, dtype="<f8", count=n).copy()
        out["str"] = np.frombuffer(raw, dtype="<f8", count=n, offset=8 * n).copy()
        out["Ttype"] = np.frombuffer(raw, dtype="<i4", count=n, offset=16 * n).copy()
        out["Ttr"] = np.frombuffer(raw, dtype="<f8", count=n, offset=20 * n).copy()
        out["Ctr"] = out["Ttype"].astype(np.float64)
        return out
    buf = np.frombuffer(raw, dtype="<f8")
    names = ["rtr", "str"] + (["Ctr"] if comp else []) + ["Ttr"]
    for j, name in enumerate(names):
        out[name] = buf[j * n:(j + 1) * n].copy()
    if not comp:
        out["Ctr"] = np.zeros(n)
    return out
