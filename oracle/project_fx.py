"""CPU restatement of the mixed-precision tracer->grid projection (test infrastructure only: the
tests compare the GPU kernel against it bit for bit; nothing in the library calls it).

The reference's projection, tracers_to_corners_iC_continuous (composition.f90:942-1087) with the
bilinear shape_func (composition.f90:896-921), sums T*S, C*S and S over the tracers around each
node in FP64 and counts, per node, the tracers whose nearest node (nint of the position) it is.
The mixed-precision path forms the same sums in fixed point, so that they are exact integer sums
whose value does not depend on the order of the tracers:

  * position: u = r / dr (exactly r * 2^p when dr = 2^-p); i0 = floor(u); the fraction truncated
    to 28 bits, fx = floor((u - i0) * 2^28).  A tracer on the right wall (i0 = nx) is placed in
    cell nx-1 with fx = 2^28.  Same in z with ds and nz.
  * nearest node (the reference's nint cell): i0 + (fx >= 2^27), taken before the wall rule.
  * weights: wx = (2^28 - fx, fx) for the nodes i0 and i0+1 (the reference's hat functions; the
    third node of its 3x3 neighbourhood has weight 0), wz likewise;
    S_ab = floor((wx_a * wz_b + 2^27) / 2^28).
  * values: T28 = round(T * 2^28), half away from zero, for |T| < 4;
    TS_ab = floor((T28 * S_ab + 2^27) / 2^28); C likewise.
  * per node: the integer sums of TS, CS and S; Tratio = sum TS / sum S (FP64 division of the
    exactly converted sums) where sum S > 0, else the node keeps its previous value.
"""

from __future__ import annotations

import numpy as np

ONE = 1 << 28
HALF = 1 << 27


def floor_fix(x: np.ndarray, h: float):
    """(floor(x / h), 28-bit truncated fraction) as int64 arrays."""
    u = x / h
    i0 = np.floor(u)
    f = np.floor((u - i0) * float(ONE))  # u - i0 and the power-of-two scaling are exact
    return i0.astype(np.int64), f.astype(np.int64)


def fix28(v: np.ndarray) -> np.ndarray:
    """round(v * 2^28), half away from zero (|v| < 4)."""
    if np.any(~(np.abs(v) < 4.0)):
        raise ValueError("fixed-point projection: |value| must stay below 4")
    a = np.abs(v) * float(ONE)
    fl = np.floor(a)
    q = (fl + (a - fl >= 0.5)).astype(np.int64)
    return np.where(v < 0, -q, q)


def project_fx(nx: int, nz: int, aspect: float, r, s, T, C=None):
    """Integer node sums of the projection: (TS, CS, S, count), each (nz+1, nx+1) int64, node
    (i, k) at [k, i]; CS is zero when C is None."""
    r, s, T = (np.asarray(a, dtype=np.float64) for a in (r, s, T))
    if np.any((r < 0) | (r > aspect) | (s < 0) | (s > 1.0)):
        raise ValueError("Tracer advected outside of domain")
    dr, ds = aspect / nx, 1.0 / nz
    i0, fx = floor_fix(r, dr)
    k0, fz = floor_fix(s, ds)
    ni = i0 + (fx >= HALF)
    nk = k0 + (fz >= HALF)
    wall = i0 >= nx
    i0, fx = np.where(wall, nx - 1, i0), np.where(wall, ONE, fx)
    wall = k0 >= nz
    k0, fz = np.where(wall, nz - 1, k0), np.where(wall, ONE, fz)
    nn = (nx + 1) * (nz + 1)
    t28 = fix28(T)
    c28 = fix28(np.asarray(C, dtype=np.float64)) if C is not None else None
    wx = (ONE - fx, fx)
    wz = (ONE - fz, fz)
    sums = {q: np.zeros(nn, dtype=np.int64) for q in ("T", "C", "S")}
    for b in (0, 1):
        for a in (0, 1):
            node = (i0 + a) + (nx + 1) * (k0 + b)
            S = (wx[a] * wz[b] + HALF) >> 28
            # integer-valued float64 weights: every partial sum stays below 2^53, so exact
            sums["S"] += np.bincount(node, weights=S.astype(np.float64), minlength=nn).astype(np.int64)
            sums["T"] += np.bincount(node, weights=((t28 * S + HALF) >> 28).astype(np.float64),
                                     minlength=nn).astype(np.int64)
            if c28 is not None:
                sums["C"] += np.bincount(node, weights=((c28 * S + HALF) >> 28).astype(np.float64),
                                         minlength=nn).astype(np.int64)
    count = np.bincount(ni + (nx + 1) * nk, minlength=nn).astype(np.int64)
    shape = (nz + 1, nx + 1)
    return sums["T"].reshape(shape), sums["C"].reshape(shape), sums["S"].reshape(shape), count.reshape(shape)


def ratios(TS, CS, S, prev_T, prev_C=None):
    """Tratio (and Cnew) on the nodes: the sums' ratio where S > 0, else the previous value."""
    Sd = S.astype(np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        Tr = np.where(S > 0, TS.astype(np.float64) / Sd, prev_T)
        Cr = None if prev_C is None else np.where(S > 0, CS.astype(np.float64) / Sd, prev_C)
    return Tr, Cr
