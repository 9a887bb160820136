"""The schedule of the direct solve's substitution kernel (k_direct_solve, csrc/pt_direct.cu),
restated in Python and checked on the CPU against the oracle's DGBTRS restatement bit for bit.

The kernel runs the column recurrence in one CTA: element i of b belongs to thread (i - 1) mod
NT, which alone writes it; in a column step every thread applies the column to its own elements
and the owner of the value the next step needs first publishes it (the pivot row's b in the
forward step, x = b / U_jj in the back substitution), so a step has one barrier.  b stays in
global memory; the elements a step touches live in a window of W slots, loaded by their owner two
steps ahead (into a register, then into the slot) and written back in the step they become
final.  The band columns arrive through a ring of AHEAD + 1 slots, AHEAD columns ahead, copied in
16-byte pairs from the even index at or below each column's first entry.

Here the threads of a step run in a random order, window and ring slots hold NaN until filled (a
read of a stale or missing value shows up in the result), the global copy of b is poisoned ahead
of the forward write-backs, and every column copy is checked against the band array's bounds and
the slot length.
"""
import random

import numpy as np
import pytest

from oracle.ptref import band_lu, band_solve

NT = 256


def window_size(kl, ku):
    w = 64
    while w < kl + ku + 4:
        w *= 2
    return w


def schedule(ab_f, ipiv, bvec, n, kl, ku, ahead, rng):
    ldab, kd, kp1, k = 2 * kl + ku + 1, kl + ku + 1, kl + ku + 1, kl + ku
    ab = ab_f.ravel(order="F")  # AB(r, c) = ab[(r - 1) + (c - 1) ldab]
    ring_n, slot_len = ahead + 1, (kl + ku + 3) & ~1
    ring = np.full((ring_n, slot_len), np.nan)
    piv = [None] * ring_n
    W = window_size(kl, ku)
    win = np.full(W, np.nan)
    bg = bvec.copy()
    pub = [None] * 4
    pend = {}  # thread -> (element, value) loaded for the window, stored the next step

    def B(i):
        return win[(i - 1) % W]

    def setB(i, v):
        win[(i - 1) % W] = v

    def copy(slot, s0, length, live):
        ring[slot, :] = np.nan
        if live:
            a0 = s0 & ~1
            pairs = ((s0 - a0) + length + 1) >> 1
            assert a0 + 2 * pairs <= ab.size and 2 * pairs <= slot_len
            ring[slot, :2 * pairs] = ab[a0:a0 + 2 * pairs]

    def owner(i):
        return (i - 1) % NT

    def first_owned(a, t):
        return a + (t - (a - 1)) % NT

    def threads():
        order = list(range(NT))
        rng.shuffle(order)
        return order

    def store_pending(t):
        if t in pend:
            i, v = pend.pop(t)
            assert not np.isnan(v)
            setB(i, v)

    def issue_fwd(c):
        if c <= n - 1:
            piv[c % ring_n] = int(ipiv[c - 1])
        copy(c % ring_n, kd + (c - 1) * ldab, kl, c <= n - 1)

    for c in range(1, ahead + 1):
        issue_fwd(c)
    for i in range(1, min(n, kl + 1) + 1):
        setB(i, bg[i - 1])
    if kl + 2 <= n:
        pend[owner(kl + 2)] = (kl + 2, bg[kl + 1])
    bg[kl + 2:] = np.nan  # entries the forward pass reads only through its window loads
    pub[1], pub[3] = B(piv[1 % ring_n]), B(1)
    rhs = bvec.copy()
    for j in range(1, n):
        sl, off = j % ring_n, (kd + (j - 1) * ldab) & 1
        l, T, S = piv[sl], pub[j & 1], pub[2 + (j & 1)]
        lm = min(kl, n - j)
        nxt = {}
        for t in threads():
            store_pending(t)
            if owner(j) == t:
                setB(j, T)
                bg[j - 1] = T
            if l != j and owner(l) == t:
                setB(l, S)
            temp = -T
            for i in range(first_owned(j + 1, t), j + lm + 1, NT):
                setB(i, B(i) + ring[sl, off + i - j - 1] * temp)
            if j + 1 <= n - 1:
                l1 = piv[(j + 1) % ring_n]
                if owner(l1) == t:
                    nxt[(j + 1) & 1] = B(l1)
                if owner(j + 1) == t:
                    nxt[2 + ((j + 1) & 1)] = B(j + 1)
            f = j + kl + 2
            if f <= n and owner(f) == t:
                pend[t] = (f, rhs[f - 1])  # not yet written back: the right-hand side itself
        for q, v in nxt.items():
            pub[q] = v
        issue_fwd(j + ahead)
    bg[n - 1] = B(n)
    assert not pend and not np.isnan(bg).any()

    def issue_bwd(m):
        c = n - m + 1
        copy(m % ring_n, (c - 1) * ldab, kp1, c >= 1)

    def ucol(m, r):
        c = n - m + 1
        return ring[m % ring_n, (((c - 1) * ldab) & 1) + r]

    for m in range(1, ahead + 1):
        issue_bwd(m)
    win[:] = np.nan
    for i in range(max(1, n - k), n + 1):
        setB(i, bg[i - 1])
    if n - k - 1 >= 1:
        pend[owner(n - k - 1)] = (n - k - 1, bg[n - k - 2])
    x = B(n) / ucol(1, kp1 - 1)
    setB(n, x)
    bg[n - 1] = x
    pub[1] = x
    for m in range(1, n + 1):
        j = n - m + 1
        x, lo, i0 = pub[m & 1], kp1 - j, max(1, j - k)
        for t in threads():
            store_pending(t)
            for i in range(first_owned(i0, t), j, NT):
                setB(i, B(i) - x * ucol(m, lo + i - 1))
            if j >= 2 and owner(j - 1) == t:
                x1 = B(j - 1) / ucol(m + 1, kp1 - 1)
                setB(j - 1, x1)
                bg[j - 2] = x1
                pub[(m + 1) & 1] = x1
            f = j - k - 2
            if f >= 1 and owner(f) == t:
                pend[t] = (f, bg[f - 1])
        issue_bwd(m + ahead)
    return bg


def _band(n, kl, ku, rng):
    ldab = 2 * kl + ku + 1
    A = np.zeros((ldab, n))
    for c in range(n):
        for r in range(max(0, c - ku), min(n, c + kl + 1)):
            A[kl + ku + r - c, c] = rng.standard_normal() + (4.0 if r == c and rng.random() < 0.6 else 0.0)
    return A


@pytest.mark.parametrize("ahead", [8, 2])
@pytest.mark.parametrize("n,kl,ku", [(60, 3, 4), (300, 12, 7), (600, 1, 1), (400, 37, 2), (500, 40, 40), (500, 30, 30)])
def test_substitution_schedule_matches_dgbtrs_bit_for_bit(n, kl, ku, ahead):
    rng = np.random.default_rng(n + kl + ku)
    ab, ipiv, info = band_lu(_band(n, kl, ku, rng).copy(order="F"), n, kl, ku)
    assert info == 0 and np.any(ipiv != np.arange(1, n + 1))  # rows were exchanged
    bvec = rng.standard_normal(n)
    bvec[::7] = 0.0  # zeros and their signs propagate too
    ref = band_solve(ab, ipiv, bvec, n, kl, ku)
    got = schedule(np.asfortranarray(ab), ipiv, bvec, n, kl, ku, ahead, random.Random(n))
    assert np.array_equal(ref.view(np.int64), got.view(np.int64))
