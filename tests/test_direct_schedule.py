"""The schedule of the direct solve's substitution kernel (k_direct_solve, csrc/pt_direct.cu),
restated in Python and checked on the CPU against the oracle's DGBTRS restatement bit for bit.

The kernel runs the column recurrence in one CTA: element i of b belongs to thread (i - 1) mod
NT, which alone writes it; in a column step every thread applies the column to its own elements
and the owner of the value the next step needs first publishes it (the pivot row's b in the
forward step, x = b / U_jj in the back substitution), so a step has one barrier.  The band
columns arrive through a ring of AHEAD + 1 slots, AHEAD columns ahead, copied in 16-byte pairs
from the even index at or below each column's first entry.

Here the threads of a step run in a random order, slots not yet filled hold NaN (a read of a
stale or missing column shows up in the result), and every copy is checked against the band
array's bounds and the slot length.
"""
import random

import numpy as np
import pytest

from oracle.ptref import band_lu, band_solve

NT = 256


def schedule(ab_f, ipiv, bvec, n, kl, ku, ahead, rng):
    ldab, kd, kp1, k = 2 * kl + ku + 1, kl + ku + 1, kl + ku + 1, kl + ku
    ab = ab_f.ravel(order="F")  # AB(r, c) = ab[(r - 1) + (c - 1) ldab]
    ring_n, slot_len = ahead + 1, (kl + ku + 3) & ~1
    ring = np.full((ring_n, slot_len), np.nan)
    piv = [None] * ring_n
    b = bvec.copy()
    pub = [None] * 4

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

    def issue_fwd(c):
        if c <= n - 1:
            piv[c % ring_n] = int(ipiv[c - 1])
        copy(c % ring_n, kd + (c - 1) * ldab, kl, c <= n - 1)

    for c in range(1, ahead + 1):
        issue_fwd(c)
    pub[1], pub[3] = b[piv[1 % ring_n] - 1], b[0]
    for j in range(1, n):
        sl, off = j % ring_n, (kd + (j - 1) * ldab) & 1
        l, T, S = piv[sl], pub[j & 1], pub[2 + (j & 1)]
        lm = min(kl, n - j)
        nxt = {}
        threads = list(range(NT))
        rng.shuffle(threads)
        for t in threads:
            if owner(j) == t:
                b[j - 1] = T
            if l != j and owner(l) == t:
                b[l - 1] = S
            temp = -T
            for i in range(first_owned(j + 1, t), j + lm + 1, NT):
                b[i - 1] = b[i - 1] + ring[sl, off + i - j - 1] * temp
            if j + 1 <= n - 1:
                l1 = piv[(j + 1) % ring_n]
                if owner(l1) == t:
                    nxt[(j + 1) & 1] = b[l1 - 1]
                if owner(j + 1) == t:
                    nxt[2 + ((j + 1) & 1)] = b[j]
        for q, v in nxt.items():
            pub[q] = v
        issue_fwd(j + ahead)

    def issue_bwd(m):
        c = n - m + 1
        copy(m % ring_n, (c - 1) * ldab, kp1, c >= 1)

    def ucol(m, r):
        c = n - m + 1
        return ring[m % ring_n, (((c - 1) * ldab) & 1) + r]

    for m in range(1, ahead + 1):
        issue_bwd(m)
    b[n - 1] = b[n - 1] / ucol(1, kp1 - 1)
    pub[1] = b[n - 1]
    for m in range(1, n + 1):
        j = n - m + 1
        x, lo, i0 = pub[m & 1], kp1 - j, max(1, j - k)
        threads = list(range(NT))
        rng.shuffle(threads)
        for t in threads:
            for i in range(first_owned(i0, t), j, NT):
                b[i - 1] = b[i - 1] - x * ucol(m, lo + i - 1)
            if j >= 2 and owner(j - 1) == t:
                b[j - 2] = b[j - 2] / ucol(m + 1, kp1 - 1)
                pub[(m + 1) & 1] = b[j - 2]
        issue_bwd(m + ahead)
    return b


def _band(n, kl, ku, rng):
    ldab = 2 * kl + ku + 1
    A = np.zeros((ldab, n))
    for c in range(n):
        for r in range(max(0, c - ku), min(n, c + kl + 1)):
            A[kl + ku + r - c, c] = rng.standard_normal() + (4.0 if r == c and rng.random() < 0.6 else 0.0)
    return A


@pytest.mark.parametrize("ahead", [8, 2])
@pytest.mark.parametrize("n,kl,ku", [(60, 3, 4), (300, 12, 7), (600, 1, 1), (400, 37, 2), (500, 40, 40)])
def test_substitution_schedule_matches_dgbtrs_bit_for_bit(n, kl, ku, ahead):
    rng = np.random.default_rng(n + kl + ku)
    ab, ipiv, info = band_lu(_band(n, kl, ku, rng).copy(order="F"), n, kl, ku)
    assert info == 0 and np.any(ipiv != np.arange(1, n + 1))  # rows were exchanged
    bvec = rng.standard_normal(n)
    bvec[::7] = 0.0  # zeros and their signs propagate too
    ref = band_solve(ab, ipiv, bvec, n, kl, ku)
    got = schedule(np.asfortranarray(ab), ipiv, bvec, n, kl, ku, ahead, random.Random(n))
    assert np.array_equal(ref.view(np.int64), got.view(np.int64))
