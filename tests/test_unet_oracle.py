"""The U-Net CPU oracle's backward pass against central finite differences (no GPU)."""
import numpy as np

import oracle.unet_ref as ur


def test_oracle_gradients_match_finite_differences():
    ur.EXACT = True
    try:
        rng = np.random.default_rng(5)
        offs, out_w, out_b, total = ur.layout()
        params = rng.standard_normal(total) * 0.1
        for (wo, bo), spec in zip(offs, ur.SPEC):  # He-scaled weights keep the loss O(1)
            params[wo:bo] *= 10.0 * np.sqrt(2.0 / (9 * spec[3]))
        x = rng.standard_normal((1, 4, 8, 8))
        t = rng.standard_normal((1, 8, 8))
        loss, g = ur.gradients(params, x, t)
        picks = [offs[0][0] + 3, offs[0][1] + 1, offs[2][0] + 50, offs[6][0] + 100, offs[8][0] + 7, offs[12][0] + 11,
                 offs[13][1], out_w + 5, out_b]
        picks += [int(q) for q in rng.integers(0, total, 10)]
        checked = 0
        for q in picks:
            h = 1e-7 * max(1.0, abs(params[q]))
            pp, pm = params.copy(), params.copy()
            pp[q] += h
            pm[q] -= h
            lp, lm = ur.gradients(pp, x, t)[0], ur.gradients(pm, x, t)[0]
            fwd, bwd = (lp - loss) / h, (loss - lm) / h
            if abs(fwd - bwd) > 1e-4 * max(1.0, abs(fwd)):
                continue  # a ReLU changes sign inside [p-h, p+h]: no derivative to compare
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[q]) <= 1e-5 * max(1.0, abs(fd)), (q, fd, g[q])
            checked += 1
        assert checked >= len(picks) - 3
    finally:
        ur.EXACT = False
