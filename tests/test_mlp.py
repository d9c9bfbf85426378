"""The learned-guess network's CPU restatement: BF16 rounding and the FP64
gradient against central finite differences."""
import numpy as np

import mlp_oracle as mo


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, -2.5, 0.0, 3.0e38])
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0            # tie rounds to even
    assert r[2] == 1.0 + 2.0 ** -7                # above the tie rounds up
    assert r[3] == -2.5 and r[4] == 0.0
    assert abs(r[5] - 3.0e38) / 3.0e38 < 2.0 ** -8


def test_fp64_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(0.0, 0.3, mo.NPARAM)
    x = rng.uniform(-1, 1, (16, 8))
    x[:, 4:] = np.eye(4)[rng.integers(0, 4, 16)]
    lab = rng.normal(0.0, 1.0, (16, 2))
    loss, g = mo.loss_and_gradients(p, x, lab, bf=False)
    h = 1e-6
    idx = rng.choice(mo.NPARAM, 60, replace=False)
    for i in idx:
        e = np.zeros(mo.NPARAM)
        e[i] = h
        lp, _ = mo.loss_and_gradients(p + e, x, lab, bf=False)
        lm, _ = mo.loss_and_gradients(p - e, x, lab, bf=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])
