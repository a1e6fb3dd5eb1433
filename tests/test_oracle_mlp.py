"""The numpy restatement of the learned far field's network (oracle/mlp_ref.py),
which checks the GPU's gradients, checked itself: with BF16 rounding off its
analytic gradients equal central finite differences of its own loss."""
import numpy as np

from oracle import mlp_ref


def test_restatement_gradients_match_finite_differences():
    rng = np.random.default_rng(5)
    p = rng.normal(0.0, 0.2, size=mlp_ref.NP)
    freq = rng.normal(size=(32, 3)) * 2.0
    centre = np.array([0.1, -0.2, 0.05])
    pts = rng.uniform(-1.0, 1.0, size=(64, 3))
    tgt = rng.uniform(0.0, 1.0, size=64)
    mlp_ref.ROUND = False
    try:
        loss, g = mlp_ref.gradients(p, freq, centre, 0.9, pts, tgt)
        idx = np.concatenate([rng.choice(4096, 12, replace=False), 4096 + rng.choice(64, 4, replace=False),
                              4160 + rng.choice(4096, 12, replace=False), 8256 + rng.choice(64, 4, replace=False),
                              8320 + rng.choice(64, 4, replace=False), [8384]])
        eps = 1e-6
        for i in idx:
            q = p.copy()
            q[i] += eps
            lp, _ = mlp_ref.gradients(q, freq, centre, 0.9, pts, tgt)
            q[i] -= 2 * eps
            lm, _ = mlp_ref.gradients(q, freq, centre, 0.9, pts, tgt)
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])
    finally:
        mlp_ref.ROUND = True
