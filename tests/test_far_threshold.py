"""The sign pass tests a node as far without a square root: in float32,
RN(sqrt(x)) > t holds exactly when x > RD(m^2), m the midpoint between t and
the next float above it (ref_tree.cu, far_tau).  Restated here in numpy
(float32 sqrt is correctly rounded) and checked on random and adversarial
values around every threshold."""
import numpy as np

INF = np.float32(np.inf)


def far_tau(radius, beta):
    t = np.float32(np.float32(radius) * np.float32(beta))
    if t != t:
        return t
    if t < 0:
        return np.float32(-1.0)
    if t == INF:
        return t
    tp = np.nextafter(t, INF)
    if tp == INF:
        return np.float32(3.40282347e38)
    m = (np.float64(t) + np.float64(tp)) * 0.5
    m2 = m * m
    f = np.float32(m2)
    if np.float64(f) > m2:
        f = np.nextafter(f, -INF)
    return f


def test_threshold_matches_sqrt_compare():
    rng = np.random.default_rng(1)
    radii = np.concatenate([10.0 ** rng.uniform(-20, 18, 3000), [0.0, 1e-45, 1.0, 3.0e38]]).astype(np.float32)
    betas = np.array([2.0, 1.5, 3.0, 0.7, 1e-3], np.float32)
    checked = 0
    with np.errstate(over="ignore", invalid="ignore"):
        for r in radii:
            for b in betas:
                t = np.float32(r * b)
                tau = far_tau(r, b)
                # squares of t and its neighbours, and floats around them
                c = np.float32(t) * np.float32(t)
                cands = [c, np.float32(t * np.float32(1.0000001)) ** 2, np.float32(0.0), INF]
                for base in cands[:2]:
                    x = np.float32(base)
                    for _ in range(3):
                        x = np.nextafter(x, -INF)
                    for _ in range(7):
                        cands.append(x)
                        x = np.nextafter(x, INF)
                for x in cands:
                    x = np.float32(x)
                    if not np.isfinite(x) and x != INF:
                        continue
                    assert (np.sqrt(x) > t) == (x > tau), (r, b, x, t, tau)
                    checked += 1
    assert checked > 100000
