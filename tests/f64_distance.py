"""Float64 point-triangle distances (Ericson's Voronoi-region closest point,
the method of triangle3.rs:317-382) for measuring the float32 path's error."""
import numpy as np


def point_triangle_dist_f64(p, a, b, c):
    p, a, b, c = (np.asarray(x, np.float64) for x in (p, a, b, c))
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = (ab * ap).sum(1), (ac * ap).sum(1)
    bp = p - b
    d3, d4 = (ab * bp).sum(1), (ac * bp).sum(1)
    cp = p - c
    d5, d6 = (ab * cp).sum(1), (ac * cp).sum(1)
    vc = d1 * d4 - d3 * d2
    vb = d5 * d2 - d1 * d6
    va = d3 * d6 - d5 * d4
    q = np.empty_like(p)
    done = np.zeros(len(p), bool)

    def put(mask, val):
        m = mask & ~done
        q[m] = val[m] if val.ndim == 2 else val
        done[m] = True

    put((d1 <= 0) & (d2 <= 0), a)
    put((d3 >= 0) & (d4 <= d3), b)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = d1 / (d1 - d3)
        put((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + ab * v[:, None])
        put((d6 >= 0) & (d5 <= d6), c)
        w = d2 / (d2 - d6)
        put((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + ac * w[:, None])
        d43, d56 = d4 - d3, d5 - d6
        w2 = d43 / (d43 + d56)
        put((va <= 0) & (d43 >= 0) & (d56 >= 0), b + (c - b) * w2[:, None])
        den = 1.0 / (va + vb + vc)
        put(np.ones(len(p), bool), a + ab * (vb * den)[:, None] + ac * (vc * den)[:, None])
    return np.sqrt(((q - p) ** 2).sum(1))


def min_distance_f64(vox, h, sub, box):
    """Float64 minimum over the reference's candidates (sub-triangles whose
    widened box holds the voxel) for each voxel index in `vox` (n, 3)."""
    out = np.full(len(vox), np.inf)
    grid = vox.astype(np.float32) * np.float32(h)  # the float32 grid point, then exact arithmetic
    for i, g in enumerate(vox):
        m = np.all((box[:, :3] <= g) & (g <= box[:, 3:]), axis=1)
        if not m.any():
            continue
        t = sub[m]
        d = point_triangle_dist_f64(np.repeat(grid[i:i + 1], len(t), 0), t[:, 0], t[:, 1], t[:, 2])
        out[i] = d.min()
    return out
