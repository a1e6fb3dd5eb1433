"""The pair culling of the distance pass (m2v.cu: cull_coeffs, the column
test in k_brick_distance) checked as a property, on the CPU, in float32 with
the GPU's operation order: whenever the test drops a (voxel, sub-triangle)
pair against a running minimum `cur`, the pair's float32 distance by the
reference's closest-point formula (triangle3.rs:317-382, no fused
multiply-adds) is not below `cur`, so dropping it cannot change the
minimum.  Triangles of every shape (well-shaped, needles, near-collinear
slivers, tiny, large, far from the origin) and voxels anywhere in their
widened boxes, most of them placed where the test is tight."""
import numpy as np

F = np.float32
U = F(5.9604645e-8)
INF = F(np.inf)
CULL_SCALE = F(1.0) - F(2.0 ** -20)


def dot3(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def cross3(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1], a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], axis=-1)


def closest_dist2(a, b, c, p):
    """Float32 |closest(p) - p|^2, Ericson's Voronoi regions in the
    reference's operation order (vectorised; every branch computed, the
    first region whose test holds selected)."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = dot3(ab, ap), dot3(ac, ap)
    bp = p - b
    d3, d4 = dot3(ab, bp), dot3(ac, bp)
    vc = d1 * d4 - d3 * d2
    cp = p - c
    d5, d6 = dot3(ab, cp), dot3(ac, cp)
    vb = d5 * d2 - d1 * d6
    va = d3 * d6 - d5 * d4
    d43, d56 = d4 - d3, d5 - d6
    with np.errstate(all="ignore"):
        v_ab = d1 / (d1 - d3)
        w_ac = d2 / (d2 - d6)
        w_bc = d43 / (d43 + d56)
        denom = F(1.0) / ((va + vb) + vc)
        v_f, w_f = vb * denom, vc * denom
        q_face = (a + ab * v_f[..., None]) + ac * w_f[..., None]
        q = q_face
        sel = lambda m, val: np.where(m[..., None], val, q)
        q = sel((va <= 0) & (d43 >= 0) & (d56 >= 0), b + (c - b) * w_bc[..., None])
        q = sel((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + ac * w_ac[..., None])
        q = sel((d6 >= 0) & (d5 <= d6), c)
        q = sel((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + ab * v_ab[..., None])
        q = sel((d3 >= 0) & (d4 <= d3), b)
        q = sel((d1 <= 0) & (d2 <= 0), a)
        d = q - p
        return dot3(d, d)


def cull_coeffs(a, b, c, R, M):
    ab, ac, cb = b - a, c - a, c - b
    e2 = np.maximum(dot3(ab, ab), np.maximum(dot3(ac, ac), dot3(cb, cb)))
    e = np.sqrt(e2)
    n = cross3(ab, ac)
    a2sq = dot3(n, n)
    with np.errstate(all="ignore"):
        cc = F(1024.0) * U * (e2 * e / a2sq)
        e0 = F(2.0) * cc * e2 + F(19.0) * U * (R + e) + F(16.0) * U * e + F(4.0) * U * M
        ok = (cc * R * R <= e) & (cc * (R + e) <= F(0.25)) & \
             (F(132.0) * cc * (F(2.0) * cc * R * R + e0) <= F(0.5)) & (e0 < INF)
    return np.where(ok, F(2.0) * cc, INF).astype(F), np.where(ok, e0, F(0.0)).astype(F)


def fmaf(x, y, z):
    """Fused multiply-add of float32 operands: the float64 product is exact,
    the float64 sum then rounds to float32 (a double rounding that can differ
    from a true fma by one ulp in rare ties)."""
    with np.errstate(all="ignore"):
        return (x.astype(np.float64) * y.astype(np.float64) + z.astype(np.float64)).astype(F)


def triangles(rng, n):
    """Mixed shapes: regular, needles, slivers, tiny, large; far from the origin."""
    centre = rng.uniform(-40, 40, size=(n, 1, 3))
    kind = rng.integers(0, 5, size=n)
    scale = np.choose(kind, [1.0, 1.0, 1.0, 0.02, 6.0])[:, None, None] * 0.004
    t = rng.normal(size=(n, 3, 3))
    needle = kind == 1
    t[needle, 1] = t[needle, 0] + rng.normal(size=(needle.sum(), 3)) * 1e-4
    sliver = kind == 2
    lam = rng.uniform(0.1, 0.9, size=(sliver.sum(), 1))
    t[sliver, 2] = t[sliver, 0] + lam * (t[sliver, 1] - t[sliver, 0]) + \
        rng.normal(size=(sliver.sum(), 3)) * 10.0 ** rng.uniform(-6, -2, size=(sliver.sum(), 1))
    return (centre + scale * t).astype(F)


def test_culled_pairs_never_lower_the_minimum():
    rng = np.random.default_rng(123)
    h = F(0.002)
    inv_h = F(1.0) / h
    band = 3
    checked = culled_ever = tight = 0
    for _ in range(8):
        n = 150_000
        tri = triangles(rng, n)
        a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
        mn, mx = np.minimum(np.minimum(a, b), c), np.maximum(np.maximum(a, b), c)
        lo = np.floor(mn * inv_h).astype(np.int64) - band
        hi = np.ceil(mx * inv_h).astype(np.int64) + band
        flat = np.any(hi == lo, axis=1)
        lo[flat] -= 1
        hi[flat] += 1
        ext = (hi - lo).astype(F)
        R = h * (np.sqrt(dot3(ext, ext)) + F(2.0))
        gm = h * (np.maximum(np.abs(lo), np.abs(hi)).max(axis=1) + 1).astype(F)
        M = np.maximum(gm, np.abs(tri).reshape(n, 9).max(axis=1))
        c2, e0 = cull_coeffs(a, b, c, R.astype(F), M.astype(F))
        # a voxel of the widened box: biased towards the triangle's interior
        # projection and its edges, where the face formula and region
        # boundaries are exercised
        u = rng.random((n, 3)) ** 2
        vox = lo + np.floor(u * (hi - lo + 1)).astype(np.int64)
        vox = np.minimum(vox, hi)
        g = (vox.astype(F) * h).astype(F)
        d2 = closest_dist2(a, b, c, g)
        dx = np.maximum(np.maximum(mn - g, g - mx), F(0.0))
        sq = (dx * dx) * CULL_SCALE
        lb = sq[:, 0] + (sq[:, 1] + sq[:, 2])  # the kernel's order: dx' + (dy' + dz')
        tt = fmaf(c2, lb, e0)
        extra = F(33.0) * (tt * tt)
        # the largest cur the test still culls against: lb > fma(cur, 33/32, extra)
        with np.errstate(all="ignore"):
            cur = ((lb.astype(np.float64) - extra.astype(np.float64)) / 1.03125).astype(F)
            for _ in range(4):  # step down until the float32 test culls
                bad = ~(lb > fmaf(cur, np.full_like(cur, F(1.03125)), extra))
                cur = np.where(bad, np.nextafter(cur, F(-np.inf)), cur)
        cull = np.isfinite(c2) & (cur > 0) & (lb > fmaf(cur, np.full_like(cur, F(1.03125)), extra))
        ok = ~cull | ~np.isfinite(d2) | (d2 >= cur)
        assert ok.all(), (np.flatnonzero(~ok)[:5], d2[~ok][:5], cur[~ok][:5])
        checked += n
        culled_ever += int(cull.sum())
        tight += int((cull & (d2 < F(1.25) * cur)).sum())
    # the property is exercised, and on pairs where the margin is thin
    assert culled_ever > 0.25 * checked and tight > 0.01 * checked, (culled_ever, tight, checked)


def test_cull_test_is_monotone_in_the_bound():
    """cull_coeffs keeps a sub-triangle eligible only while 132 c (2 c R^2 +
    E0) <= 1/2, which makes lb - 33 (c2 lb + E0)^2 grow with lb over the
    widened box: a pair culled at a bound lb is culled at every larger bound
    against the same running minimum.  Checked in float32 with the kernel's
    operations over random eligible sub-triangles, bounds in [0, R^2] and
    minima at the smaller bound's threshold."""
    rng = np.random.default_rng(11)
    h = F(0.002)
    inv_h = F(1.0) / h
    n = 400_000
    tri = triangles(rng, n)
    a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
    mn, mx = np.minimum(np.minimum(a, b), c), np.maximum(np.maximum(a, b), c)
    lo = np.floor(mn * inv_h).astype(np.int64) - 3
    hi = np.ceil(mx * inv_h).astype(np.int64) + 3
    ext = (hi - lo).astype(F)
    R = (h * (np.sqrt(dot3(ext, ext)) + F(2.0))).astype(F)
    gm = h * (np.maximum(np.abs(lo), np.abs(hi)).max(axis=1) + 1).astype(F)
    M = np.maximum(gm, np.abs(tri).reshape(n, 9).max(axis=1)).astype(F)
    c2, e0 = cull_coeffs(a, b, c, R, M)
    ok = np.isfinite(c2)
    c2, e0, R = c2[ok], e0[ok], R[ok]
    lb1 = (rng.random(len(R)) * R * R).astype(F)
    lb2 = (lb1 + rng.random(len(R)) * (R * R - lb1)).astype(F)
    with np.errstate(all="ignore"):
        t1 = fmaf(c2, lb1, e0)
        t2 = fmaf(c2, lb2, e0)
        k = F(1.03125)
        extra1 = F(33.0) * (t1 * t1)
        cur = ((lb1.astype(np.float64) - extra1.astype(np.float64)) / 1.03125).astype(F)
        for _ in range(4):  # the largest minimum the test culls against at lb1
            bad = ~(lb1 > fmaf(cur, np.full_like(cur, k), extra1))
            cur = np.where(bad, np.nextafter(cur, F(-np.inf)), cur)
        cull1 = (cur > 0) & (lb1 > fmaf(cur, np.full_like(cur, k), extra1))
        cull2 = lb2 > fmaf(cur, np.full_like(cur, k), F(33.0) * (t2 * t2))
    assert cull1.sum() > 0.3 * len(cur)
    assert np.all(cull2[cull1])
