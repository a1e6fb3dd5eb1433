"""Parity of the CUDA mesh -> SDF path (bs_mesh_to_volume) with the oracle.

Bar: identical leaf set and active masks, bit-identical |distance| for every
active voxel, and zero sign mismatches (the sign is the fast winding number
thresholded at 0.2, mesh_to_volume.rs:264-271).
"""
import json
import os

import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import compare_volumes, context, unpack_mask

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def run_both(v, f, h, band):
    ctx = context()
    vol = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(band).convert((v, f))
    ov, stats, _ = ob.mesh_to_volume(v, f, h, band)
    return vol, ov, stats


def assert_parity(vol, ov):
    rep = compare_volumes(vol.export(), ov.export(), check_inactive=True)
    assert rep["leaf_set_equal"], rep
    assert rep["mask_mismatch_leaves"] == 0, rep
    assert rep["value_mismatch"] == 0, rep
    assert rep["sign_mismatch"] == 0, rep
    assert rep["inactive_mismatch"] == 0, rep
    return rep


def box2():
    tris = np.array(GOLD["box2_stl"]["triangles"], np.float32)
    v = tris.reshape(-1, 3)
    return v, np.arange(len(v), dtype=np.uint32).reshape(-1, 3)


@pytest.mark.parametrize("h,band", [(0.2, 0), (0.1, 1), (0.07, 3)])
def test_box2(h, band):
    v, f = box2()
    vol, ov, _ = run_both(v, f, h, band)
    assert_parity(vol, ov)


def test_icosphere_config1():
    """Icosphere s4 (5,120 triangles), radial noise 0.05, voxel 0.02, band 3."""
    v, f = synthetic.config1()
    vol, ov, stats = run_both(v, f, 0.02, 3)
    rep = assert_parity(vol, ov)
    assert rep["active"] == stats["band_voxels"]
    assert vol.counts()["active_voxels"] == stats["band_voxels"]


def test_small_torus():
    v, f = synthetic.torus(1.0, 0.3, 96, 48, 0.02, seed=5)
    vol, ov, _ = run_both(v, f, 0.01, 2)
    assert_parity(vol, ov)


def test_rotated_shifted_torus_negative_coords():
    v, f = synthetic.torus(0.6, 0.2, 64, 32, 0.01, seed=7, rotate_x_deg=90.0, shift=(-0.73, 0.21, -0.4))
    vol, ov, _ = run_both(v, f, 0.013, 3)
    assert_parity(vol, ov)


def test_far_from_origin_matches_oracle():
    """A mesh two thousand units from the origin at voxel 0.05: the float32
    coordinates keep only about 1e-4 of absolute precision there (ulp 1.2e-4
    at 2000), so the grid points, sub-triangles, distances and the tree's
    far-field terms all round coarsely; the volume is still the oracle's bit
    for bit."""
    v, f = synthetic.icosphere(3, 0.5, 0.02, seed=21)
    v = (v.astype(np.float64) + np.array([1000.25, -2000.5, 333.0])).astype(np.float32)
    vol, ov, _ = run_both(v, f, 0.05, 2)
    assert_parity(vol, ov)


ATAN2_RESIDUE = 1e-6  # |wn - 0.2| below which last-place atan2f differences may flip a sign


def parity_open(v, f, h, band, tree="reference"):
    """Open meshes: distances and the active set bit-exact; returns the sign
    flips against the oracle with the oracle's winding number at each."""
    ctx = context()
    vol = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(band).with_sign_tree(tree).convert((v, f))
    ov, stats, wn = ob.mesh_to_volume(v, f, h, band, with_wn=True)
    go, gv, gm = vol.export()
    oo, ovv, om = ov.export()
    oact = np.stack([unpack_mask(m) for m in om])
    wfull = np.zeros(oact.shape, np.float32)
    wfull[oact] = wn  # oracle order: leaves in tree order, voxels by index
    perm = np.lexsort((oo[:, 2], oo[:, 1], oo[:, 0]))  # GPU order: leaves sorted by (x, y, z)
    oo, ovv, om, oact, wfull = oo[perm], ovv[perm], om[perm], oact[perm], wfull[perm]
    assert np.array_equal(go, oo) and np.array_equal(gm, om)
    ga, oa, w = gv[oact], ovv[oact], wfull[oact]
    assert np.array_equal(np.abs(ga).view(np.uint32), np.abs(oa).view(np.uint32))
    flips = np.signbit(ga) != np.signbit(oa)
    return w[flips], len(oa)


def assert_parity_open(v, f, h, band):
    """The reference's tree (the default): signs bit-exact.  A flip is allowed
    only where the reference's own winding number lies within 1e-6 of the
    0.2 threshold, where CUDA's atan2f and the host's can differ in the last
    place; every such flip is returned so a test can list it."""
    w, n = parity_open(v, f, h, band)
    assert np.all(np.abs(w - 0.2) < ATAN2_RESIDUE), (len(w), w)
    return len(w), n


def assert_parity_open_fast(v, f, h, band):
    """The library's PLOC tree (with_sign_tree("fast")): its far field differs
    from the reference's SAH tree by approximation error, so a sign may differ
    only where the reference's own winding number lies within 0.01 of 0.2."""
    w, n = parity_open(v, f, h, band, tree="fast")
    assert np.all(np.abs(w - 0.2) < 0.01), (len(w), w)
    return len(w), n


def test_open_soup_with_holes():
    """Open soup (10 % of faces removed): signs equal the reference's."""
    v, f = synthetic.icosphere(3, 0.8, 0.05, seed=3)
    f = synthetic.remove_faces(f, 0.1, seed=4)
    flips, n = assert_parity_open(v, f, 0.03, 2)
    assert flips == 0, flips


def test_open_soup_with_holes_fast_tree():
    v, f = synthetic.icosphere(3, 0.8, 0.05, seed=3)
    f = synthetic.remove_faces(f, 0.1, seed=4)
    flips, n = assert_parity_open_fast(v, f, 0.03, 2)
    assert flips <= 1e-3 * n


def test_open_icosphere_subdivision5():
    """A finer open soup (20,480 triangles before removal, band 3): large
    enough for the tree build's whole-GPU levels; signs equal the reference's."""
    v, f = synthetic.icosphere(5, 1.0, 0.03, seed=8)
    f = synthetic.remove_faces(f, 0.1, seed=9)
    flips, n = assert_parity_open(v, f, 0.01, 3)
    assert n > 500_000
    assert flips == 0, flips


def test_single_triangle_and_grid_aligned():
    # a triangle lying in the plane z = 0 (flat integer box -> widened by 1, mesh_to_volume.rs:137-141)
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    f = np.array([[0, 1, 2]], np.uint32)
    vol, ov, _ = run_both(v, f, 0.25, 0)
    assert_parity(vol, ov)
    vol, ov, _ = run_both(v, f, 0.1, 2)
    assert_parity(vol, ov)


def test_degenerate_triangles():
    """Zero-area triangles (collinear, repeated vertex) next to one real,
    open triangle."""
    v = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0.5, 0.5, 0.5], [0.5, 0.5, 0.5]], np.float32)
    f = np.array([[0, 1, 2], [3, 4, 0], [0, 1, 3]], np.uint32)
    flips, _ = assert_parity_open(v, f, 0.1, 1)
    assert flips == 0


def test_duplicates_ties_and_degenerates():
    """A soup built to stress the tree build's order rules: 300 copies of one
    triangle (a leaf the SAH cannot split), triangles on a grid (equal box
    centres along every axis), exact degenerates and the cull-stress soup."""
    rng = np.random.default_rng(21)
    base = np.array([[0.1, 0.2, 0.3], [0.4, 0.25, 0.3], [0.2, 0.6, 0.35]], np.float32)
    dup = np.repeat(base[None], 300, axis=0)
    g = np.stack(np.meshgrid(np.arange(6), np.arange(6), np.arange(3), indexing="ij"), -1).reshape(-1, 3) * 0.125
    grid = np.stack([g, g + [0.1, 0.0, 0.0], g + [0.0, 0.1, 0.02]], axis=1).astype(np.float32)
    degen = rng.uniform(-0.5, 0.5, (40, 1, 3)).astype(np.float32).repeat(3, axis=1)
    degen[:, 2] += np.float32(0.05)
    tri = np.concatenate([dup, grid, degen, grid[::-1] + np.float32(0.01)])
    v = tri.reshape(-1, 3)
    f = np.arange(len(v), dtype=np.uint32).reshape(-1, 3)
    flips, _ = assert_parity_open(v, f, 0.05, 2)
    assert flips == 0
    v2, f2 = cull_stress_soup(0.05, 13)
    flips, _ = assert_parity_open(v2, f2, 0.05, 2)
    assert flips == 0


def cull_stress_soup(h, seed):
    """Random soup for the pair culling of the distance pass: well-shaped
    triangles of 0.3-2 voxels, needles (two vertices within 1e-4 voxel),
    near-collinear slivers, exactly degenerate triangles and large
    triangles of ~10 voxels, randomly oriented, far from the origin."""
    rng = np.random.default_rng(seed)
    centre = np.array([37.3, -51.9, 12.1], np.float64)
    tris = []

    def rnd_dir(n):
        d = rng.normal(size=(n, 3))
        return d / np.linalg.norm(d, axis=1, keepdims=True)

    n = 300
    c = centre + rng.uniform(-8 * h, 8 * h, size=(n, 3))
    s = rng.uniform(0.3, 2.0, size=(n, 1)) * h
    tris.append(np.stack([c + s * rnd_dir(n), c + s * rnd_dir(n), c + s * rnd_dir(n)], axis=1))
    n = 120  # needles
    c = centre + rng.uniform(-8 * h, 8 * h, size=(n, 3))
    far = c + 1.5 * h * rnd_dir(n)
    tris.append(np.stack([c, c + 1e-4 * h * rnd_dir(n), far], axis=1))
    n = 120  # slivers: the third vertex within 1e-5..1e-2 voxel of the line of the others
    a = centre + rng.uniform(-8 * h, 8 * h, size=(n, 3))
    b = a + 2.0 * h * rnd_dir(n)
    t = rng.uniform(0.1, 0.9, size=(n, 1))
    off = 10.0 ** rng.uniform(-5, -2, size=(n, 1)) * h
    tris.append(np.stack([a, b, a + t * (b - a) + off * rnd_dir(n)], axis=1))
    n = 30  # exactly degenerate
    a = centre + rng.uniform(-8 * h, 8 * h, size=(n, 3))
    tris.append(np.stack([a, a, a + h * rnd_dir(n)], axis=1))
    n = 40  # large
    c = centre + rng.uniform(-6 * h, 6 * h, size=(n, 3))
    tris.append(np.stack([c + 10 * h * rnd_dir(n), c + 10 * h * rnd_dir(n), c + 10 * h * rnd_dir(n)], axis=1))
    tri = np.concatenate(tris).astype(np.float32)
    v = tri.reshape(-1, 3)
    return v, np.arange(len(v), dtype=np.uint32).reshape(-1, 3)


@pytest.mark.parametrize("seed", [11, 12])
def test_culled_distances_on_slivers_and_needles(seed):
    """The distance pass skips pairs whose lower bound exceeds the voxel's
    running minimum; on triangles of every conditioning the distances and
    the active set stay bit-identical to the oracle's full evaluation."""
    h, band = 0.05, 2
    v, f = cull_stress_soup(h, seed)
    ctx = context()
    vol = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(band).convert((v, f))
    st = ctx.last_stats()
    ov, _, _ = ob.mesh_to_volume(v, f, h, band)
    go, gv, gm = vol.export()
    oo, ovv, om = ov.export()
    perm = np.lexsort((oo[:, 2], oo[:, 1], oo[:, 0]))
    oo, ovv, om = oo[perm], ovv[perm], om[perm]
    assert np.array_equal(go, oo) and np.array_equal(gm, om)
    act = np.stack([unpack_mask(m) for m in om])
    assert np.array_equal(np.abs(gv[act]).view(np.uint32), np.abs(ovv[act]).view(np.uint32))
    assert 0 < st["voxel_pairs_evaluated"] < st["voxel_pairs"]


def test_empty_mesh_is_none():
    ctx = context()
    v = np.zeros((0, 3), np.float32)
    f = np.zeros((0, 3), np.uint32)
    assert bs.MeshToVolume(ctx).with_voxel_size(0.1).convert((v, f)) is None


def test_bad_index_raises():
    ctx = context()
    v = np.zeros((3, 3), np.float32)
    f = np.array([[0, 1, 7]], np.uint32)
    with pytest.raises(bs.BsError) as e:
        bs.MeshToVolume(ctx).with_voxel_size(0.1).convert((v, f))
    assert e.value.status == 1


def test_deterministic_repeat():
    v, f = synthetic.config1()
    ctx = context()
    a = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((v, f)).export()
    b = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((v, f)).export()
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                              y.view(np.uint32) if y.dtype == np.float32 else y)


def test_full_size_torus_sign_property():
    """Config-2 torus at full size (1,048,576 triangles, voxel 0.002, band 3):
    signs agree with the analytic torus wherever the voxel is farther from the
    undisplaced surface than the displacement amplitude plus two voxels, and
    every |value| is below the widened-box bound."""
    (v, f), _ = synthetic.config2()
    ctx = context()
    h = 0.002
    vol = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(3).convert((v, f))
    o, val, m = vol.export()
    act = np.stack([unpack_mask(mm) for mm in m])
    idx = np.nonzero(act)
    li, vi = idx
    x = (o[li, 0] + (vi >> 6)) * np.float32(h)
    y = (o[li, 1] + ((vi >> 3) & 7)) * np.float32(h)
    z = (o[li, 2] + (vi & 7)) * np.float32(h)
    d_tube = np.hypot(np.hypot(x, y) - 1.0, z) - 0.3
    vals = val[li, vi]
    sure = np.abs(d_tube) > 0.02 + 2 * h
    assert sure.sum() > 1000
    assert np.all(np.signbit(vals[sure]) == (d_tube[sure] < 0))
    assert np.all(np.abs(vals) <= (3 + 2) * h * np.sqrt(3) + 1e-6)
    assert vol.counts()["active_voxels"] == act.sum()


def test_exact_winding_numbers_match_oracle_f64():
    """bs_winding_numbers_exact against the oracle's float64 direct sum."""
    v, f = synthetic.icosphere(3, 0.8, 0.04, seed=4)
    f = synthetic.remove_faces(f, 0.1, seed=5)
    rng = np.random.default_rng(6)
    pts = rng.uniform(-1.0, 1.0, (4000, 3)).astype(np.float32)
    g = bs.winding_numbers_exact(v, f, pts, ctx=context()).cpu().numpy()
    o = ob.exact_wn_f64(v, f.astype(np.uint32), pts)
    assert np.max(np.abs(g - o)) < 2e-5


def test_fast_sign_agrees_with_exact_on_watertight():
    """Every band voxel's sign from the tree approximation equals the exact
    winding number's classification (wn < 0.2 outside) on a closed mesh."""
    v, f = synthetic.config1()
    vol = bs.MeshToVolume(context()).with_voxel_size(0.02).with_narrow_band_width(3).convert((v, f))
    o, val, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    idx = np.nonzero(act)
    off = idx[1]
    vox = o[idx[0]] + np.stack([off >> 6, (off >> 3) & 7, off & 7], 1)
    pts = vox.astype(np.float32) * np.float32(0.02)
    wn = bs.winding_numbers_exact(v, f, pts, ctx=context()).cpu().numpy()
    inside_gpu = np.signbit(val[idx])
    assert np.array_equal(inside_gpu, wn >= 0.2)


def test_distance_error_vs_float64():
    """The float32 distances (bit-identical to the reference's) against a
    float64 evaluation of the same candidate minimum, in voxel units: the
    error stays at the float32 rounding of the inputs (about 1e-5 voxel here)."""
    from tests.f64_distance import min_distance_f64
    v, f = synthetic.config1()
    h = 0.02
    vol = bs.MeshToVolume(context()).with_voxel_size(h).with_narrow_band_width(3).convert((v, f))
    o, val, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    li, vi = np.nonzero(act)
    pick = np.random.default_rng(3).choice(len(li), 1500, replace=False)
    li, vi = li[pick], vi[pick]
    vox = o[li].astype(np.int64) + np.stack([vi >> 6, (vi >> 3) & 7, vi & 7], 1)
    sub, box = ob.subtriangles(v, f, h, 3)
    d64 = min_distance_f64(vox, h, sub, box)
    err = np.abs(np.abs(val[li, vi]).astype(np.float64) - d64) / h
    assert np.all(np.isfinite(d64))
    assert err.max() < 1e-5


def test_distance_error_vs_float64_fine_voxel():
    """The same on a patch of the boolean workload's torus at its voxel size
    0.002: the float32 inputs themselves (ulp 1.2e-7 at coordinates ~1.3 =
    6e-5 voxel) bound the error; it stays within 2e-4 voxel."""
    from tests.f64_distance import min_distance_f64
    (v, f), _ = synthetic.config2(nu=1024, nv=512)
    c = (v[f[:, 0]] + v[f[:, 1]] + v[f[:, 2]]) / 3
    keep = np.linalg.norm(c - v[0], axis=1) < 0.02
    v2, f2 = v, f[keep]
    h = 0.002
    vol = bs.MeshToVolume(context()).with_voxel_size(h).with_narrow_band_width(3).convert((v2, f2))
    o, val, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    li, vi = np.nonzero(act)
    pick = np.random.default_rng(4).choice(len(li), 800, replace=False)
    li, vi = li[pick], vi[pick]
    vox = o[li].astype(np.int64) + np.stack([vi >> 6, (vi >> 3) & 7, vi & 7], 1)
    sub, box = ob.subtriangles(v2, f2, h, 3)
    d64 = min_distance_f64(vox, h, sub, box)
    err = np.abs(np.abs(val[li, vi]).astype(np.float64) - d64) / h
    assert err.max() < 2e-4


def _f64_error_on_patch(v, f, centre, radius, h, n_pick, seed):
    """Max and mean |float32 distance - float64 candidate minimum| / h over a
    seeded sample of the band voxels of the faces within `radius` of `centre`."""
    from tests.f64_distance import min_distance_f64
    c = (v[f[:, 0]].astype(np.float64) + v[f[:, 1]] + v[f[:, 2]]) / 3
    f2 = f[np.linalg.norm(c - centre, axis=1) < radius]
    vol = bs.MeshToVolume(context()).with_voxel_size(h).with_narrow_band_width(3).convert((v, f2))
    o, val, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    li, vi = np.nonzero(act)
    pick = np.random.default_rng(seed).choice(len(li), min(n_pick, len(li)), replace=False)
    li, vi = li[pick], vi[pick]
    vox = o[li].astype(np.int64) + np.stack([vi >> 6, (vi >> 3) & 7, vi & 7], 1)
    sub, box = ob.subtriangles(v, f2, h, 3)
    d64 = min_distance_f64(vox, h, sub, box)
    assert np.all(np.isfinite(d64))
    err = np.abs(np.abs(val[li, vi]).astype(np.float64) - d64) / h
    return err.max(), err.mean(), len(f2), float(np.abs(v).max())


def test_distance_error_vs_float64_open_icosphere():
    """The holed subdivision-9 icosphere at its voxel size 0.001: the float32
    vertices (ulp 1.2e-7 at |coordinates| up to 1.1 = 1.2e-4 voxel) bound the
    error, which stays within 3e-4 voxel."""
    v, f = synthetic.open_icosphere()
    mx, mean, nf, vmax = _f64_error_on_patch(v, f, v[f[0, 0]].astype(np.float64), 0.025, 0.001, 600, 5)
    print("open icosphere patch: %d faces, max %.3g voxel, mean %.3g voxel" % (nf, mx, mean))
    assert nf > 300 and mx < 3e-4


def test_distance_error_vs_float64_large_union_torus():
    """The first torus of the 16-torus union at its voxel size 0.0005: the
    float32 vertices (ulp 1.2e-7 to 2.4e-7 at |coordinates| up to ~2.2 =
    up to 4.8e-4 voxel) bound the error, which stays within 1e-3 voxel."""
    (v, f), = synthetic.large_union(n=1)
    mx, mean, nf, vmax = _f64_error_on_patch(v, f, v[f[0, 0]].astype(np.float64), 0.07, 0.0005, 600, 6)
    print("large-union torus patch: %d faces, |coord| <= %.2f, max %.3g voxel, mean %.3g voxel" % (nf, vmax, mx, mean))
    assert nf > 300 and mx < 1e-3


def test_launch_shapes_give_identical_volumes_and_autotune_picks_one():
    """Every launch shape and tile the autotuner chooses from gives the same
    volume, bit for bit, on both sign trees; the autotuner returns one of
    them."""
    ctx = bs.Context(0)
    v, f = synthetic.torus(1.0, 0.3, 96, 48, 0.02, seed=5)
    for tree in ("reference", "fast"):
        ref = None
        for dt, ww, ti in ((64, 2, 8), (128, 4, 16), (256, 8, 16), (64, 8, 32), (256, 2, 8), (128, 2, 32)):
            ctx.set_launch_shape(dt, ww, ti)
            vol = bs.MeshToVolume(ctx).with_voxel_size(0.01).with_narrow_band_width(2).with_sign_tree(tree).convert(
                (v, f))
            o, val, m = vol.export()
            if ref is None:
                ref = (o, val, m)
            else:
                assert np.array_equal(o, ref[0]) and np.array_equal(m, ref[2])
                assert np.array_equal(val.view(np.uint32), ref[1].view(np.uint32))
    with pytest.raises(bs.BsError):
        ctx.set_launch_shape(256, 0, 32)
    choice = ctx.autotune((v, f), 0.01, 2)
    assert choice["dist_threads"] in (64, 128, 256) and choice["wn_warps"] in (2, 4, 8)
    assert choice["dist_tile"] in (8, 16, 32)
    assert all(t > 0 for t in choice["distance_ms"].values())
