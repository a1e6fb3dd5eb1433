"""Parity of the CUDA dual contouring (bs_dual_contour) with the oracle: the
same triangles, bit for bit, as a multiset (the reference's own face order
depends on thread scheduling, dual_contouring.rs:145-173)."""
import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import context

pytestmark = pytest.mark.gpu


def both(v, f, h, band):
    ctx = context()
    g = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(band).convert((v, f))
    o, _, _ = ob.mesh_to_volume(v, f, h, band)
    return g, o


def tri_multiset(tris):
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 9).view(np.uint32)
    order = np.lexsort(t.T[::-1])
    return t[order]


def assert_same_mesh(gv, ov, h):
    gt = bs.DualContouringMesher().with_voxel_size(h).mesh(gv)
    ot, status, _, _ = ov.dual_contour()
    assert status == 0
    assert gt.shape == ot.shape, (gt.shape, ot.shape)
    assert np.array_equal(tri_multiset(gt), tri_multiset(ot))
    return gt


def test_icosphere_config1_dc():
    """Icosphere s4, voxel 0.02, band 3, then dual contouring."""
    v, f = synthetic.config1()
    gv, ov = both(v, f, 0.02, 3)
    gt = assert_same_mesh(gv, ov, 0.02)
    assert len(gt) > 10000


def test_torus_dc():
    v, f = synthetic.torus(1.0, 0.3, 128, 64, 0.02, seed=2)
    gv, ov = both(v, f, 0.01, 3)
    assert_same_mesh(gv, ov, 0.01)


def test_offset_then_dc():
    """The boolean workload's tail: subtract, offset, dual contouring."""
    va, fa = synthetic.torus(1.0, 0.3, 96, 48, 0.02, seed=2)
    vb, fb = synthetic.torus(1.0, 0.3, 96, 48, 0.02, seed=3, rotate_x_deg=90.0, shift=(0.5, 0.0, 0.0))
    ga, oa = both(va, fa, 0.012, 3)
    gb, ob_ = both(vb, fb, 0.012, 3)
    g = ga.subtract(gb).offset(0.024)
    o = oa.subtract(ob_).offset(0.024)
    assert_same_mesh(g, o, 0.012)


def test_dc_union_with_tiles_matches_oracle_extension():
    """Active tiles: the reference stops with todo!() (dual_contouring.rs:139);
    both the oracle (tiles_via_at) and the GPU read tile voxels through the
    tree's `at` and give the same triangles, bit for bit."""
    va, fa = synthetic.icosphere(3, 0.6, 0.02, seed=11)
    vb, fb = synthetic.icosphere(3, 0.5, 0.02, seed=12)
    vb = vb + np.array([0.45, 0.1, -0.05], np.float32)
    ctx = context()
    a = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((va, fa))
    b = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((vb, fb))
    u = a.union(b)
    assert u.counts()["tiles"] > 0
    oa, _, _ = ob.mesh_to_volume(va, fa, 0.02, 3)
    obb, _, _ = ob.mesh_to_volume(vb, fb, 0.02, 3)
    ou = oa.union(obb)
    _, status, _, _ = ou.dual_contour()
    assert status == 1  # the reference's behaviour
    ot, status, _, _ = ou.dual_contour(tiles_via_at=True)
    assert status == 0
    gt = bs.DualContouringMesher().with_voxel_size(0.02).mesh(u)
    assert gt.shape == ot.shape and len(gt) > 1000
    assert np.array_equal(tri_multiset(gt), tri_multiset(ot))


def test_corner_table_from_dc_matches_oracle_builder():
    """VoxelRemesher(FeaturePreserving) tail: DC soup -> CornerTable.  The
    merged vertex set and the face/vertex counts match the oracle's builder on
    the oracle's soup."""
    v, f = synthetic.config1()
    gv, ov = both(v, f, 0.02, 3)
    ct = bs.CornerTable.from_dual_contouring(gv, 0.02)
    ot, status, _, _ = ov.dual_contour()
    nf, nv = ob.corner_table_from_soup(ot.reshape(-1, 3))
    c = ct.counts()
    assert (c["faces"], c["vertices"]) == (nf, nv)
    ex = ct.export()
    live = ex["positions"][~ex["deleted"]]
    uniq_ref = np.unique(ot.reshape(-1, 3).view(np.uint32), axis=0)
    assert np.array_equal(np.unique(live.view(np.uint32), axis=0), uniq_ref)


def test_corner_table_reference_kats_on_gpu_builder():
    """The reference builder tests replayed through the GPU soup builder:
    192 faces / 100 vertices (builder.rs:378-524) and 4 faces
    (builder.rs:361-376); the merged soup gives the same counts."""
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))
    for name in ("non_manifold_topology", "non_manifold_edge"):
        g = gold[name]
        verts = np.array(g["vertices"], np.float32)
        idx = np.array(g["indices"], np.int64).reshape(-1, 3)
        soup = verts[idx]
        c = bs.CornerTable.from_triangles_soup(soup, context()).counts()
        assert c["faces"] == g["expected_faces"]
        if "expected_vertices" in g:
            assert c["vertices"] == g["expected_vertices"]
        assert (c["faces"], c["vertices"]) == ob.corner_table_from_soup(soup.reshape(-1, 3))


def test_voxel_remesher_feature_preserving():
    v, f = synthetic.config1()
    r = bs.VoxelRemesher(context()).with_voxel_size(0.02).with_narrow_band_width(3) \
        .with_meshing_method(bs.VoxelRemesher.FEATURE_PRESERVING)
    ct = r.remesh((v, f))
    assert ct.faces_count() > 10000 and ct.vertices_count() > 5000


def test_qef_vertices_sphere_and_cuboid():
    """bs_dual_contour_qef: the same cells and quads as the particle solver
    (same triangle count), vertices on a sphere's surface, and on a cuboid's
    flat faces (rank-1 systems) every vertex exactly on its face plane."""
    h = 0.02
    sph = bs.VolumeBuilder(context()).with_voxel_size(h).sphere(0.5, (0.013, -0.007, 0.004))
    part = bs.DualContouringMesher().with_voxel_size(h).mesh(sph)
    qef = bs.DualContouringMesher().with_voxel_size(h).with_qef_vertices().mesh(sph)
    assert abs(len(qef) - len(part)) <= len(part) // 1000
    r = np.linalg.norm(qef.reshape(-1, 3) - np.array([0.013, -0.007, 0.004], np.float32), axis=1)
    assert np.abs(r - 0.5).max() < 0.25 * h and np.abs(r - 0.5).mean() < 0.05 * h
    mn, mx = np.array([-0.301, -0.203, -0.105]), np.array([0.307, 0.252, 0.196])
    cub = bs.VolumeBuilder(context()).with_voxel_size(h).cuboid(mn, mx)
    q = np.unique(bs.DualContouringMesher().with_voxel_size(h).with_qef_vertices().mesh(cub).reshape(-1, 3), axis=0)
    # distance of each vertex to the six face planes; vertices 3 voxels away
    # from every edge of the box sit on exactly one face
    dp = np.abs(np.concatenate([q - mn, q - mx], axis=1)).astype(np.float64)
    near = np.sort(dp, axis=1)
    interior = near[:, 1] > 3 * h
    assert interior.sum() > 500
    assert near[interior, 0].max() < 1e-3 * h
