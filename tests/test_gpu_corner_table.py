"""The CornerTable soup builder (CornerTable::builder_soup().finish(),
mesh/corner_table/builder.rs:168-309) on the GPU — point merge, the
order-dependent face skipping, isolated-vertex deletion and vertex splitting
— against the oracle's restatement of the same builder on the same merged
indexed mesh: every table equal, entry for entry (corner -> vertex, corner ->
opposite corner, vertex -> corner, deleted flags, positions).  New vertices
of split fans are numbered in vertex order on both sides (the reference
iterates a hash map there, so only its counts are order free)."""
import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import context

pytestmark = pytest.mark.gpu


def merge_first_appearance(soup):
    """merge_points (algo/merge_points.rs:12-41): equal points (-0 == +0)
    share a vertex, numbered in order of first appearance."""
    p = np.ascontiguousarray(soup, np.float32).reshape(-1, 3) + np.float32(0.0)  # -0 -> +0
    rows = p.view(np.dtype((np.void, 12))).ravel()
    _, first, inv = np.unique(rows, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    ids = rank[inv.ravel()]
    uniq = np.ascontiguousarray(soup, np.float32).reshape(-1, 3)[first[order]]
    return uniq, ids.reshape(-1, 3)


def assert_same_tables(soup):
    soup = np.ascontiguousarray(soup, np.float32).reshape(-1, 3, 3)
    g = bs.CornerTable.from_triangles_soup(soup, context())
    ex = g.export()
    uniq, faces = merge_first_appearance(soup)
    o = ob.corner_table_from_indexed(uniq, faces)
    assert o["status"] == 0
    assert np.array_equal(ex["corner_vertex"], o["corner_vertex"])
    assert np.array_equal(ex["corner_opposite"], o["corner_opposite"])
    assert np.array_equal(ex["vertex_corner"], o["vertex_corner"])
    assert np.array_equal(ex["deleted"], o["vertex_deleted"].astype(bool))
    n0 = len(uniq)
    assert np.array_equal(ex["positions"][:n0].view(np.uint32), uniq.view(np.uint32))
    c = g.counts()
    assert (c["faces"], c["vertices"]) == (o["faces"], o["vertices"])
    return c


def test_dual_contouring_soup():
    v, f = synthetic.config1()
    vol = bs.MeshToVolume(context()).with_voxel_size(0.02).with_narrow_band_width(3).convert((v, f))
    c = assert_same_tables(bs.DualContouringMesher().with_voxel_size(0.02).mesh(vol))
    assert c["faces"] > 1000


def test_marching_cubes_soup_of_a_union_with_tiles():
    va, fa = synthetic.icosphere(3, 0.6, 0.02, seed=11)
    vb, fb = synthetic.icosphere(3, 0.5, 0.02, seed=12)
    vb = vb + np.array([0.45, 0.1, -0.05], np.float32)
    ctx = context()
    a = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((va, fa))
    b = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((vb, fb))
    u = a.union(b)
    assert_same_tables(bs.MarchingCubesMesher().with_voxel_size(0.02).mesh(u))


def test_reference_builder_kats_tables():
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))
    for name in ("non_manifold_topology", "non_manifold_edge"):
        g = gold[name]
        verts = np.array(g["vertices"], np.float32)
        idx = np.array(g["indices"], np.int64).reshape(-1, 3)
        c = assert_same_tables(verts[idx])
        assert c["faces"] == g["expected_faces"]


def test_non_manifold_and_degenerate_soup():
    """Repeated faces, flipped duplicates, faces sharing directed edges in
    chains, degenerate faces with repeated vertices, bow-tie vertices and
    isolated points."""
    rng = np.random.default_rng(3)
    grid = np.stack(np.meshgrid(np.arange(6), np.arange(6), indexing="ij"), -1).reshape(-1, 2).astype(np.float32)
    pts = np.concatenate([grid, np.zeros((len(grid), 1), np.float32)], 1)
    quads = [(i * 6 + j, (i + 1) * 6 + j, (i + 1) * 6 + j + 1, i * 6 + j + 1) for i in range(5) for j in range(5)]
    faces = []
    for a, b, c, d in quads:
        faces += [(a, b, c), (a, c, d)]
    faces = np.array(faces)
    extra = faces[rng.choice(len(faces), 15, replace=False)]
    flipped = faces[rng.choice(len(faces), 10, replace=False)][:, ::-1]
    fan = np.array([(14, 7, 21), (14, 21, 8), (14, 8, 20), (14, 20, 7)])  # a second fan at vertex 14
    degen = np.array([(3, 3, 3), (4, 4, 9), (9, 10, 9), (27, 28, 27)])
    allf = np.concatenate([faces, extra, flipped, fan, degen, faces[::7]])
    rng.shuffle(allf)
    soup = pts[allf]
    soup[0, 0] = [-0.0, 0.0, 0.0]  # -0 merges with +0
    assert_same_tables(soup)


def test_random_soups():
    rng = np.random.default_rng(9)
    for trial in range(4):
        pts = rng.integers(0, 12, size=(40, 3)).astype(np.float32)
        faces = rng.integers(0, 40, size=(300, 3))
        assert_same_tables(pts[faces])
