"""Pin the oracle against the reference's own known-answer tests.

Every case below replays a unit test of baby_shark v0.3.12 whose literal
inputs and expected values live in tests/golden/reference_kats.json
(extracted by tests/golden/make_reference_kats.py).
"""
import json
import os

import numpy as np
import pytest

from oracle import binding as ob

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def test_volume_offset_7944():
    """src/voxel/volume/mod.rs:134-152 — box2.stl, voxel 0.2, band 0, offset 0.5 -> 7944 MC vertices."""
    g = GOLD["volume_offset"]
    tris = np.array(GOLD["box2_stl"]["triangles"], np.float32)
    verts = tris.reshape(-1, 3)
    idx = np.arange(len(verts), dtype=np.uint32).reshape(-1, 3)
    vol, stats, _ = ob.mesh_to_volume(verts, idx, g["voxel_size"], 0)
    assert stats["band_voxels"] > 0
    vol.offset(g["offset"])
    n_tri, ambiguous, _ = vol.mc_triangles()
    assert ambiguous == 0  # the triangle counter is exact only without ambiguous faces
    assert 3 * n_tri == g["mc_vertices"]
    # the marching-cubes mesher the GPU mirrors gives the same soup size
    tri = vol.marching_cubes(g["voxel_size"])
    assert 3 * len(tri) == g["mc_vertices"]
    # every triangle faces the positive (outside) side: normals point away from the box's centre
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    centre = verts.mean(axis=0)
    assert np.mean(np.einsum("ij,ij->i", n, tri.mean(axis=1) - centre) > 0) > 0.99


@pytest.mark.parametrize("op", ["union", "subtract", "intersect"])
def test_leaf_csg(op):
    """src/voxel/leaf_node/csg.rs:53-132."""
    g = GOLD["leaf_csg"][op]
    out, full = ob.leaf1_csg(op, g["a"], g["b"])
    assert out.tolist() == g["expected"]
    assert full


def test_tree_constants():
    """src/voxel/init.rs:49-66 (BRANCHING / BRANCHING_TOTAL / children per node)."""
    c = ob.tree_constants()
    want = dict(GOLD["tree_constants"]["asserts"])
    assert c[0] == want["Grid::BRANCHING"] and c[1] == want["Grid::BRANCHING_TOTAL"] and c[2] == want["Grid::SIZE"]
    assert c[3] == want["Lvl1::BRANCHING"] and c[4] == want["Lvl1::BRANCHING_TOTAL"] and c[5] == want["Lvl1::SIZE"]
    assert c[6] == want["Lvl2::BRANCHING"] and c[7] == want["Lvl2::BRANCHING_TOTAL"]


def test_leaf_flood_fill():
    """src/voxel/leaf_node/flood_fill.rs:82-113 (static_vdb!(f32, 2))."""
    t = ob.SmallTree("leaf2")
    t.insert(2, 2, 2, 1.0)
    t.flood_fill()
    assert np.all(~np.signbit(t.values()))
    t = ob.SmallTree("leaf2")
    t.insert(2, 2, 2, -1.0)
    t.flood_fill()
    assert np.all(np.signbit(t.values()))
    t = ob.SmallTree("leaf2")
    for y in range(4):
        for z in range(4):
            t.insert(1, y, z, -1.0)
            t.insert(2, y, z, 1.0)
    t.flood_fill()
    v = t.values()
    assert np.all(np.signbit(v[:32])) and np.all(~np.signbit(v[32:64]))


def test_internal_flood_fill():
    """src/voxel/internal_node/flood_fill.rs:128-193 (static_vdb!(f32, 2, 1), resolution 8)."""
    res, leaf_res = 8, 2
    t = ob.SmallTree("internal2_1")
    t.insert(3, 2, 1, 1.0)
    t.flood_fill()
    assert all(t.sign_at(x, y, z) == 1 for x in range(res) for y in range(res) for z in range(res))
    t = ob.SmallTree("internal2_1")
    t.insert(3, 3, 3, -1.0)
    t.flood_fill()
    assert all(t.sign_at(x, y, z) == -1 for x in range(res) for y in range(res) for z in range(res))
    t = ob.SmallTree("internal2_1")
    for y in range(res):
        for z in range(res):
            t.insert(4, y, z, -1.0)
            t.insert(5, y, z, 1.0)
    t.flood_fill()
    assert all(t.sign_at(x, y, z) == -1 for x in range(5) for y in range(5) for z in range(5))
    assert all(t.sign_at(x, y, z) == 1 for x in range(5, res) for y in range(5, res) for z in range(5, res))
    t = ob.SmallTree("internal2_1")
    x_neg, x_pos = 2, 4
    for x in range(x_neg, leaf_res + x_neg):
        for y in range(res):
            for z in range(res):
                t.insert(x, y, z, -1.0)
    for x in range(x_pos, leaf_res + x_pos):
        for y in range(res):
            for z in range(res):
                t.insert(x, y, z, 1.0)
    t.flood_fill()
    n = x_neg + leaf_res
    assert all(t.sign_at(x, y, z) == -1 for x in range(n) for y in range(n) for z in range(n))
    assert all(t.sign_at(x, y, z) == 1 for x in range(x_pos, res) for y in range(x_pos, res) for z in range(x_pos, res))


def test_root_flood_fill():
    """src/voxel/root_node/flood_fill.rs:74-95 (dynamic_vdb!(f32, 1)): gap tiles between inside children."""
    t = ob.SmallTree("root1")
    o1, o2 = (0, 4, 4), (0, 4, 10)
    for o in (o1, o2):
        for x in range(o[0], o[0] + 2):
            for y in range(o[1], o[1] + 2):
                for z in range(o[2], o[2] + 2):
                    t.insert(x, y, z, -1.0)
    t.flood_fill()
    for x in range(o1[0], o2[0] + 2):
        for y in range(o1[1], o2[1] + 2):
            for z in range(o1[2], o2[2] + 2):
                assert t.sign_at(x, y, z) == -1


def test_corner_table_unit_square():
    """src/mesh/corner_table/builder.rs:337-359 (exact corner/vertex tables)."""
    g = GOLD["unit_square"]
    r = ob.corner_table_from_indexed(g["vertices"], g["indices"])
    assert r["status"] == 0
    assert r["vertex_corner"].tolist() == g["expected_vertex_corner"]
    assert [[int(o), int(v)] for v, o in zip(r["corner_vertex"], r["corner_opposite"])] == g["expected_corners"]


def test_corner_table_non_manifold_edge():
    """src/mesh/corner_table/builder.rs:361-376 -> 4 faces."""
    g = GOLD["non_manifold_edge"]
    r = ob.corner_table_from_indexed(g["vertices"], g["indices"])
    assert r["faces"] == g["expected_faces"]


def test_corner_table_non_manifold_topology():
    """src/mesh/corner_table/builder.rs:378-524 -> 192 faces, 100 vertices."""
    g = GOLD["non_manifold_topology"]
    r = ob.corner_table_from_indexed(g["vertices"], g["indices"])
    assert r["faces"] == g["expected_faces"]
    assert r["vertices"] == g["expected_vertices"]
