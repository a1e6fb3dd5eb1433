"""The CUDA marching-cubes mesher (bs_marching_cubes) against the oracle's
restatement of the same tiling (oracle/oracle_mc.hpp) bit for bit as a
triangle multiset, and against the reference's 7944-vertex golden value
(voxel/volume/mod.rs:134-152) entirely on the GPU."""
import json
import os

import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import context

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def tri_multiset(tris):
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 9).view(np.uint32)
    return t[np.lexsort(t.T[::-1])]


def both(v, f, h, band):
    ctx = context()
    g = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(band).convert((v, f))
    o, _, _ = ob.mesh_to_volume(v, f, h, band)
    return g, o


def assert_same(gv, ov, h):
    gt = bs.MarchingCubesMesher().with_voxel_size(h).mesh(gv)
    ot = ov.marching_cubes(h)
    assert gt.shape == ot.shape, (gt.shape, ot.shape)
    assert np.array_equal(tri_multiset(gt), tri_multiset(ot))
    return gt


def test_golden_7944_on_gpu():
    g = GOLD["volume_offset"]
    tris = np.array(GOLD["box2_stl"]["triangles"], np.float32).reshape(-1, 3)
    idx = np.arange(len(tris), dtype=np.uint32).reshape(-1, 3)
    gv = bs.MeshToVolume(context()).with_voxel_size(g["voxel_size"]).with_narrow_band_width(0).convert((tris, idx))
    gv.offset(g["offset"])
    gt = bs.MarchingCubesMesher().with_voxel_size(g["voxel_size"]).mesh(gv)
    assert 3 * len(gt) == g["mc_vertices"]


def test_icosphere_config1():
    v, f = synthetic.config1()
    gv, ov = both(v, f, 0.02, 3)
    gt = assert_same(gv, ov, 0.02)
    assert len(gt) > 10000


def test_torus_band0_and_offset():
    v, f = synthetic.torus(1.0, 0.3, 128, 64, 0.02, seed=2)
    gv, ov = both(v, f, 0.01, 0)
    assert_same(gv, ov, 0.01)
    gv.offset(-0.02)
    ov.offset(-0.02)
    assert_same(gv, ov, 0.01)


def test_builder_sphere_and_cache():
    h = np.float32(0.01)
    g = bs.VolumeBuilder(context()).with_voxel_size(h).sphere(0.31, (0.02, -0.01, 0.0))
    o = ob.volume_sphere(h, np.float32(0.31), np.array([0.02, -0.01, 0.0], np.float32))
    a = assert_same(g, o, h)
    b = bs.MarchingCubesMesher().with_voxel_size(h).mesh(g)  # cached result
    assert np.array_equal(a, b)
    g.offset(0.02)  # invalidates the cache
    o.offset(0.02)
    assert_same(g, o, h)


def test_union_with_tiles():
    """A union with active inside tiles: the tiles' boundary cubes are meshed
    (marching_cubes.rs:969-994) and the result equals the oracle's."""
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
    gt = assert_same(u, ou, 0.02)
    assert len(gt) > 1000


def test_voxel_remesher_manifold_default():
    v, f = synthetic.config1()
    r = bs.VoxelRemesher(context()).with_voxel_size(0.02)  # Manifold, band 0: the reference's defaults
    ct = r.remesh((v, f))
    o, _, _ = ob.mesh_to_volume(v, f, 0.02, 0)
    soup = o.marching_cubes(0.02)
    assert (ct.faces_count(), ct.vertices_count()) == ob.corner_table_from_soup(soup.reshape(-1, 3))
