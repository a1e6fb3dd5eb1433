"""Parity of the CUDA offset (bs_volume_offset: remove |v| > 2h, fast
sweeping, v -= d) with the oracle, and the reference's 7944-vertex golden
value computed on the GPU's own result."""
import json
import os

import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import compare_volumes, context

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def both(v, f, h, band):
    ctx = context()
    g = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(band).convert((v, f))
    o, _, _ = ob.mesh_to_volume(v, f, h, band)
    return g, o


def assert_same(gv, ov):
    rep = compare_volumes(gv.export(), ov.export(), check_inactive=True)
    assert rep["leaf_set_equal"], rep
    assert rep["mask_mismatch_leaves"] == 0, rep
    assert rep["value_mismatch"] == 0, rep
    assert rep["sign_mismatch"] == 0, rep
    assert rep["inactive_mismatch"] == 0, rep
    assert gv.counts()["tiles"] == 0
    assert gv.counts()["active_voxels"] == rep["active"]
    return rep


def box2():
    tris = np.array(GOLD["box2_stl"]["triangles"], np.float32)
    v = tris.reshape(-1, 3)
    return v, np.arange(len(v), dtype=np.uint32).reshape(-1, 3)


def test_volume_offset_golden_7944():
    """src/voxel/volume/mod.rs:134-152 on the GPU: box2.stl, voxel 0.2,
    band 0, offset 0.5 -> 7944 marching-cubes vertices."""
    g = GOLD["volume_offset"]
    v, f = box2()
    gv, ov = both(v, f, g["voxel_size"], 0)
    gv.offset(g["offset"])
    ov.offset(g["offset"])
    assert_same(gv, ov)
    check = ob.volume_from_leaves(*gv.export(), g["voxel_size"])
    n_tri, ambiguous, _ = check.mc_triangles()
    assert ambiguous == 0
    assert 3 * n_tri == g["mc_vertices"]


@pytest.mark.parametrize("d", [0.05, -0.05, 0.013])
def test_icosphere_offsets(d):
    v, f = synthetic.config1()
    gv, ov = both(v, f, 0.02, 3)
    gv.offset(d)
    ov.offset(d)
    assert_same(gv, ov)


@pytest.mark.parametrize("d", [0.03, -0.03])
def test_torus_offsets(d):
    v, f = synthetic.torus(1.0, 0.3, 128, 64, 0.02, seed=2)
    gv, ov = both(v, f, 0.01, 3)
    gv.offset(d)
    ov.offset(d)
    assert_same(gv, ov)


def test_offset_after_boolean():
    va, fa = synthetic.torus(1.0, 0.3, 96, 48, 0.02, seed=2)
    vb, fb = synthetic.torus(1.0, 0.3, 96, 48, 0.02, seed=3, rotate_x_deg=90.0, shift=(0.5, 0.0, 0.0))
    ga, oa = both(va, fa, 0.012, 3)
    gb, ob_ = both(vb, fb, 0.012, 3)
    g = ga.subtract(gb).offset(0.024)
    o = oa.subtract(ob_).offset(0.024)
    assert_same(g, o)
    g2 = g.offset(-0.024)
    o2 = o.offset(-0.024)
    assert_same(g2, o2)
