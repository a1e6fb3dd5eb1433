"""Parity of the CUDA booleans (bs_volume_union / subtract / intersect) with
the oracle: flood fill of both operands, then the tree CSG with tiles
(voxel/volume/mod.rs:74-93).  Every leaf value (active and flood-filled
inactive) and every active tile must match bit for bit."""
import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import compare_volumes, context

pytestmark = pytest.mark.gpu


def both(v, f, h, band):
    ctx = context()
    g = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(band).convert((v, f))
    o, _, _ = ob.mesh_to_volume(v, f, h, band)
    return g, o


def tile_set(origins, sizes, values):
    return {(tuple(int(c) for c in o), int(s), int(np.float32(val).view(np.uint32))) for o, s, val in
            zip(origins, sizes, values)}


def assert_same(gv, ov):
    rep = compare_volumes(gv.export(), ov.export(), check_inactive=True)
    assert rep["leaf_set_equal"], rep
    assert rep["mask_mismatch_leaves"] == 0, rep
    assert rep["value_mismatch"] == 0, rep
    assert rep["sign_mismatch"] == 0, rep
    assert rep["inactive_mismatch"] == 0, rep
    assert tile_set(*gv.tiles()) == tile_set(*ov.tiles())
    assert gv.counts()["active_voxels"] == rep["active"]
    return rep


def spheres(h=0.02, band=3):
    va, fa = synthetic.icosphere(3, 0.6, 0.02, seed=11)
    vb, fb = synthetic.icosphere(3, 0.5, 0.02, seed=12)
    vb = vb + np.array([0.45, 0.1, -0.05], np.float32)
    return both(va, fa, h, band), both(vb, fb, h, band)


@pytest.mark.parametrize("op", ["union", "subtract", "intersect"])
def test_spheres(op):
    (ga, oa), (gb, ob_) = spheres()
    g = getattr(ga, op)(gb)
    o = getattr(oa, op)(ob_)
    rep = assert_same(g, o)
    assert rep["active"] > 0


@pytest.mark.parametrize("op", ["union", "subtract", "intersect"])
def test_crossing_tori(op):
    """The boolean workload's two tori at a coarser grid (128 x 64, voxel 0.01)."""
    va, fa = synthetic.torus(1.0, 0.3, 128, 64, 0.02, seed=2)
    vb, fb = synthetic.torus(1.0, 0.3, 128, 64, 0.02, seed=3, rotate_x_deg=90.0, shift=(0.5, 0.0, 0.0))
    ga, oa = both(va, fa, 0.01, 3)
    gb, ob_ = both(vb, fb, 0.01, 3)
    g = getattr(ga, op)(gb)
    o = getattr(oa, op)(ob_)
    assert_same(g, o)


def test_nested_inside_tiles():
    """A small sphere deep inside a large one: the union keeps the outer band
    and replaces nothing; subtracting the big one from the small gives an
    empty band; intersect keeps the small one."""
    v1, f1 = synthetic.icosphere(3, 0.9, 0.0, seed=1)
    v2, f2 = synthetic.icosphere(2, 0.2, 0.0, seed=2)
    for op in ("union", "subtract", "intersect"):
        ga, oa = both(v1, f1, 0.01, 2)
        gb, ob_ = both(v2, f2, 0.01, 2)
        g = getattr(ga, op)(gb)
        o = getattr(oa, op)(ob_)
        assert_same(g, o)


def test_chained_ops():
    (ga, oa), (gb, ob_) = spheres()
    vc, fc = synthetic.icosphere(2, 0.3, 0.01, seed=13)
    vc = vc + np.array([-0.3, 0.2, 0.35], np.float32)
    gc, oc = both(vc, fc, 0.02, 3)
    g = ga.union(gb).subtract(gc)
    o = oa.union(ob_).subtract(oc)
    assert_same(g, o)
    # a second boolean on a volume that already holds tiles
    (gd, od), (ge, oe) = spheres(0.02, 2)
    g2 = g.intersect(gd.union(ge))
    o2 = o.intersect(od.union(oe))
    assert_same(g2, o2)


def test_consumed_operands():
    (ga, _), (gb, _) = spheres()
    g = ga.union(gb)
    with pytest.raises(ValueError):
        ga.union(g)


@pytest.mark.parametrize("op", ["union", "subtract", "intersect"])
@pytest.mark.parametrize("empty_side", ["a", "b", "both"])
def test_boolean_with_empty_volume(op, empty_side):
    """Volume::with_voxel_size (volume/mod.rs:17-24) as either operand: the
    reference's root-level CSG (root_node/csg.rs:9-58) keeps the other
    operand's nodes for union (and for subtraction of an empty volume) and
    nothing for intersection; every leaf, flood-filled value and tile equals
    the oracle's."""
    v, f = synthetic.icosphere(3, 0.6, 0.02, seed=11)
    ctx = context()
    h = 0.02
    full_g = bs.MeshToVolume(ctx).with_voxel_size(h).with_narrow_band_width(2).convert((v, f))
    full_o, _, _ = ob.mesh_to_volume(v, f, h, 2)
    empty_g = lambda: bs.Volume.with_voxel_size(h, ctx)  # noqa: E731
    empty_o = lambda: ob.volume_from_leaves(np.zeros((0, 3), np.int32), np.zeros((0, 512), np.float32),  # noqa: E731
                                            np.zeros((0, 16), np.uint32), h)
    ga, gb = (empty_g(), full_g) if empty_side == "a" else (full_g, empty_g()) if empty_side == "b" else \
        (empty_g(), empty_g())
    oa, obb = (empty_o(), full_o) if empty_side == "a" else (full_o, empty_o()) if empty_side == "b" else \
        (empty_o(), empty_o())
    g = getattr(ga, op)(gb)
    o = getattr(oa, op)(obb)
    rep = compare_volumes(g.export(), o.export(), check_inactive=True)
    assert rep["leaf_set_equal"] and rep["mask_mismatch_leaves"] == 0, rep
    assert rep["value_mismatch"] == 0 and rep["sign_mismatch"] == 0 and rep["inactive_mismatch"] == 0, rep
    go, gs, gt = g.tiles()
    oo, os_, ot = o.tiles()
    assert sorted(zip(map(tuple, go.tolist()), gs.tolist())) == sorted(zip(map(tuple, oo.tolist()), os_.tolist()))
    expect_full = (op == "union" and empty_side != "both") or (op == "subtract" and empty_side == "b")
    assert (g.counts()["leaves"] > 0) == expect_full
    # the empty volume through the rest of the path
    e = bs.Volume.with_voxel_size(h, ctx)
    e.offset(0.05)
    assert e.counts()["leaves"] == 0
    assert bs.DualContouringMesher().with_voxel_size(h).mesh(e).size == 0
