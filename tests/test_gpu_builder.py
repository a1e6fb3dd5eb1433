"""Parity of Volume::from_fn and VolumeBuilder on the GPU with the oracle
(voxel/volume/mod.rs:40-72, volume/builder.rs:21-76): sphere and cuboid bit
for bit; the IWP surface within a few ulps of cosf."""
import numpy as np
import pytest

import baby_shark_gb300 as bs
from oracle import binding as ob
from tests.gpu_common import compare_volumes, context

pytestmark = pytest.mark.gpu


def assert_identical(g, o):
    rep = compare_volumes(g.export(), o.export(), check_inactive=True)
    assert rep["leaf_set_equal"], rep
    assert rep["mask_mismatch_leaves"] == 0 and rep["value_mismatch"] == 0 and rep["sign_mismatch"] == 0, rep
    assert rep["inactive_mismatch"] == 0, rep
    return rep


@pytest.mark.parametrize("h,r,o", [(0.05, 0.5, (0.1, -0.2, 0.3)), (0.01, 0.77, (-1.3, 0.0, 2.1)),
                                   (0.003, 0.25, (0.0, 0.0, 0.0))])
def test_sphere(h, r, o):
    g = bs.VolumeBuilder(context()).with_voxel_size(h).sphere(r, o)
    rep = assert_identical(g, ob.volume_sphere(np.float32(h), np.float32(r), np.float32(o)))
    assert rep["active"] > 100
    assert g.counts()["active_voxels"] == rep["active"]


@pytest.mark.parametrize("h,mn,mx", [(0.05, (-0.3, -0.2, -0.1), (0.3, 0.25, 0.2)),
                                     (0.01, (-1.0, 0.5, -0.25), (0.35, 0.9, 1.5))])
def test_cuboid(h, mn, mx):
    g = bs.VolumeBuilder(context()).with_voxel_size(h).cuboid(mn, mx)
    assert_identical(g, ob.volume_cuboid(np.float32(h), mn, mx))


def test_iwp_within_ulps():
    h, mn, mx, cell = 0.02, (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), 0.25
    g = bs.VolumeBuilder(context()).with_voxel_size(h).iwp(mn, mx, cell)
    o = ob.volume_iwp(np.float32(h), mn, mx, np.float32(cell))
    go, gv, gm = g.export()
    oo, ov, om = o.export()
    # cosf differs from the host libm by an ulp or two: values agree within a
    # few ulps of the cell-scaled field; the active sets differ at most where
    # |value| sits within that tolerance of the band limit 3h
    gd = {tuple(k): (v, m) for k, v, m in zip(go, gv, gm)}
    od = {tuple(k): (v, m) for k, v, m in zip(oo, ov, om)}
    band = np.float32(3) * np.float32(h)
    tol = 8 * np.finfo(np.float32).eps * cell
    common = set(gd) & set(od)
    assert len(common) > 0.99 * max(len(gd), len(od))
    bad = 0
    for k in common:
        v1, m1 = gd[k]
        v2, m2 = od[k]
        a1 = np.unpackbits(m1.view(np.uint8), bitorder="little").astype(bool)
        a2 = np.unpackbits(m2.view(np.uint8), bitorder="little").astype(bool)
        both = a1 & a2
        assert np.all(np.abs(v1[both] - v2[both]) <= tol)
        diff = a1 ^ a2
        bad += int(np.sum(np.abs(np.abs(np.where(a1, v1, v2)[diff]) - band) > tol))
    assert bad == 0


def test_from_fn_numpy_matches_builder_and_oracle():
    h, r, o = np.float32(0.02), np.float32(0.4), np.array([0.05, 0.1, -0.07], np.float32)

    def f(p):
        d = p - o
        return np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]) - r

    off = np.float32(r + np.float32(1.0) * h)
    g = bs.Volume.from_fn(h, o - off, o + off, 1, f, ctx=context())
    b = bs.VolumeBuilder(context()).with_voxel_size(h).sphere(r, o)
    rep = compare_volumes(g.export(), b.export(), check_inactive=True)
    assert rep["leaf_set_equal"] and rep["value_mismatch"] == 0 and rep["inactive_mismatch"] == 0
    lo = np.floor((o - off) / h).astype(np.int64)
    hi = np.ceil((o + off) / h).astype(np.int64)
    ax = [np.arange(lo[i], hi[i] + 1).astype(np.float32) * h for i in range(3)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    samples = f(np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)).reshape(X.shape)
    assert_identical(g, ob.volume_from_samples(h, 1, lo, samples))


def test_from_fn_torch_device_closure():
    torch = pytest.importorskip("torch")
    h = np.float32(0.025)

    def f(p):
        t = torch.from_numpy(p).cuda()
        return t[:, 0] * 0.5 + t[:, 1] * 0.25 - t[:, 2] * 0.125 - 0.05  # a plane, evaluated on the GPU

    g = bs.Volume.from_fn(h, (-0.3, -0.3, -0.3), (0.3, 0.3, 0.3), 2, f, ctx=context())
    lo = np.floor(np.float32(-0.3) / h).astype(np.int64) * np.ones(3, np.int64)
    hi = np.ceil(np.float32(0.3) / h).astype(np.int64) * np.ones(3, np.int64)
    ax = [np.arange(lo[i], hi[i] + 1).astype(np.float32) * h for i in range(3)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    samples = f(pts).cpu().numpy().reshape(X.shape)
    assert_identical(g, ob.volume_from_samples(h, 2, lo, samples))


def test_builder_boolean_and_offset_chain():
    """examples/boolean.rs-style chain: sphere minus cuboid, then offset."""
    h = np.float32(0.02)
    gs = bs.VolumeBuilder(context()).with_voxel_size(h).sphere(0.5, (0.0, 0.0, 0.0))
    gc = bs.VolumeBuilder(context()).with_voxel_size(h).cuboid((-0.2, -0.2, -0.8), (0.2, 0.2, 0.8))
    os_ = ob.volume_sphere(h, np.float32(0.5), np.zeros(3, np.float32))
    oc = ob.volume_cuboid(h, (-0.2, -0.2, -0.8), (0.2, 0.2, 0.8))
    g = gs.subtract(gc).offset(0.04)
    o = os_.subtract(oc).offset(0.04)
    assert_identical(g, o)


def test_empty_and_invalid():
    with pytest.raises(bs.BsError) as e:
        bs.VolumeBuilder(context()).with_voxel_size(0.0).sphere(1.0, (0, 0, 0))
    assert e.value.status == 1
    far = bs.VolumeBuilder(context()).with_voxel_size(0.5).cuboid((0, 0, 0), (0, 0, 0))
    assert far.counts()["leaves"] >= 1
