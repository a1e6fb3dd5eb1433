"""bs_mesh_to_volume_batch: many meshes in one set of launches.  Every volume
of a batch equals the one bs_mesh_to_volume builds for that mesh alone, bit
for bit (leaf set, masks, active and inactive values with their signs) —
each mesh keeps its own full-precision LBVH — and the single calls are the
oracle-checked path."""
import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import compare_volumes, context

pytestmark = pytest.mark.gpu


def single(mesh, h, band):
    return bs.MeshToVolume(context()).with_voxel_size(h).with_narrow_band_width(band).convert(mesh)


def assert_equal(a, b):
    (o1, v1, m1), (o2, v2, m2) = a.export(), b.export()
    assert np.array_equal(o1, o2)
    assert np.array_equal(m1, m2)
    assert np.array_equal(v1.view(np.uint32), v2.view(np.uint32))
    assert a.counts() == b.counts()


def test_mixed_batch_equals_single_calls():
    ico = synthetic.config1()
    tor = synthetic.torus(1.0, 0.3, 96, 48, 0.02, seed=2)
    v, f = synthetic.icosphere(3, 0.7, 0.03, seed=5)
    open_ico = (v, synthetic.remove_faces(f, 0.1, seed=6))
    one = (np.array([[0, 0, 0], [0.3, 0, 0], [0, 0.2, 0.1]], np.float32), np.array([[0, 1, 2]], np.uint32))
    empty = (np.zeros((3, 3), np.float32), np.zeros((0, 3), np.uint32))
    meshes = [ico, tor, empty, one, open_ico]
    params = [(0.02, 3), (0.01, 2), (0.05, 1), (0.01, 2), (0.03, 1)]
    vols = bs.convert_batch(meshes, params, ctx=context())
    assert vols[2] is None
    for m, (h, band), vol in zip(meshes, params, vols):
        if vol is None:
            continue
        assert_equal(vol, single(m, h, band))
    # and the oracle agrees with the batched watertight icosphere
    o, _, _ = ob.mesh_to_volume(ico[0], ico[1], 0.02, 3)
    rep = compare_volumes(vols[0].export(), o.export(), check_inactive=True)
    assert rep["leaf_set_equal"] and rep["value_mismatch"] == 0 and rep["sign_mismatch"] == 0


def test_uneven_batch_equals_single_calls():
    batch = synthetic.uneven_batch(12, seed=9)
    vols = bs.convert_batch([(v, f) for v, f, _ in batch], [(h, 3) for _, _, h in batch], ctx=context())
    for (v, f, h), vol in zip(batch, vols):
        assert_equal(vol, single((v, f), h, 3))


def test_batch_rejects_bad_index():
    v, f = synthetic.icosphere(2, 1.0, 0.0, seed=1)
    bad = f.copy()
    bad[3, 1] = len(v) + 5
    with pytest.raises(bs.BsError) as e:
        bs.convert_batch([(v, f), (v, bad)], (0.05, 2), ctx=context())
    assert e.value.status == 1
