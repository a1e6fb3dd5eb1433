"""The large combined workload at reduced size: 16 randomly rotated and
placed displaced tori (synthetic.large_union, about 3k triangles each) at
voxel 0.02, converted in one batched call, united pairwise and dual
contoured.  The union (leaves, masks, active and inactive values, active
tiles) equals the oracle's union of its own conversions, and the
dual-contouring triangles equal the oracle's with tiles read through the
tree's `at` (the reference stops at active tiles), bit for bit."""
import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import compare_volumes, context

pytestmark = pytest.mark.gpu

H, BAND = 0.02, 3


def pairwise_union(vols):
    while len(vols) > 1:
        nxt = [vols[i].union(vols[i + 1]) for i in range(0, len(vols) - 1, 2)]
        if len(vols) % 2:
            nxt.append(vols[-1])
        vols = nxt
    return vols[0]


def sorted_tiles(t):
    o, s, v = t
    order = np.lexsort((o[:, 2], o[:, 1], o[:, 0], s))
    return o[order], s[order], v[order].view(np.uint32)


def test_large_union_reduced_matches_oracle():
    meshes = synthetic.large_union(16, seed=5, tri_min=2048, tri_max=4096)
    ctx = context()
    gv = bs.convert_batch(meshes, (H, BAND), ctx)
    assert all(v is not None for v in gv)
    g = pairwise_union(gv)
    o = pairwise_union([ob.mesh_to_volume(v, f, H, BAND)[0] for v, f in meshes])

    rep = compare_volumes(g.export(), o.export(), check_inactive=True)
    assert rep["leaf_set_equal"], rep
    assert rep["mask_mismatch_leaves"] == 0 and rep["value_mismatch"] == 0, rep
    assert rep["sign_mismatch"] == 0 and rep["inactive_mismatch"] == 0, rep
    gt, ot = sorted_tiles(g.tiles()), sorted_tiles(o.tiles())
    assert len(gt[0]) > 0
    for a, b in zip(gt, ot):
        assert np.array_equal(a, b)

    tris = bs.DualContouringMesher().with_voxel_size(H).mesh(g)
    otris, status, _, _ = o.dual_contour(tiles_via_at=True)
    assert status == 0
    assert tris.shape == otris.shape and len(tris) > 10000
    key = lambda t: np.sort(np.ascontiguousarray(t, np.float32).reshape(-1, 9).view(np.uint32).view(
        [("f%d" % i, np.uint32) for i in range(9)]).ravel())
    assert np.array_equal(key(tris), key(otris))
