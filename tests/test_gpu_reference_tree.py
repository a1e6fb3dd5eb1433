"""The reference's winding-number tree on the GPU (ref_tree.cu) against the
oracle's restatement of AABBTree::top_down::<Area> and fast_wn
(aabb_tree.rs:118-199, 422-514, 636-691).

Same tree and same traversal mean the same work: the number of far-field
evaluations and of exact triangle solid angles must equal the oracle's
exactly (they depend on every node's dipole centre and radius, bit for bit,
and on every triangle's leaf).  The values then differ only through
last-place differences between CUDA's atan2f and the host C library's: most
are bit-identical and the rest within a few float32 ulps of the sum."""
import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import synthetic
from oracle import binding as ob
from tests.gpu_common import context

pytestmark = pytest.mark.gpu


def band_points(v, f, h, band, n, seed):
    vol = bs.MeshToVolume(context()).with_voxel_size(h).with_narrow_band_width(band).convert((v, f))
    o, _, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    li, vi = np.nonzero(act)
    pick = np.random.default_rng(seed).choice(len(li), min(n, len(li)), replace=False)
    vox = o[li[pick]] + np.stack([vi[pick] >> 6, (vi[pick] >> 3) & 7, vi[pick] & 7], 1)
    return (vox.astype(np.float32) * np.float32(h)).astype(np.float32)


def check_against_oracle(v, f, pts, beta=2.0):
    ctx = context()
    wn = bs.WindingNumbers.from_mesh((v, f), ctx=ctx, tree="reference")
    g = wn.approximate(pts, beta)
    st = ctx.last_stats()
    o, cnt = ob.fast_wn(v, f, pts, beta)
    assert st["wn_warp_far"] == cnt["far_evals"] & 0xffffffff
    assert st["wn_warp_exact"] == cnt["leaf_tri_evals"]
    same = g.view(np.uint32) == o.view(np.uint32)
    diff = np.abs(g.astype(np.float64) - o.astype(np.float64))
    # the only operation whose float32 result may differ is atan2f (CUDA's
    # against the host C library's, last place): most values are
    # bit-identical and the rest differ by a few float32 ulps of the sum
    assert same.mean() > 0.75, same.mean()
    assert diff.max() <= 2e-6, diff.max()
    return same.mean(), diff.max()


@pytest.mark.parametrize("subdiv,holes", [(3, 0.1), (5, 0.1), (5, 0.0)])
def test_values_and_work_match_oracle(subdiv, holes):
    v, f = synthetic.icosphere(subdiv, 1.0, 0.04, seed=subdiv)
    if holes:
        f = synthetic.remove_faces(f, holes, seed=7)
    rng = np.random.default_rng(subdiv)
    pts = np.concatenate([band_points(v, f, 0.02, 3, 20000, subdiv),
                          rng.uniform(-1.5, 1.5, (20000, 3)).astype(np.float32)])
    check_against_oracle(v, f, pts)


def test_torus_slice_with_ties_and_large_levels():
    """An open slice of a torus (grid-aligned parametrisation: many equal box
    centres) of 65,536 triangles, past the build's per-CTA node size."""
    v, f = synthetic.torus(1.0, 0.3, 256, 256, 0.02, seed=3)
    f = f[(f[:, 0] // 256) < 64]
    rng = np.random.default_rng(2)
    pts = np.concatenate([band_points(v, f, 0.01, 2, 20000, 4),
                          rng.uniform(-1.4, 1.4, (10000, 3)).astype(np.float32)])
    check_against_oracle(v, f, pts)


def test_coincident_triangles_make_one_large_leaf():
    """600 copies of a triangle plus a few others: no axis splits the copies
    (all centres coincide), so they form one leaf whose order follows the
    reference's stable sorts (the build's large-leaf path)."""
    base = np.array([[0.1, 0.2, 0.3], [0.4, 0.25, 0.3], [0.2, 0.6, 0.35]], np.float32)
    rng = np.random.default_rng(5)
    other = rng.uniform(-1, 1, (50, 3, 3)).astype(np.float32)
    tri = np.concatenate([np.repeat(base[None], 600, axis=0), other])
    v = tri.reshape(-1, 3)
    f = np.arange(len(v), dtype=np.uint32).reshape(-1, 3)
    pts = rng.uniform(-1.2, 1.2, (5000, 3)).astype(np.float32)
    check_against_oracle(v, f, pts)


def test_tiny_meshes():
    """Root leaves (1 to 3 triangles) and a 4-triangle mesh."""
    rng = np.random.default_rng(9)
    for n in (1, 2, 3, 4, 7):
        tri = rng.uniform(-1, 1, (n, 3, 3)).astype(np.float32)
        v = tri.reshape(-1, 3)
        f = np.arange(len(v), dtype=np.uint32).reshape(-1, 3)
        pts = rng.uniform(-1.5, 1.5, (2000, 3)).astype(np.float32)
        check_against_oracle(v, f, pts)
