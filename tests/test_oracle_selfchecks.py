"""Self-checks of the oracle against independent float64 evaluations, on the
CPU: the restatement's distances, signs and fast winding numbers are compared
with direct float64 computations (exact point-triangle distance over all
candidate sub-triangles; direct-sum winding number over all triangles), so
that the oracle is checked against the mathematics as well as against the
reference's known-answer tests.  Workload: the 5,120-triangle displaced
icosphere at voxel 0.02, band 3."""
import numpy as np
import pytest

import oracle.binding as ob
from baby_shark_gb300 import synthetic
from tests.f64_distance import min_distance_f64

H, BAND = 0.02, 3


@pytest.fixture(scope="module")
def icosphere_volume():
    ob.build()
    v, f = synthetic.config1()
    vol, stats, wn = ob.mesh_to_volume(v, f, H, BAND, with_wn=True)
    o, val, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    li, vi = np.nonzero(act)
    vox = o[li].astype(np.int64) + np.stack([vi >> 6, (vi >> 3) & 7, vi & 7], 1)
    return v, f, vox, val[li, vi], stats


def test_signs_match_exact_winding_numbers(icosphere_volume):
    """Watertight mesh: every band voxel's sign (wn < 0.2 outside,
    mesh_to_volume.rs:264-271) equals the one the exact float64 winding
    number gives, and the exact values sit at 0 or 1."""
    v, f, vox, val, stats = icosphere_volume
    assert stats["band_voxels"] == len(vox)
    pick = np.random.default_rng(1).choice(len(vox), 40_000, replace=False)
    pts = (vox[pick].astype(np.float32) * np.float32(H)).astype(np.float32)
    ex = ob.exact_wn_f64(v, f, pts)
    assert np.all((np.abs(ex) < 0.01) | (np.abs(ex - 1.0) < 0.01))
    assert np.array_equal(np.signbit(val[pick]), ex >= 0.2)


def test_fast_winding_number_error_against_direct_sum():
    """The oracle's fast winding number (order-2 far field, beta 2,
    aabb_tree.rs:662-691) stays within its approximation error of the
    float64 direct sum at points anywhere around the mesh, and a larger
    beta (fewer far-field evaluations accepted) reduces that error."""
    ob.build()
    v, f = synthetic.config1()
    pts = np.random.default_rng(2).uniform(-1.3, 1.3, (20_000, 3)).astype(np.float32)
    ex = ob.exact_wn_f64(v, f, pts)
    w2, c2 = ob.fast_wn(v, f, pts, 2.0)
    w4, c4 = ob.fast_wn(v, f, pts, 4.0)
    e2, e4 = np.abs(w2 - ex), np.abs(w4 - ex)
    assert e2.max() < 0.1 and e2.mean() < 0.01
    assert e4.mean() < 0.5 * e2.mean() and c4["far_evals"] > 0
    # the far field is used at all (not a direct sum in disguise)
    assert c2["far_evals"] > c2["leaf_tri_evals"]


def test_distances_against_float64(icosphere_volume):
    """Stored |values| are the float32 minimum over the voxel's candidate
    sub-triangles (mesh_to_volume.rs:147-195); against the same minimum in
    float64 they differ by float32 rounding only (< 1e-5 voxel)."""
    v, f, vox, val, _ = icosphere_volume
    pick = np.random.default_rng(3).choice(len(vox), 300, replace=False)
    sub, box = ob.subtriangles(v, f, H, BAND)
    d64 = min_distance_f64(vox[pick], H, sub, box)
    assert np.all(np.isfinite(d64))
    err = np.abs(np.abs(val[pick]).astype(np.float64) - d64) / H
    assert err.max() < 1e-5
