"""The seeded synthetic workloads (baby_shark_gb300/synthetic.py): declared
sizes, determinism, and watertight tori (every edge shared by exactly two
triangles, consistently oriented)."""
import numpy as np

from baby_shark_gb300 import synthetic


def edge_use(f):
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    key = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) * (1 << 32) + np.maximum(e[:, 0], e[:, 1])
    _, counts = np.unique(key, return_counts=True)
    directed = e[:, 0].astype(np.int64) * (1 << 32) + e[:, 1]
    return counts, len(np.unique(directed)) == len(directed)


def test_config1_and_config2_sizes():
    v, f = synthetic.config1()
    assert f.shape == (5120, 3) and v.dtype == np.float32 and f.dtype == np.uint32
    (va, fa), (vb, fb) = synthetic.config2()
    assert fa.shape == (1048576, 3) and fb.shape == (1048576, 3)
    counts, oriented = edge_use(fa)
    assert np.all(counts == 2) and oriented  # closed, consistently oriented


def test_generators_are_deterministic():
    a = synthetic.torus(1.0, 0.3, 64, 32, 0.02, seed=9)
    b = synthetic.torus(1.0, 0.3, 64, 32, 0.02, seed=9)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    c = synthetic.torus(1.0, 0.3, 64, 32, 0.02, seed=10)
    assert not np.array_equal(a[0], c[0])
    m1 = synthetic.large_union(3, seed=5, tri_min=2048, tri_max=4096)
    m2 = synthetic.large_union(3, seed=5, tri_min=2048, tri_max=4096)
    for (v1, f1), (v2, f2) in zip(m1, m2):
        assert np.array_equal(v1, v2) and np.array_equal(f1, f2)
        assert 2048 * 0.9 <= len(f1) <= 4096 * 1.1


def test_uneven_batch_ranges():
    batch = synthetic.uneven_batch(12, seed=4)
    assert len(batch) == 12
    for v, f, h in batch:
        extent = float((v.max(axis=0) - v.min(axis=0)).max())
        assert 60 <= extent / h <= 520  # grids between 64^3 and 512^3
        assert 500 <= len(f) <= 600_000
