"""The oracle's Volume::from_fn / VolumeBuilder restatement (no GPU): the
sampled from_fn path and the sphere builder agree bit for bit, and the
sphere's active voxels are the grid points within 2h of the surface."""
import numpy as np

from oracle import binding as ob


def test_from_samples_equals_sphere_builder():
    h, r, o = np.float32(0.05), np.float32(0.5), np.array([0.1, -0.2, 0.3], np.float32)
    s = ob.volume_sphere(h, r, o)
    off = np.float32(r + np.float32(1.0) * h)
    lo = np.floor((o - off) / h).astype(np.int64)
    hi = np.ceil((o + off) / h).astype(np.int64)
    ax = [np.arange(lo[i], hi[i] + 1).astype(np.float32) * h for i in range(3)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    d = [X - o[0], Y - o[1], Z - o[2]]
    val = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) - r
    t = ob.volume_from_samples(h, 1, lo, val.astype(np.float32))
    (o1, v1, m1), (o2, v2, m2) = s.export(), t.export()
    assert np.array_equal(o1, o2) and np.array_equal(m1, m2)
    assert np.array_equal(v1.view(np.uint32), v2.view(np.uint32))
    n_active = int(np.unpackbits(m1.view(np.uint8)).sum())
    assert n_active == int(np.sum(np.abs(val) <= np.float32(2) * h))


def test_cuboid_inside_negative():
    h = np.float32(0.05)
    c = ob.volume_cuboid(h, (-0.3, -0.2, -0.1), (0.3, 0.25, 0.2))
    o, v, m = c.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    vals = v[act]
    assert (vals < 0).any() and (vals > 0).any()
    assert np.all(np.abs(vals) <= np.float32(2) * h)
