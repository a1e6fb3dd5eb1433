"""ORACLE — test infrastructure only (an analysis tool): ranks winding-number
tree designs for the sign pass by the work of its warp-coherent traversal,
with oracle/tree_sim.cpp (a CPU restatement of the library's tree build and
traversal, plus binned-SAH and radius variants).

Workload: the first torus of the headline workload (1,048,576 triangles) and
warps of its band voxels (voxel 0.002, band 3) as the sign pass forms them:
the band of the oracle's conversion of a 1/16 ring slice, bricks in
(x, y, z) order, the active voxels of a brick in Morton order, 32 consecutive
voxels a warp; 20,000 warps drawn at random (seed 1).  Prints one line per
tree variant.

With --accuracy it instead takes every band voxel of two open icospheres
(subdivision 3, voxel 0.03, band 2; subdivision 5, voxel 0.01, band 3; 10 %
of the faces removed), writes each lane's winding number and compares it
with the oracle's own traversal (the reference's tree) and with exact
values: mean and largest error, sign flips against the oracle, flips where
the oracle's value lies 0.01 or more from the 0.2 threshold, and sign
differences from exact values.

    python oracle/tree_sim.py [--accuracy]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from baby_shark_gb300 import synthetic  # noqa: E402
from oracle import binding as ob  # noqa: E402

VARIANTS = [  # (S, leafmax, radius): see tree_sim.cpp
    (0, 1, 0),   # the library's tree today: PLOC, its radius rule
    (0, 1, 2),   # PLOC, farthest-vertex radii
    (1, 3, 1),   # the reference's SAH tree (leaves of up to 3 triangles, box-bound radii)
    (1, 3, 2),   # the same with farthest-vertex radii
    (1, 1, 1),   # SAH with one-triangle leaves
    (1, 1, 2),
    (1, 3, 0),   # SAH with the library's radius rule
    (64, 1, 0),  # binned SAH down to 64-triangle segments, PLOC inside
    (64, 1, 2),
    (64, 3, 0),  # the same with subtrees of up to 3 triangles as leaves
    (1024, 1, 0),
]


def morton9(off):
    x, y, z = off >> 6, (off >> 3) & 7, off & 7
    m = np.zeros_like(off)
    for b in range(3):
        m |= (((z >> b) & 1) << (3 * b)) | (((y >> b) & 1) << (3 * b + 1)) | (((x >> b) & 1) << (3 * b + 2))
    return m


def warps_of_band(v, f, h=0.002, band=3, n_warps=20000, seed=1):
    vol, _, _ = ob.mesh_to_volume(v, f[: len(f) // 16], h, band)
    o, _, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    order = np.argsort(morton9(np.arange(512)))
    pts = []
    for b in np.lexsort((o[:, 2], o[:, 1], o[:, 0])):
        sel = order[act[b][order]]
        pts.append(o[b][None, :] + np.stack([sel >> 6, (sel >> 3) & 7, sel & 7], 1))
    p = np.concatenate(pts)
    w = (p[: len(p) // 32 * 32].astype(np.float32) * np.float32(h)).astype(np.float32).reshape(-1, 32, 3)
    return w[np.random.default_rng(seed).choice(len(w), n_warps, replace=False)]


ACCURACY_VARIANTS = [(0, 1, 0), (0, 1, 2), (64, 1, 0), (64, 3, 0), (1, 3, 1), (1, 3, 0), (1, 3, 2)]


def band_warps(v, f, h, band):
    """Every band voxel of the oracle's conversion in the sign pass's warp
    order (the last warp padded with its last voxel), with the oracle's own
    winding number of each."""
    vol, _, wn = ob.mesh_to_volume(v, f, h, band, with_wn=True)
    o, _, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    w_all = np.zeros(act.shape, np.float32)
    w_all[act] = wn  # the oracle's order: leaves as exported, voxels by index
    order = np.argsort(morton9(np.arange(512)))
    pts, ref = [], []
    for b in np.lexsort((o[:, 2], o[:, 1], o[:, 0])):
        sel = order[act[b][order]]
        pts.append(o[b][None, :] + np.stack([sel >> 6, (sel >> 3) & 7, sel & 7], 1))
        ref.append(w_all[b][sel])
    p, ref = np.concatenate(pts), np.concatenate(ref)
    p = np.concatenate([p, np.repeat(p[-1:], (-len(p)) % 32, 0)])
    return (p.astype(np.float32) * np.float32(h)).astype(np.float32), ref


def accuracy(exe, out):
    cases = [(synthetic.icosphere(3, 0.8, 0.05, seed=3), (4,), 0.03, 2),
             (synthetic.icosphere(5, 0.8, 0.05, seed=5), (6,), 0.01, 3)]
    for (v, f), (seed,), h, band in cases:
        f = synthetic.remove_faces(f, 0.1, seed=seed)
        pts, ref = band_warps(v, f, h, band)
        n = len(ref)
        exact = ob.exact_wn_f64(v, f, pts[:n])
        files = [os.path.join(out, name) for name in ("av.f32", "at.u32", "aw.f32", "vals.f32")]
        v.astype(np.float32).tofile(files[0])
        f.astype(np.uint32).tofile(files[1])
        pts.tofile(files[2])
        print("open icosphere, %d triangles, voxel %g, band %d: %d band voxels; oracle vs exact: mean %.2e"
              % (len(f), h, band, n, np.abs(ref - exact).mean()))
        for s, leafmax, radius in ACCURACY_VARIANTS:
            subprocess.check_call([exe, *files[:3], str(s), str(leafmax), str(radius), files[3]],
                                  stdout=subprocess.DEVNULL)
            g = np.fromfile(files[3], np.float32)[:n]
            flips = (g < 0.2) != (ref < 0.2)
            print("  S %d leafmax %d radius %d: error vs exact mean %.2e max %.2e; flips vs oracle %d, "
                  "%d with the oracle's value >= 0.01 from 0.2; sign differences from exact %d"
                  % (s, leafmax, radius, np.abs(g - exact).mean(), np.abs(g - exact).max(), flips.sum(),
                     (flips & (np.abs(ref - 0.2) >= 0.01)).sum(), ((g < 0.2) != (exact < 0.2)).sum()))


def main():
    ob.build()
    out = os.path.join(HERE, "_build", "tree_sim")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "tree_sim")
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-o", exe,
                           os.path.join(HERE, "tree_sim.cpp")])
    if "--accuracy" in sys.argv[1:]:
        accuracy(exe, out)
        return
    (v, f), _ = synthetic.config2()
    files = [os.path.join(out, n) for n in ("v.f32", "t.u32", "w.f32")]
    v.astype(np.float32).tofile(files[0])
    f.astype(np.uint32).tofile(files[1])
    warps_of_band(v, f).tofile(files[2])
    for s, leafmax, radius in VARIANTS:
        subprocess.check_call([exe, *files, str(s), str(leafmax), str(radius)])


if __name__ == "__main__":
    main()
