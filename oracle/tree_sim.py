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

    python oracle/tree_sim.py
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
    (64, 1, 0),  # binned SAH down to 64-triangle segments, PLOC inside
    (64, 1, 2),
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


def main():
    ob.build()
    out = os.path.join(HERE, "_build", "tree_sim")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "tree_sim")
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-o", exe,
                           os.path.join(HERE, "tree_sim.cpp")])
    (v, f), _ = synthetic.config2()
    files = [os.path.join(out, n) for n in ("v.f32", "t.u32", "w.f32")]
    v.astype(np.float32).tofile(files[0])
    f.astype(np.uint32).tofile(files[1])
    warps_of_band(v, f).tofile(files[2])
    for s, leafmax, radius in VARIANTS:
        subprocess.check_call([exe, *files, str(s), str(leafmax), str(radius)])


if __name__ == "__main__":
    main()
