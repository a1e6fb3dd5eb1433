"""ORACLE — test infrastructure only: counts the work of the reference's own
winding-number traversal per band voxel on the headline workload, the
algorithmic unit of the sign kernel's roofline.

The reference's tree (the `Area` SAH tree, aabb_tree.rs:118-199, 422-514) is
built over all 1,048,576 triangles of the first torus; the queries are the
band voxels (voxel 0.002, band 3) of the oracle's conversion of the first
1/16 of its ring (a uniform slice of a rotationally uniform surface, 4.5 M
voxels); every query runs fast_wn at accuracy scale 2
(aabb_tree.rs:662-691).  Prints far-field evaluations and exact leaf
triangles per voxel.

    python oracle/traversal_counts.py
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from baby_shark_gb300 import synthetic  # noqa: E402
from oracle import binding as ob  # noqa: E402


def main():
    ob.build()
    (v, f), _ = synthetic.config2()
    n = len(f) // 16
    vol, stats, _ = ob.mesh_to_volume(v, f[:n], 0.002, 3)
    o, _, m = vol.export()
    act = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(len(o), 512).astype(bool)
    li, vi = np.nonzero(act)
    vox = o[li].astype(np.int64) + np.stack([vi >> 6, (vi >> 3) & 7, vi & 7], 1)
    pts = (vox.astype(np.float32) * np.float32(0.002)).astype(np.float32)
    _, c = ob.fast_wn(v, f, pts, 2.0)
    print("band voxels %d; per voxel: far-field evaluations %.2f, exact leaf triangles %.2f (tree nodes %d)"
          % (len(pts), c["far_evals"] / len(pts), c["leaf_tri_evals"] / len(pts), c["nodes"]))


if __name__ == "__main__":
    main()
