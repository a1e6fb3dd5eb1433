"""Extract the reference's known-answer tests into tests/golden/reference_kats.json.

The reference crate (baby_shark v0.3.12) is Rust and cannot be built here, so
its unit tests are read as text: the literal inputs and expected values of
the tests that pin the implicit-modelling path are copied into a JSON fixture
that the oracle tests replay.  Run from the repository root:

    python tests/golden/make_reference_kats.py /path/to/baby_shark

Sources (paths inside the reference tree):
  assets/box2.stl                                 mesh of test_volume_offset
  src/voxel/volume/mod.rs        test_volume_offset (voxel 0.2, offset 0.5, 7944)
  src/voxel/leaf_node/csg.rs     test_union / test_subtract / test_intersect
  src/voxel/init.rs              test_static_vdb_macro_5_4_3 constants
  src/mesh/corner_table/builder.rs  from_vertices_and_indices,
                                  should_remove_face_that_introduces_non_manifold_edge,
                                  should_fix_non_manifold_topology
  src/mesh/corner_table/test_helpers.rs  create_unit_square_mesh
"""
import json
import os
import re
import struct
import sys

NUM = r"-?\d+(?:\.\d+)?(?:[eE][-+]?\d+)?"


def read_stl(path):
    with open(path, "rb") as f:
        data = f.read()
    n = struct.unpack_from("<I", data, 80)[0]
    tris = []
    for i in range(n):
        off = 84 + 50 * i
        v = struct.unpack_from("<12f", data, off)
        tris.append([list(v[3:6]), list(v[6:9]), list(v[9:12])])
    return tris


def fn_body(src, name):
    i = src.index("fn " + name)
    j = src.index("{", i)
    depth, k = 0, j
    while True:
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[j:k + 1]
        k += 1


def floats(s):
    return [float(x) for x in re.findall(NUM, s)]


def line_of(src, needle):
    return src[: src.index(needle)].count("\n") + 1


def main(ref):
    out = {"source": "baby_shark v0.3.12 unit tests, read as text"}
    out["box2_stl"] = {"file": "assets/box2.stl", "triangles": read_stl(os.path.join(ref, "assets/box2.stl"))}

    vol = open(os.path.join(ref, "src/voxel/volume/mod.rs")).read()
    body = fn_body(vol, "test_volume_offset")
    out["volume_offset"] = {
        "file": "src/voxel/volume/mod.rs:%d" % line_of(vol, "fn test_volume_offset"),
        "voxel_size": float(re.search(r"with_voxel_size\((" + NUM + r")\)", body).group(1)),
        "offset": float(re.search(r"\.offset\((" + NUM + r")\)", body).group(1)),
        "mc_vertices": int(re.search(r"vertices\.len\(\),\s*(\d+)", body).group(1)),
    }

    csg = open(os.path.join(ref, "src/voxel/leaf_node/csg.rs")).read()
    out["leaf_csg"] = {}
    for op in ("union", "subtract", "intersect"):
        b = fn_body(csg, "test_" + op)
        arrs = re.findall(r"\[([^\[\]]*)\]", b)
        arrs = [floats(a) for a in arrs if len(floats(a)) == 8]
        out["leaf_csg"][op] = {
            "file": "src/voxel/leaf_node/csg.rs:%d" % line_of(csg, "fn test_" + op),
            "a": arrs[0], "b": arrs[1], "expected": arrs[2],
        }

    init = open(os.path.join(ref, "src/voxel/init.rs")).read()
    b = fn_body(init, "test_static_vdb_macro_5_4_3")
    out["tree_constants"] = {
        "file": "src/voxel/init.rs:%d" % line_of(init, "fn test_static_vdb_macro_5_4_3"),
        "asserts": [[m[0], int(m[1])] for m in re.findall(r"assert_eq!\((\w+::\w+),\s*(\d+)\)", b)],
    }

    bld = open(os.path.join(ref, "src/mesh/corner_table/builder.rs")).read()
    helpers = open(os.path.join(ref, "src/mesh/corner_table/test_helpers.rs")).read()
    hb = fn_body(helpers, "create_unit_square_mesh")
    sq_verts = [floats(m) for m in re.findall(r"Vec3f::new\(([^)]*)\)", hb)]
    sq_idx = [int(x) for x in re.search(r"indices = vec!\[([^\]]*)\]", hb).group(1).split(",")]
    b = fn_body(bld, "from_vertices_and_indices")
    exp_v = [(int(c), floats(p)) for c, p in re.findall(r"Vertex::new\(CornerId::new\((\d+)\),\s*Vec3f::new\(([^)]*)\)\)", b)]
    exp_c = []
    for opp, v in re.findall(r"Corner::new\((None|Some\(CornerId::new\(\d+\)\)),\s*VertexId::new\((\d+)\)\)", b):
        m = re.search(r"(\d+)", opp)
        exp_c.append([int(m.group(1)) if m else -1, int(v)])
    out["unit_square"] = {
        "file": "src/mesh/corner_table/builder.rs:%d" % line_of(bld, "fn from_vertices_and_indices"),
        "vertices": sq_verts, "indices": sq_idx,
        "expected_vertex_corner": [c for c, _ in exp_v],
        "expected_vertex_pos": [p for _, p in exp_v],
        "expected_corners": exp_c,
    }
    b = fn_body(bld, "should_remove_face_that_introduces_non_manifold_edge")
    out["non_manifold_edge"] = {
        "file": "src/mesh/corner_table/builder.rs:%d" % line_of(bld, "fn should_remove_face_that_introduces_non_manifold_edge"),
        "vertices": [floats(m) for m in re.findall(r"Vec3::new\(([^)]*)\)", b)],
        "indices": [int(x) for x in re.search(r"&\[([\d,\s]*)\]", b).group(1).replace("\n", "").split(",") if x.strip()],
        "expected_faces": int(re.search(r"count\(\)\s*==\s*(\d+)", b).group(1)),
    }
    b = fn_body(bld, "should_fix_non_manifold_topology")
    idx_txt = re.search(r"&vec!\[([\d,\s]*)\]", b).group(1)
    out["non_manifold_topology"] = {
        "file": "src/mesh/corner_table/builder.rs:%d" % line_of(bld, "fn should_fix_non_manifold_topology"),
        "vertices": [floats(m) for m in re.findall(r"Vec3f::new\(([^)]*)\)", b)],
        "indices": [int(x) - 1 for x in idx_txt.split(",") if x.strip()],
        "expected_faces": int(re.search(r"assert_eq!\(num_faces,\s*(\d+)", b).group(1)),
        "expected_vertices": int(re.search(r"assert_eq!\(\s*num_vertices,\s*(\d+)", b).group(1)),
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_reference_kats.py /path/to/baby_shark")
    main(sys.argv[1])
