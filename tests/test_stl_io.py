"""Binary STL reader/writer (io/stl.rs:15-199): byte layout, normals,
round trip, truncated data; and the reader feeding the GPU soup builder."""
import json
import os

import numpy as np
import pytest

from baby_shark_gb300 import io as bio

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def box2():
    return np.array(GOLD["box2_stl"]["triangles"], np.float32).reshape(-1, 3, 3)


def test_layout_and_round_trip(tmp_path):
    tri = box2()
    data = bio.stl_bytes(tri)
    assert len(data) == 80 + 4 + 50 * len(tri)
    assert data[:80] == bytes(80)
    assert int(np.frombuffer(data, "<u4", 1, 80)[0]) == len(tri)
    rec = np.frombuffer(data, bio.FACE_DTYPE, len(tri), 84)
    assert np.all(rec["attr"] == 0)
    assert np.array_equal(rec["v"], tri)
    p = tmp_path / "box2.stl"
    bio.StlWriter().write_stl_to_file(tri, p)
    back = bio.StlReader().read_soup(p)
    assert np.array_equal(back.view(np.uint32), tri.view(np.uint32))


def test_normals_unit_and_degenerate_zero():
    tri = np.array([[[0, 0, 0], [2, 0, 0], [0, 3, 0]],     # +z
                    [[0, 0, 0], [0, 0, 1], [1, 0, 0]],     # +y
                    [[1, 1, 1], [2, 2, 2], [3, 3, 3]]],    # degenerate
                   np.float32)
    n = np.frombuffer(bio.stl_bytes(tri), bio.FACE_DTYPE, 3, 84)["normal"]
    assert np.array_equal(n[0], [0, 0, 1]) and np.array_equal(n[1], [0, 1, 0])
    assert np.array_equal(n[2], [0, 0, 0])


def test_indexed_input_and_truncated():
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    f = np.array([[0, 1, 2], [0, 2, 3]])
    data = bio.stl_bytes((v, f))
    assert np.array_equal(bio.read_stl_soup(data), v[f])
    with pytest.raises(bio.ReadError):
        bio.read_stl_soup(data[:-1])
    with pytest.raises(bio.ReadError):
        bio.read_stl_soup(data[:50])


@pytest.mark.gpu
def test_reader_builds_corner_table():
    from tests.gpu_common import context
    ct = bio.StlReader().read_stl(bio.stl_bytes(box2()), context())
    assert (ct.faces_count(), ct.vertices_count()) == (12, 8)
    out = bio.read_stl_soup(bio.stl_bytes(ct))
    assert out.shape == (12, 3, 3)
    assert np.array_equal(np.unique(out.reshape(-1, 3), axis=0), np.unique(box2().reshape(-1, 3), axis=0))
