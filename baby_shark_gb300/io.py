"""Binary STL reader and writer (io/stl.rs:15-199).

The reader returns the triangle soup, or builds a CornerTable from it on the
GPU the way `StlReader::read_from_buffer::<CornerTable>` feeds the soup
builder (corner_table/builder.rs:292-309).  The writer emits the reference's
layout: an 80-byte zero header, the face count as u32, then per face the unit
normal ((b - a) x (c - a), normalised; zeros for degenerate faces), the three
vertices and two zero attribute bytes, all little-endian.
"""
import os

import numpy as np

STL_HEADER_SIZE = 80
FACE_DTYPE = np.dtype([("normal", "<f4", (3,)), ("v", "<f4", (3, 3)), ("attr", "<u2")])


class ReadError(IOError):
    """The STL data is shorter than its face count says (io/mod.rs ReadError)."""


def read_stl_soup(source):
    """Triangles of a binary STL file (path or bytes) as float32[n, 3, 3]."""
    data = source if isinstance(source, (bytes, bytearray, memoryview)) else open(os.fspath(source), "rb").read()
    if len(data) < STL_HEADER_SIZE + 4:
        raise ReadError("STL data ends inside the header")
    n = int(np.frombuffer(data, "<u4", 1, STL_HEADER_SIZE)[0])
    need = STL_HEADER_SIZE + 4 + n * FACE_DTYPE.itemsize
    if len(data) < need:
        raise ReadError("STL data holds fewer faces than its count (%d)" % n)
    faces = np.frombuffer(data, FACE_DTYPE, n, STL_HEADER_SIZE + 4)
    return np.ascontiguousarray(faces["v"], dtype=np.float32)


class StlReader:
    """StlReader (io/stl.rs:15-100)."""

    def read_stl(self, source, ctx=None):
        """A CornerTable built on the GPU from the file's triangle soup."""
        from .api import CornerTable
        return CornerTable.from_triangles_soup(read_stl_soup(source), ctx)

    def read_soup(self, source):
        return read_stl_soup(source)


def _normals(tri):
    """Triangle3::normal (geometry/primitives/triangle3.rs:261-269) in f32."""
    a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
    u, v = b - a, c - a
    n = np.stack([u[:, 1] * v[:, 2] - u[:, 2] * v[:, 1],
                  u[:, 2] * v[:, 0] - u[:, 0] * v[:, 2],
                  u[:, 0] * v[:, 1] - u[:, 1] * v[:, 0]], axis=1).astype(np.float32)
    sq = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
    out = np.zeros_like(n)
    ok = sq != 0
    out[ok] = n[ok] / np.sqrt(sq[ok])[:, None]
    return out


def _as_soup(mesh):
    """float32[n, 3, 3] from a soup, a (vertices, faces) pair or a CornerTable."""
    if hasattr(mesh, "export") and hasattr(mesh, "faces_count"):
        ex = mesh.export()
        cv = ex["corner_vertex"].reshape(-1, 3)
        cv = cv[(cv >= 0).all(axis=1)]
        return ex["positions"][cv]
    if isinstance(mesh, tuple):
        v, f = mesh
        return np.asarray(v, np.float32)[np.asarray(f, np.int64)]
    return np.asarray(mesh, np.float32).reshape(-1, 3, 3)


def stl_bytes(mesh):
    tri = np.ascontiguousarray(_as_soup(mesh), np.float32)
    n = len(tri)
    if n > 0xFFFFFFFF:
        raise ValueError("Mesh is too big for STL")
    faces = np.zeros(n, FACE_DTYPE)
    faces["normal"] = _normals(tri)
    faces["v"] = tri
    return bytes(STL_HEADER_SIZE) + np.uint32(n).astype("<u4").tobytes() + faces.tobytes()


class StlWriter:
    """StlWriter (io/stl.rs:101-199)."""

    def write_stl_to_file(self, mesh, path):
        with open(os.fspath(path), "wb") as f:
            f.write(stl_bytes(mesh))
