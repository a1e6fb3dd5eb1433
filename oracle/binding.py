"""ORACLE — test infrastructure only.

ctypes binding of the CPU restatement of baby_shark's implicit-modelling
path (oracle/*.hpp).  It is the parity checker: the test-suite, the smoke
check and the benchmark's CPU-baseline leg use it; the product package never
imports it.
"""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(force=False):
    """Compile the oracle with its Makefile (g++, OpenMP, -ffp-contract=off)."""
    cmd = ["make", "-C", _HERE]
    if force:
        cmd.insert(1, "-B")
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            vp, i64, f32 = C.c_void_p, C.c_int64, C.c_float
            sig = {
                "orc_num_threads": (C.c_int, []),
                "orc_set_num_threads": (None, [C.c_int]),
                "orc_mesh_to_volume": (vp, [f32p, i64, u32p, i64, f32, i64, vp, vp]),
                "orc_volume_free": (None, [vp]),
                "orc_volume_from_leaves": (vp, [i32p, f32p, u32p, i64, f32]),
                "orc_volume_clone": (vp, [vp]),
                "orc_volume_sphere": (vp, [f32, f32, f32, f32, f32]),
                "orc_volume_cuboid": (vp, [f32, f32p, f32p]),
                "orc_volume_iwp": (vp, [f32, f32p, f32p, f32]),
                "orc_volume_from_samples": (vp, [f32, i64, i64p, i64p, f32p]),
                "orc_volume_num_leaves": (i64, [vp]),
                "orc_volume_export": (None, [vp, i32p, vp, vp]),
                "orc_volume_num_tiles": (i64, [vp]),
                "orc_volume_export_tiles": (None, [vp, i32p, i32p, f32p]),
                "orc_volume_union": (C.c_int, [vp, vp]),
                "orc_volume_subtract": (C.c_int, [vp, vp]),
                "orc_volume_intersect": (C.c_int, [vp, vp]),
                "orc_volume_flood_fill": (C.c_int, [vp]),
                "orc_volume_offset": (C.c_int, [vp, f32]),
                "orc_dual_contour": (i64, [vp, f32, vp, i64, vp, vp, vp, C.c_int]),
                "orc_mc_count": (i64, [vp, vp, vp]),
                "orc_marching_cubes": (i64, [vp, f32, vp, i64]),
                "orc_subtriangles": (i64, [f32p, i64, u32p, i64, f32, i64, vp, vp, i64]),
                "orc_corner_table_from_soup": (C.c_int, [f32p, i64, vp, vp]),
                "orc_corner_table_from_indexed": (C.c_int, [f32p, i64, i64p, i64, vp, vp, vp, vp, vp, vp, vp, vp]),
                "orc_fast_wn": (None, [f32p, i64, u32p, i64, f32p, i64, f32, f32p, vp]),
                "orc_exact_wn_f64": (None, [f32p, i64, u32p, i64, f32p, i64, f64p]),
                "orc_small_new": (vp, [C.c_int]),
                "orc_small_free": (None, [vp]),
                "orc_small_insert": (None, [vp, i64, i64, i64, f32]),
                "orc_small_flood_fill": (None, [vp]),
                "orc_small_sign_at": (C.c_int, [vp, i64, i64, i64]),
                "orc_small_values": (C.c_int, [vp, f32p]),
                "orc_leaf1_csg": (C.c_int, [C.c_int, f32p, f32p, f32p]),
                "orc_tree_constants": (None, [i64p]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleVolume:
    """Handle on an oracle volume (the reference's `Volume`)."""

    def __init__(self, handle, voxel_size):
        self.h = handle
        self.voxel_size = voxel_size

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_volume_free(self.h)
            self.h = None

    def _take(self):
        h, self.h = self.h, None
        return h

    def clone(self):
        return OracleVolume(lib().orc_volume_clone(self.h), self.voxel_size)

    def export(self):
        """Leaves in tree order: (origins int32[n,3], values f32[n,512], masks uint32[n,16])."""
        n = lib().orc_volume_num_leaves(self.h)
        o = np.zeros((n, 3), np.int32)
        v = np.zeros((n, 512), np.float32)
        m = np.zeros((n, 16), np.uint32)
        lib().orc_volume_export(self.h, o, _ptr(v), _ptr(m))
        return o, v, m

    def tiles(self):
        n = lib().orc_volume_num_tiles(self.h)
        o = np.zeros((n, 3), np.int32)
        s = np.zeros(n, np.int32)
        v = np.zeros(n, np.float32)
        if n:
            lib().orc_volume_export_tiles(self.h, o, s, v)
        return o, s, v

    def union(self, other):
        lib().orc_volume_union(self.h, other._take())
        return self

    def subtract(self, other):
        lib().orc_volume_subtract(self.h, other._take())
        return self

    def intersect(self, other):
        lib().orc_volume_intersect(self.h, other._take())
        return self

    def flood_fill(self):
        lib().orc_volume_flood_fill(self.h)
        return self

    def offset(self, d):
        rc = lib().orc_volume_offset(self.h, float(d))
        if rc:
            raise RuntimeError("oracle offset met a tile")
        return self

    def dual_contour(self, tiles_via_at=False):
        """Triangles, status, crossings, cells.  tiles_via_at: read active
        tiles through Grid::at instead of stopping (status 1) at them."""
        st = C.c_int(0)
        ne, nc = C.c_int64(0), C.c_int64(0)
        f = int(bool(tiles_via_at))
        n = lib().orc_dual_contour(self.h, self.voxel_size, None, 0, C.byref(st), C.byref(ne), C.byref(nc), f)
        out = np.zeros((max(n, 1), 9), np.float32)
        lib().orc_dual_contour(self.h, self.voxel_size, _ptr(out), n, C.byref(st), None, None, f)
        return out[:n].reshape(n, 3, 3), st.value, ne.value, nc.value

    def marching_cubes(self, voxel_size=None):
        """Triangles (n, 3, 3) of the oracle's marching-cubes mesher (oracle_mc.hpp)."""
        h = self.voxel_size if voxel_size is None else float(voxel_size)
        n = lib().orc_marching_cubes(self.h, h, None, 0)
        out = np.zeros((max(n, 1), 9), np.float32)
        lib().orc_marching_cubes(self.h, h, _ptr(out), n)
        return out[:n].reshape(n, 3, 3)

    def mc_triangles(self):
        amb, cubes = C.c_int64(0), C.c_int64(0)
        n = lib().orc_mc_count(self.h, C.byref(amb), C.byref(cubes))
        return n, amb.value, cubes.value


def mesh_to_volume(verts, tris, voxel_size, band, with_wn=False):
    """MeshToVolume::default().with_voxel_size(h).with_narrow_band_width(b).convert(mesh)."""
    verts = np.ascontiguousarray(verts, np.float32)
    tris = np.ascontiguousarray(tris, np.uint32)
    stats = np.zeros(6, np.int64)
    # the band size is unknown before the run: allocate for the worst case lazily
    wn = None
    h = lib().orc_mesh_to_volume(verts, len(verts), tris, len(tris), float(voxel_size), int(band), _ptr(stats), None)
    if not h:
        return None, stats, None
    vol = OracleVolume(h, float(voxel_size))
    if with_wn:
        wn = np.zeros(int(stats[4]), np.float32)
        h2 = lib().orc_mesh_to_volume(verts, len(verts), tris, len(tris), float(voxel_size), int(band), None, _ptr(wn))
        lib().orc_volume_free(h2)
    keys = ["subtris", "pairs", "far_evals", "leaf_tri_evals", "band_voxels", "near_threshold"]
    return vol, dict(zip(keys, (int(x) for x in stats))), wn


def volume_from_leaves(origins, values, masks, voxel_size):
    """An oracle volume holding exported leaves (e.g. a GPU result)."""
    o = np.ascontiguousarray(origins, np.int32)
    v = np.ascontiguousarray(values, np.float32)
    m = np.ascontiguousarray(masks, np.uint32)
    return OracleVolume(lib().orc_volume_from_leaves(o, v, m, len(o), float(voxel_size)), float(voxel_size))


def volume_sphere(h, radius, origin):
    """VolumeBuilder::sphere (volume/builder.rs:21-31)."""
    o = [float(x) for x in origin]
    return OracleVolume(lib().orc_volume_sphere(float(h), float(radius), *o), float(h))


def volume_cuboid(h, vmin, vmax):
    """VolumeBuilder::cuboid (volume/builder.rs:33-54)."""
    a, b = np.asarray(vmin, np.float32), np.asarray(vmax, np.float32)
    return OracleVolume(lib().orc_volume_cuboid(float(h), a, b), float(h))


def volume_iwp(h, vmin, vmax, cell_size):
    """VolumeBuilder::iwp (volume/builder.rs:57-76)."""
    a, b = np.asarray(vmin, np.float32), np.asarray(vmax, np.float32)
    return OracleVolume(lib().orc_volume_iwp(float(h), a, b, float(cell_size)), float(h))


def volume_from_samples(h, band, idx_min, values):
    """Volume::from_fn (volume/mod.rs:40-72) over values sampled at grid
    points (idx_min + (i, j, k)) * h, values[i, j, k]."""
    v = np.ascontiguousarray(values, np.float32)
    lo = np.ascontiguousarray(idx_min, np.int64)
    dims = np.array(v.shape, np.int64)
    return OracleVolume(lib().orc_volume_from_samples(float(h), int(band), lo, dims, v), float(h))


def subtriangles(verts, tris, voxel_size, band):
    """The reference's sub-triangles (n, 3, 3) float32 and widened boxes (n, 6) int64."""
    v = np.ascontiguousarray(verts, np.float32)
    t = np.ascontiguousarray(tris, np.uint32)
    n = lib().orc_subtriangles(v, len(v), t, len(t), float(voxel_size), int(band), None, None, 0)
    out = np.zeros((max(n, 1), 9), np.float32)
    box = np.zeros((max(n, 1), 6), np.int64)
    lib().orc_subtriangles(v, len(v), t, len(t), float(voxel_size), int(band), _ptr(out), _ptr(box), n)
    return out[:n].reshape(n, 3, 3), box[:n]


def fast_wn(verts, tris, points, beta=2.0):
    verts = np.ascontiguousarray(verts, np.float32)
    tris = np.ascontiguousarray(tris, np.uint32)
    pts = np.ascontiguousarray(points, np.float32)
    out = np.zeros(len(pts), np.float32)
    cnt = np.zeros(3, np.int64)
    lib().orc_fast_wn(verts, len(verts), tris, len(tris), pts, len(pts), float(beta), out, _ptr(cnt))
    return out, {"far_evals": int(cnt[0]), "leaf_tri_evals": int(cnt[1]), "nodes": int(cnt[2])}


def exact_wn_f64(verts, tris, points):
    verts = np.ascontiguousarray(verts, np.float32)
    tris = np.ascontiguousarray(tris, np.uint32)
    pts = np.ascontiguousarray(points, np.float32)
    out = np.zeros(len(pts), np.float64)
    lib().orc_exact_wn_f64(verts, len(verts), tris, len(tris), pts, len(pts), out)
    return out


def corner_table_from_soup(points):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    nf, nv = C.c_int64(0), C.c_int64(0)
    rc = lib().orc_corner_table_from_soup(pts, len(pts), C.byref(nf), C.byref(nv))
    if rc:
        raise RuntimeError("corner table build error")
    return nf.value, nv.value


def corner_table_from_indexed(verts, faces):
    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.int64).reshape(-1)
    nf, nv, nct, nvt = C.c_int64(0), C.c_int64(0), C.c_int64(0), C.c_int64(0)
    cap_c = len(f)
    cap_v = len(v) + len(f)
    cv = np.zeros(cap_c, np.int32)
    co = np.zeros(cap_c, np.int32)
    vc = np.zeros(cap_v, np.int32)
    vd = np.zeros(cap_v, np.uint8)
    rc = lib().orc_corner_table_from_indexed(v, len(v), f, len(f), C.byref(nf), C.byref(nv), C.byref(nct),
                                             C.byref(nvt), _ptr(cv), _ptr(co), _ptr(vc), _ptr(vd))
    return {
        "status": rc, "faces": nf.value, "vertices": nv.value,
        "corner_vertex": cv[: nct.value], "corner_opposite": co[: nct.value],
        "vertex_corner": vc[: nvt.value], "vertex_deleted": vd[: nvt.value],
    }


class SmallTree:
    """The small static/dynamic trees of the reference's unit tests."""

    KINDS = {"leaf1": 0, "leaf2": 1, "internal2_1": 2, "root1": 3}

    def __init__(self, kind):
        self.h = lib().orc_small_new(self.KINDS[kind])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_small_free(self.h)

    def insert(self, x, y, z, v):
        lib().orc_small_insert(self.h, int(x), int(y), int(z), float(v))

    def flood_fill(self):
        lib().orc_small_flood_fill(self.h)

    def sign_at(self, x, y, z):
        return lib().orc_small_sign_at(self.h, int(x), int(y), int(z))

    def values(self):
        out = np.zeros(512, np.float32)
        n = lib().orc_small_values(self.h, out)
        return out[:n]


def leaf1_csg(op, a, b):
    out = np.zeros(8, np.float32)
    full = lib().orc_leaf1_csg({"union": 0, "subtract": 1, "intersect": 2}[op],
                               np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32), out)
    return out, bool(full)


def tree_constants():
    out = np.zeros(9, np.int64)
    lib().orc_tree_constants(out)
    return out


def set_threads(n):
    lib().orc_set_num_threads(int(n))


def num_threads():
    return lib().orc_num_threads()
