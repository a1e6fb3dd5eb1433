"""Host-side API mirroring the reference crate's voxel builders.

Names, argument meaning and failure behaviour follow baby_shark v0.3.12:

  MeshToVolume        voxel/mesh_to_volume.rs:17-73
  Volume              voxel/volume/mod.rs:11-123 (booleans consume both operands)
  DualContouringMesher voxel/meshing/dual_contouring.rs:12-91
  CornerTable         mesh/corner_table/builder.rs:292-309 (soup builder)
  VoxelRemesher       remeshing/voxel.rs:44-95

Where the reference returns `None` (empty mesh), these return None; every
other failure raises BsError with the native status.  All compute runs in
libbs_gb300.so on the GPU.
"""
import ctypes as C

import numpy as np

from . import _native as N


class Context:
    """A device + CUDA stream + memory pool (bs_ctx)."""

    def __init__(self, device=0, stream=None):
        self._lib = N.load()
        h = C.c_void_p()
        N.check(self._lib.bs_ctx_create(int(device), stream, C.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self._lib.bs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        """The cudaStream_t the context runs on (as an int handle)."""
        return self._lib.bs_ctx_stream(self.h)

    def synchronize(self):
        N.check(self._lib.bs_ctx_synchronize(self.h), self.h)

    @property
    def kernel_launches(self):
        return int(self._lib.bs_ctx_kernel_launches(self.h))

    def set_stage_timing(self, enable=True):
        N.check(self._lib.bs_ctx_set_stage_timing(self.h, 1 if enable else 0), self.h)

    def stage_times(self, reset=False):
        """{kernel name: (total ms, launches)} recorded with CUDA events."""
        n = C.c_int()
        N.check(self._lib.bs_ctx_stage_count(self.h, C.byref(n)), self.h)
        out = {}
        for i in range(n.value):
            name, ms, cnt = C.c_char_p(), C.c_double(), C.c_uint64()
            N.check(self._lib.bs_ctx_stage_info(self.h, i, C.byref(name), C.byref(ms), C.byref(cnt)), self.h)
            out[name.value.decode()] = (ms.value, cnt.value)
        if reset:
            N.check(self._lib.bs_ctx_stage_reset(self.h), self.h)
        return out

    def autotune(self, mesh, voxel_size, band_width):
        """bs_autotune_mesh_to_volume on a mesh ((vertices, faces) numpy
        arrays): keeps the fastest launch shapes for this context and
        returns them with the per-candidate times."""
        import torch
        v, f = _mesh_arrays(mesh)
        dv = torch.from_numpy(v).cuda()
        df = torch.from_numpy(f.astype(np.int32)).cuda()
        torch.cuda.synchronize()
        P = N.M2VParams()
        self._lib.bs_m2v_params_default(C.byref(P))
        P.voxel_size = float(voxel_size)
        P.band_width = int(band_width)
        ch = (C.c_int32 * 3)()
        ms = (C.c_float * 11)()
        N.check(self._lib.bs_autotune_mesh_to_volume(self.h, dv.data_ptr(), len(v), df.data_ptr(), len(f),
                                                     C.byref(P), ch, ms), self.h)
        shapes = [(64, 8), (64, 16), (64, 32), (128, 8), (128, 16), (128, 32), (256, 8), (256, 16)]
        return {"dist_threads": ch[0], "wn_warps": ch[1], "dist_tile": ch[2],
                "distance_ms": {sh: ms[k] for k, sh in enumerate(shapes)},
                "sign_ms": {2: ms[8], 4: ms[9], 8: ms[10]}}

    def set_launch_shape(self, dist_threads=0, wn_warps=0, dist_tile=0):
        N.check(self._lib.bs_ctx_set_launch_shape(self.h, int(dist_threads), int(wn_warps), int(dist_tile)), self.h)

    def memory(self):
        """Bytes of the context's device pool: in use, peak in use, reserved."""
        u, hi, r = C.c_uint64(), C.c_uint64(), C.c_uint64()
        N.check(self._lib.bs_ctx_memory(self.h, C.byref(u), C.byref(hi), C.byref(r)), self.h)
        return {"used": u.value, "used_high": hi.value, "reserved": r.value}

    def memory_reset(self, trim=False):
        N.check(self._lib.bs_ctx_memory_reset(self.h, int(bool(trim))), self.h)

    def last_stats(self):
        """Counters of the last mesh -> volume, offset, dual contouring or
        winding-number call (bs_ctx_last_counters), named for that call."""
        a = (C.c_uint64 * 16)()
        N.check(self._lib.bs_ctx_last_counters(self.h, a), self.h)
        a = [int(x) for x in a]
        kind = a[8]
        if kind == 2:
            return {"call": "offset", "offset_passes": a[6], "offset_leaf_sweeps": a[7]}
        if kind == 3:
            return {"call": "dual_contouring", "crossings": a[6], "cells": a[7]}
        out = {"call": "winding_numbers" if kind == 4 else "mesh_to_volume"}
        if kind != 4:
            keys = ["triangles", "subtris", "brick_pairs", "voxel_pairs", "leaves", "active_voxels"]
            out.update(zip(keys, a[:6]))
            out["voxel_pairs_evaluated"] = a[9]
        out["wn_warp_visits"] = a[6]
        out["wn_warp_far"] = a[7] & 0xffffffff
        out["wn_warp_exact"] = a[7] >> 32
        out["wn_far"] = a[10]
        out["wn_exact"] = a[11]
        out["wn_tree"] = "reference" if a[12] == 0 else "fast"
        out["wn_far_warp_sections"] = a[13]
        out["wn_exact_warp_sections"] = a[14]
        return out


class VolumeBuilder:
    """VolumeBuilder (volume/builder.rs:5-84): sphere, cuboid and the IWP
    surface, evaluated and built on the GPU."""

    def __init__(self, ctx=None):
        self.ctx = ctx or default_context()
        self.voxel_size = 1.0

    def with_voxel_size(self, voxel_size):
        self.voxel_size = float(voxel_size)
        return self

    def set_voxel_size(self, voxel_size):
        self.voxel_size = float(voxel_size)

    def _make(self, fn, *args):
        out = C.c_void_p()
        N.check(fn(self.ctx.h, C.c_float(self.voxel_size), *args, C.byref(out)), self.ctx.h)
        return Volume(out, self.ctx)

    @staticmethod
    def _v3(a):
        return (C.c_float * 3)(*[float(x) for x in a])

    def sphere(self, radius, origin):
        return self._make(N.load().bs_volume_sphere, C.c_float(radius), self._v3(origin))

    def cuboid(self, vmin, vmax):
        return self._make(N.load().bs_volume_cuboid, self._v3(vmin), self._v3(vmax))

    def iwp(self, vmin, vmax, cell_size):
        return self._make(N.load().bs_volume_iwp, self._v3(vmin), self._v3(vmax), C.c_float(cell_size))


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _mesh_arrays(mesh):
    """Accepts (vertices, faces) or an object with .vertices/.faces, or an (n,3,3) soup."""
    if isinstance(mesh, tuple) and len(mesh) == 2:
        v, f = mesh
    elif hasattr(mesh, "vertices") and hasattr(mesh, "faces"):
        v, f = mesh.vertices, mesh.faces
    else:
        soup = np.asarray(mesh, np.float32).reshape(-1, 3)
        v, f = soup, np.arange(len(soup), dtype=np.uint32).reshape(-1, 3)
    v = np.ascontiguousarray(v, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(f, np.uint32).reshape(-1, 3)
    return v, f


class Volume:
    """Narrow-band signed distance volume on the GPU (bs_volume)."""

    def __init__(self, handle, ctx):
        self.h = handle
        self.ctx = ctx

    @staticmethod
    def with_voxel_size(voxel_size, ctx=None):
        """Volume::with_voxel_size (volume/mod.rs:17-24): an empty volume."""
        ctx = ctx or default_context()
        out = C.c_void_p()
        N.check(N.load().bs_volume_create(ctx.h, C.c_float(voxel_size), C.byref(out)), ctx.h)
        return Volume(out, ctx)

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            try:
                N.load().bs_volume_free(self.h)
            except Exception:
                pass
            self.h = None

    def _take(self):
        if self.h is None or not self.h.value:
            raise ValueError("volume was consumed by a boolean operation")
        h, self.h = self.h, None
        return h

    def voxel_size(self):
        out = C.c_float()
        N.check(N.load().bs_volume_voxel_size(self.h, C.byref(out)))
        return out.value

    @staticmethod
    def from_fn(voxel_size, vmin, vmax, narrow_band_width, func, ctx=None):
        """Volume::from_fn (volume/mod.rs:40-72): `func` maps an (N, 3) float32
        array of grid points (numpy, or a torch tensor on the context's GPU) to
        N signed values, inside negative; the sparse volume is built on the GPU.
        Grid points are idx * voxel_size for idx from floor(min / voxel_size)
        to ceil(max / voxel_size), as the reference."""
        ctx = ctx or default_context()
        h = np.float32(voxel_size)
        lo = np.floor(np.asarray(vmin, np.float32) / h).astype(np.int64)
        hi = np.ceil(np.asarray(vmax, np.float32) / h).astype(np.int64)
        dims = (hi - lo + 1).astype(np.uint64)
        if np.any(hi < lo):
            raise ValueError("from_fn: max below min")
        axes = [np.arange(lo[i], hi[i] + 1).astype(np.float32) * h for i in range(3)]
        X, Y, Z = np.meshgrid(*axes, indexing="ij")
        pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        out = C.c_void_p()
        vals = func(pts)
        if hasattr(vals, "is_cuda") and vals.is_cuda:
            import torch
            v = vals.to(torch.float32).contiguous()
            N.check(N.load().bs_volume_from_samples_device(ctx.h, float(h), int(narrow_band_width),
                                                           lo.ctypes.data, dims.ctypes.data, v.data_ptr(),
                                                           C.byref(out)), ctx.h)
        else:
            v = np.ascontiguousarray(np.asarray(vals, np.float32).reshape(-1))
            N.check(N.load().bs_volume_from_samples(ctx.h, float(h), int(narrow_band_width), lo.ctypes.data,
                                                    dims.ctypes.data, v.ctypes.data, C.byref(out)), ctx.h)
        return Volume(out, ctx)

    def counts(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        N.check(N.load().bs_volume_counts(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"leaves": a.value, "tiles": b.value, "active_voxels": c.value}

    def clone(self):
        out = C.c_void_p()
        N.check(N.load().bs_volume_clone(self.ctx.h, self.h, C.byref(out)), self.ctx.h)
        return Volume(out, self.ctx)

    def export(self):
        """(origins int32[n,3], values f32[n,512], masks uint32[n,16]) with leaves sorted by origin."""
        n = self.counts()["leaves"]
        o = np.zeros((n, 3), np.int32)
        v = np.zeros((n, 512), np.float32)
        m = np.zeros((n, 16), np.uint32)
        N.check(N.load().bs_volume_export(self.ctx.h, self.h, o.ctypes.data, v.ctypes.data, m.ctypes.data),
                self.ctx.h)
        return o, v, m

    def tiles(self):
        n = self.counts()["tiles"]
        o = np.zeros((n, 3), np.int32)
        s = np.zeros(n, np.int32)
        v = np.zeros(n, np.float32)
        if n:
            N.check(N.load().bs_volume_export_tiles(self.ctx.h, self.h, o.ctypes.data, s.ctypes.data,
                                                    v.ctypes.data), self.ctx.h)
        return o, s, v

    def _csg(self, other, fn):
        out = C.c_void_p()
        a, b = self._take(), other._take()
        N.check(fn(self.ctx.h, a, b, C.byref(out)), self.ctx.h)
        return Volume(out, self.ctx)

    def union(self, other):
        """Volume::union (volume/mod.rs:74-79); consumes self and other."""
        return self._csg(other, N.load().bs_volume_union)

    def subtract(self, other):
        """Volume::subtract (volume/mod.rs:88-93); consumes self and other."""
        return self._csg(other, N.load().bs_volume_subtract)

    def intersect(self, other):
        """Volume::intersect (volume/mod.rs:81-86); consumes self and other."""
        return self._csg(other, N.load().bs_volume_intersect)

    def offset(self, distance):
        """Volume::offset (volume/mod.rs:95-108)."""
        N.check(N.load().bs_volume_offset(self.ctx.h, self.h, float(distance)), self.ctx.h)
        return self


class MeshToVolume:
    """MeshToVolume (voxel/mesh_to_volume.rs:17-73)."""

    def __init__(self, ctx=None):
        self.ctx = ctx or default_context()
        self.params = N.M2VParams()
        N.load().bs_m2v_params_default(C.byref(self.params))

    def with_voxel_size(self, size):
        self.params.voxel_size = float(size)
        return self

    def with_narrow_band_width(self, width):
        self.params.band_width = int(width)
        return self

    def set_voxel_size(self, size):
        return self.with_voxel_size(size)

    def set_narrow_band_width(self, width):
        return self.with_narrow_band_width(width)

    def with_winding_number_order(self, order):
        """Far-field order of the sign pass: 2 as the reference, or 3 (an
        extension, evaluated over the library's own tree)."""
        self.params.wn_order = int(order)
        if int(order) == 3:
            self.params.wn_tree = 1
        return self

    def with_sign_tree(self, tree):
        """Tree of the sign pass: "reference" (default; the reference's SAH
        tree and summation order, bit-exact signs) or "fast" (the library's
        PLOC tree with a warp-coherent traversal)."""
        if tree not in ("reference", "fast"):
            raise ValueError("tree must be 'reference' or 'fast'")
        self.params.wn_tree = 0 if tree == "reference" else 1
        return self

    def convert(self, mesh):
        """Returns a Volume, or None for an empty mesh (as the reference)."""
        v, f = _mesh_arrays(mesh)
        out = C.c_void_p()
        st = N.load().bs_mesh_to_volume(self.ctx.h, v.ctypes.data, len(v), f.ctypes.data, len(f),
                                        C.byref(self.params), C.byref(out))
        if st == 2:  # BS_ERR_EMPTY
            return None
        N.check(st, self.ctx.h)
        return Volume(out, self.ctx)


def convert_batch(meshes, params, ctx=None):
    """Many meshes in one set of GPU launches (bs_mesh_to_volume_batch).

    `meshes` is a list of (vertices, triangles) pairs, `params` a list of
    (voxel_size, band_width) pairs or one pair for all.  Returns one Volume
    per mesh (None for a mesh without triangles); each equals what
    MeshToVolume(...).convert returns for that mesh alone."""
    ctx = ctx or default_context()
    K = len(meshes)
    if isinstance(params, tuple):
        params = [params] * K
    arrays = [_mesh_arrays(m) for m in meshes]
    xyz = np.ascontiguousarray(np.concatenate([v for v, _ in arrays]) if K else np.zeros((0, 3), np.float32))
    tri = np.ascontiguousarray(np.concatenate([f for _, f in arrays]) if K else np.zeros((0, 3), np.uint32))
    nv = np.array([len(v) for v, _ in arrays], np.uint64)
    nt = np.array([len(f) for _, f in arrays], np.uint64)
    P = (N.M2VParams * K)()
    for k, (h, band) in enumerate(params):
        N.load().bs_m2v_params_default(C.byref(P[k]))
        P[k].voxel_size = float(h)
        P[k].band_width = int(band)
    out = (C.c_void_p * K)()
    N.check(N.load().bs_mesh_to_volume_batch(ctx.h, K, xyz.ctypes.data, nv.ctypes.data, tri.ctypes.data,
                                             nt.ctypes.data, P, out), ctx.h)
    return [Volume(C.c_void_p(out[k]), ctx) if out[k] else None for k in range(K)]


class WindingNumbers:
    """WindingNumbers (spatial_partitioning/aabb_tree.rs:622-691) on the GPU:
    from_mesh builds the tree and far-field records, approximate evaluates the
    fast winding number at points.  order=3 adds the third-order far-field
    term (an extension; the reference stops at order 2)."""

    def __init__(self, handle, ctx):
        self.h = handle
        self.ctx = ctx

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            try:
                N.load().bs_winding_numbers_free(self.h)
            except Exception:
                pass
            self.h = None

    @staticmethod
    def from_mesh(mesh, order=2, ctx=None, tree="fast"):
        """tree="reference": the reference's own SAH tree, traversed once per
        point in its summation order (order 2 only); "fast": the library's
        PLOC tree with warp-coherent traversal."""
        import torch
        ctx = ctx or default_context()
        v, f = _mesh_arrays(mesh)
        dv = torch.from_numpy(v).cuda()
        df = torch.from_numpy(f.astype(np.int32)).cuda()
        torch.cuda.synchronize()
        out = C.c_void_p()
        if tree not in ("reference", "fast"):
            raise ValueError("tree must be 'reference' or 'fast'")
        N.check(N.load().bs_winding_numbers_build_ex(ctx.h, dv.data_ptr(), len(v), df.data_ptr(), len(f), int(order),
                                                     0 if tree == "reference" else 1, C.byref(out)), ctx.h)
        return WindingNumbers(out, ctx)

    def approximate(self, points, accuracy_scale=2.0):
        """Winding numbers (float32) of an (n, 3) array of points
        (WindingNumbers::approximate, aabb_tree.rs:654-660).  From 2^20
        points on, the library traverses them in Morton order and returns the
        values in the given order."""
        import torch
        p = torch.from_numpy(np.ascontiguousarray(points, np.float32).reshape(-1, 3)).cuda()
        out = torch.empty(p.shape[0], dtype=torch.float32, device=p.device)
        torch.cuda.synchronize()
        N.check(N.load().bs_winding_numbers_approximate(self.ctx.h, self.h, p.data_ptr(), p.shape[0],
                                                        float(accuracy_scale), out.data_ptr()), self.ctx.h)
        return out.cpu().numpy()


class LearnedFarField:
    """Learned far field (no reference counterpart; the reference evaluates
    winding numbers only at band voxels, mesh_to_volume.rs:245-280): a small
    per-mesh network trained on the GPU (bs_mlp_*) on winding numbers that
    the tree traversal computes at sampled points, 70 % uniform in the padded
    bounding box and 30 % near the surface.  It answers only points outside
    the narrow band of a volume of the mesh (by default voxel 1/200 of the
    largest extent, band 3): classify() takes the network's value there when
    it lies more than the calibrated margin from the sign threshold, and the
    traversal's everywhere else.  The margin is the smallest one under which
    no calibration point outside the band (a separate sample) gets the other
    side of the threshold than the traversal gives it, times a safety factor.
    `timings` holds the seconds spent on the tree, the band, sampling, labels,
    training and calibration; comparisons against the plain traversal count
    them all."""

    def __init__(self):
        self.h = None

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            try:
                N.load().bs_mlp_free(self.h)
            except Exception:
                pass
            self.h = None

    @staticmethod
    def sample(vertices, faces, n, seed, near_fraction=0.3, sigma=0.02, pad=0.1):
        """Sample points as a CUDA tensor (n, 3): uniform in the box padded by
        `pad` of its extent, and near the surface (area-weighted triangle
        points moved along the normal by N(0, sigma times the largest
        extent)), in random order."""
        import torch
        gen = torch.Generator(device="cuda")
        gen.manual_seed(int(seed))
        v = torch.as_tensor(np.ascontiguousarray(vertices, np.float32)).cuda()
        f = torch.as_tensor(np.ascontiguousarray(faces, np.int64)).cuda()
        lo, hi = v.min(dim=0).values, v.max(dim=0).values
        ext = hi - lo
        n_near = int(n * near_fraction)
        uni = lo - pad * ext + torch.rand(n - n_near, 3, generator=gen, device=v.device) * (ext * (1 + 2 * pad))
        a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
        cr = torch.cross(b - a, c - a, dim=1)
        area = cr.norm(dim=1)
        idx = torch.multinomial(area, n_near, replacement=True, generator=gen)
        r1 = torch.rand(n_near, generator=gen, device=v.device)
        r2 = torch.rand(n_near, generator=gen, device=v.device)
        sq = r1.sqrt()
        pts = ((1 - sq)[:, None] * a[idx] + (sq * (1 - r2))[:, None] * b[idx] + (sq * r2)[:, None] * c[idx])
        nrm = cr[idx] / area[idx].clamp_min(1e-30)[:, None]
        pts = pts + nrm * (torch.randn(n_near, 1, generator=gen, device=v.device) * (sigma * float(ext.max())))
        out = torch.cat([uni, pts])
        return out[torch.randperm(n, generator=gen, device=v.device)].contiguous()

    @classmethod
    def train(cls, mesh, ctx=None, tree=None, band=None, n_samples=2_000_000, n_calibration=262_144, epochs=16,
              batch=8192, lr=3e-3, lr_min=1e-4, beta=2.0, thresh=0.2, order=2, max_frequency=16.0, seed=0,
              safety=1.25, band_voxel=None, band_width=3):
        import time

        import torch
        ctx = ctx or default_context()
        v, f = _mesh_arrays(mesh)
        rng = np.random.default_rng(seed)
        self = cls()
        self.ctx = ctx
        self.beta = float(beta)
        self.thresh = float(thresh)
        L = N.load()

        def sync():
            ctx.synchronize()
            torch.cuda.synchronize()

        lo, hi = v.min(axis=0), v.max(axis=0)
        extent = float((hi - lo).max())
        t0 = time.perf_counter()
        self.tree = tree if tree is not None else WindingNumbers.from_mesh((v, f), order=order, ctx=ctx)
        sync()
        t1 = time.perf_counter()
        if band is None:
            hb = band_voxel if band_voxel is not None else extent / 200.0
            band = MeshToVolume(ctx).with_voxel_size(hb).with_narrow_band_width(band_width).convert((v, f))
        self.band = band
        sync()
        t2 = time.perf_counter()
        dp = cls.sample(v, f, n_samples, seed)
        dc = cls.sample(v, f, n_calibration, seed + 1)
        sync()
        t3 = time.perf_counter()
        lab = torch.empty(len(dp), dtype=torch.float32, device=dp.device)
        clab = torch.empty(len(dc), dtype=torch.float32, device=dp.device)
        N.check(L.bs_winding_numbers_approximate(ctx.h, self.tree.h, dp.data_ptr(), len(dp), self.beta,
                                                 lab.data_ptr()), ctx.h)
        N.check(L.bs_winding_numbers_approximate(ctx.h, self.tree.h, dc.data_ptr(), len(dc), self.beta,
                                                 clab.data_ptr()), ctx.h)
        sync()
        t4 = time.perf_counter()
        centre = ((lo + hi) * 0.5).astype(np.float32)
        scale = np.float32(1.0 / (0.55 * extent))
        dirs = rng.normal(size=(32, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        mags = np.exp(np.linspace(0.0, np.log(max_frequency), 32))
        self.freq = np.ascontiguousarray(dirs * mags[:, None], np.float32)
        p = np.zeros(L.bs_mlp_num_params(), np.float32)
        lim = np.sqrt(6.0 / 128.0)
        p[0:4096] = rng.uniform(-lim, lim, 4096)
        p[4160:8256] = rng.uniform(-lim, lim, 4096)
        p[8320:8384] = rng.uniform(-0.1, 0.1, 64)
        p[8384] = float(lab.mean().item())
        self.centre, self.scale = centre, float(scale)
        h = C.c_void_p()
        N.check(L.bs_mlp_create(ctx.h, centre.ctypes.data, float(scale), self.freq.ctypes.data, p.ctypes.data,
                                C.byref(h)), ctx.h)
        self.h = h
        loss = np.zeros(epochs, np.float32)
        N.check(L.bs_mlp_train(ctx.h, self.h, dp.data_ptr(), lab.data_ptr(), len(dp), int(batch), int(epochs),
                               float(lr), float(lr_min), loss.ctypes.data), ctx.h)
        self.epoch_loss = loss
        sync()
        t5 = time.perf_counter()
        pred = torch.empty(len(dc), dtype=torch.float32, device=dp.device)
        N.check(L.bs_mlp_predict(ctx.h, self.h, dc.data_ptr(), len(dc), pred.data_ptr()), ctx.h)
        inb = self.band_flags(dc)
        pr, cl = pred.cpu().numpy(), clab.cpu().numpy()
        out = inb == 0
        wrong = out & ((pr > self.thresh) != (cl > self.thresh))
        worst = float(np.abs(pr[wrong] - self.thresh).max()) if wrong.any() else 0.0
        self.margin = safety * worst + 0.01
        self.calibration = {"points": len(dc), "outside_band": int(out.sum()), "wrong_side": int(wrong.sum()),
                            "worst_wrong_margin": worst,
                            "answered_fraction": float(np.mean(out & (np.abs(pr - self.thresh) > self.margin))),
                            "mean_abs_error_outside_band": float(np.mean(np.abs(pr - cl)[out]))}
        sync()
        t6 = time.perf_counter()
        self.timings = {"tree_s": t1 - t0, "band_s": t2 - t1, "sampling_s": t3 - t2, "labels_s": t4 - t3,
                        "training_s": t5 - t4, "calibration_s": t6 - t5}
        self.timings["total_s"] = sum(self.timings.values())
        return self

    def band_flags(self, points):
        """1 where a point's nearest grid point is in the band volume's active set."""
        import torch
        p = points if isinstance(points, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(points, np.float32).reshape(-1, 3)).cuda()
        out = torch.empty(p.shape[0], dtype=torch.int32, device=p.device)
        torch.cuda.synchronize()
        N.check(N.load().bs_volume_band_flags(self.ctx.h, self.band.h, p.data_ptr(), p.shape[0], out.data_ptr()),
                self.ctx.h)
        return out.cpu().numpy()

    def params(self):
        out = np.zeros(N.load().bs_mlp_num_params(), np.float32)
        N.check(N.load().bs_mlp_get_params(self.ctx.h, self.h, out.ctypes.data), self.ctx.h)
        return out

    def predict(self, points):
        """Network predictions (float32 numpy array) at an (n, 3) array or CUDA tensor of points."""
        import torch
        p = points if isinstance(points, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(points, np.float32).reshape(-1, 3)).cuda()
        out = torch.empty(p.shape[0], dtype=torch.float32, device=p.device)
        torch.cuda.synchronize()
        N.check(N.load().bs_mlp_predict(self.ctx.h, self.h, p.data_ptr(), p.shape[0], out.data_ptr()), self.ctx.h)
        return out.cpu().numpy()

    def classify(self, points):
        """Winding numbers at the points (numpy array or CUDA tensor): the
        network's where the point is outside the band and the prediction is
        confident, the traversal's elsewhere.  Returns (CUDA tensor of
        values, number of points that went to the traversal)."""
        import torch
        p = points if isinstance(points, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(points, np.float32).reshape(-1, 3)).cuda()
        out = torch.empty(p.shape[0], dtype=torch.float32, device=p.device)
        nt = C.c_uint64()
        torch.cuda.synchronize()
        N.check(N.load().bs_mlp_classify(self.ctx.h, self.h, self.tree.h, self.band.h, p.data_ptr(), p.shape[0],
                                         self.thresh, float(self.margin), self.beta, out.data_ptr(), C.byref(nt)),
                self.ctx.h)
        return out, int(nt.value)


def winding_numbers_exact(vertices, triangles, points, ctx=None):
    """Exact generalised winding numbers (float64) of `points` w.r.t. a mesh by
    direct summation on the GPU (bs_winding_numbers_exact).  Arguments are
    numpy arrays or torch CUDA tensors."""
    import torch
    ctx = ctx or default_context()
    dev = torch.device("cuda", torch.cuda.current_device())

    def as_dev(a, dtype):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
        return t.to(device=dev, dtype=dtype).contiguous()

    v = as_dev(vertices, torch.float32).reshape(-1, 3)
    f = as_dev(np.asarray(triangles, np.int64) if not isinstance(triangles, torch.Tensor) else triangles,
               torch.int32).reshape(-1, 3)
    p = as_dev(points, torch.float32).reshape(-1, 3)
    out = torch.empty(p.shape[0], dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    N.check(N.load().bs_winding_numbers_exact(ctx.h, v.data_ptr(), v.shape[0], f.data_ptr(), f.shape[0],
                                              p.data_ptr(), p.shape[0], out.data_ptr()), ctx.h)
    return out


class DualContouringMesher:
    """DualContouringMesher (voxel/meshing/dual_contouring.rs:12-91).

    with_qef_vertices() switches the cell vertices from the reference's
    particle solver to a float64 quadratic-error solve (bs_dual_contour_qef),
    an extension without a reference counterpart."""

    def __init__(self):
        self.voxel_size = 1.0
        self.qef = False

    def with_voxel_size(self, size):
        self.voxel_size = float(size)
        return self

    def with_qef_vertices(self, on=True):
        self.qef = bool(on)
        return self

    def mesh(self, volume):
        """Triangle soup as float32[n, 3, 3] in world units."""
        L = N.load()
        fn = L.bs_dual_contour_qef if self.qef else L.bs_dual_contour
        n = C.c_uint64()
        N.check(fn(volume.ctx.h, volume.h, self.voxel_size, None, 0, C.byref(n)), volume.ctx.h)
        out = np.zeros((max(n.value, 1), 3, 3), np.float32)
        N.check(fn(volume.ctx.h, volume.h, self.voxel_size, out.ctypes.data, n.value, C.byref(n)), volume.ctx.h)
        return out[: n.value]


class MarchingCubesMesher:
    """MarchingCubesMesher (voxel/meshing/marching_cubes.rs:17-63) on the GPU:
    the reference's cubes and edge intersections with a face-consistent
    polygon tiling of this library's own (see bs_marching_cubes)."""

    def __init__(self):
        self.voxel_size = 1.0

    def with_voxel_size(self, size):
        self.voxel_size = float(size)
        return self

    def set_voxel_size(self, size):
        self.voxel_size = float(size)
        return self

    def mesh(self, volume):
        """Triangle soup as float32[n, 3, 3] in world units."""
        L = N.load()
        n = C.c_uint64()
        N.check(L.bs_marching_cubes(volume.ctx.h, volume.h, self.voxel_size, None, 0, C.byref(n)), volume.ctx.h)
        out = np.zeros((max(n.value, 1), 3, 3), np.float32)
        N.check(L.bs_marching_cubes(volume.ctx.h, volume.h, self.voxel_size, out.ctypes.data, n.value, C.byref(n)),
                volume.ctx.h)
        return out[: n.value]


class CornerTable:
    """Corner-table mesh built from a triangle soup (bs_corner_table)."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            try:
                N.load().bs_corner_table_free(self.h)
            except Exception:
                pass
            self.h = None

    @staticmethod
    def from_triangles_soup(tris, ctx=None):
        """CornerTable::from_triangles_soup (builder.rs:97-101)."""
        ctx = ctx or default_context()
        t = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        out = C.c_void_p()
        N.check(N.load().bs_corner_table_from_soup(ctx.h, t.ctypes.data, len(t), C.byref(out)), ctx.h)
        return CornerTable(out)

    @staticmethod
    def from_marching_cubes(volume, voxel_size):
        out = C.c_void_p()
        N.check(N.load().bs_corner_table_from_marching_cubes(volume.ctx.h, volume.h, float(voxel_size), C.byref(out)),
                volume.ctx.h)
        return CornerTable(out)

    @staticmethod
    def from_dual_contouring(volume, voxel_size):
        out = C.c_void_p()
        N.check(N.load().bs_corner_table_from_dual_contour(volume.ctx.h, volume.h, float(voxel_size), C.byref(out)),
                volume.ctx.h)
        return CornerTable(out)

    def counts(self):
        a, b, c, d = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        N.check(N.load().bs_corner_table_counts(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return {"faces": a.value, "vertices": b.value, "vertex_slots": c.value, "corners": d.value}

    def faces_count(self):
        return self.counts()["faces"]

    def vertices_count(self):
        return self.counts()["vertices"]

    def export(self):
        c = self.counts()
        pos = np.zeros((c["vertex_slots"], 3), np.float32)
        dele = np.zeros(c["vertex_slots"], np.uint8)
        vc = np.zeros(c["vertex_slots"], np.int32)
        cv = np.zeros(c["corners"], np.int32)
        co = np.zeros(c["corners"], np.int32)
        N.check(N.load().bs_corner_table_export(self.h, pos.ctypes.data, dele.ctypes.data, vc.ctypes.data,
                                                cv.ctypes.data, co.ctypes.data))
        return {"positions": pos, "deleted": dele.astype(bool), "vertex_corner": vc, "corner_vertex": cv,
                "corner_opposite": co}


class VoxelRemesher:
    """VoxelRemesher (remeshing/voxel.rs:44-95): mesh -> SDF -> surface -> CornerTable.

    Manifold (the reference's default) meshes with MarchingCubesMesher,
    FeaturePreserving with dual contouring.  The band width defaults to 0
    like the reference; with_narrow_band_width is an extension."""

    FEATURE_PRESERVING = "FeaturePreserving"
    MANIFOLD = "Manifold"

    def __init__(self, ctx=None):
        self.m2v = MeshToVolume(ctx)
        self.voxel_size = 1.0
        self.method = self.MANIFOLD

    def with_voxel_size(self, size):
        self.m2v.with_voxel_size(size)
        self.voxel_size = float(size)
        return self

    def with_narrow_band_width(self, width):
        self.m2v.with_narrow_band_width(width)
        return self

    def with_meshing_method(self, method):
        self.method = method
        return self

    def remesh(self, mesh):
        vol = self.m2v.convert(mesh)
        if vol is None:
            return None
        if self.method == self.FEATURE_PRESERVING:
            return CornerTable.from_dual_contouring(vol, self.voxel_size)
        return CornerTable.from_marching_cubes(vol, self.voxel_size)
