"""bs_dual_contour_noalloc: dual contouring for callers that cannot allocate
device memory (their host pre-allocates everything, or forbids driver
allocations while it runs).  The entry point works in a static device array;
these tests check, through the C ABI, that two calls in a row give exactly the
triangles of the allocating entry point bs_dual_contour (the tolerance of the
dual-contouring tests: bit-identical), on a tile-free volume and on a union
with active tiles, that over-limit inputs are rejected, and that a rejected
call leaves the next one correct."""
import ctypes

import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import _native as N
from baby_shark_gb300 import synthetic
from tests.gpu_common import context

pytestmark = pytest.mark.gpu

BS_ERR_CAPACITY = 4


def _device_arrays(torch, vol):
    dev = torch.device("cuda", 0)
    o, val, m = vol.export()
    to, ts, tv = vol.tiles()
    put = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dt)).to(dev)  # noqa: E731
    return dict(
        o=put(o, np.int32), v=put(val, np.float32), m=put(np.asarray(m, np.uint32).view(np.int32), np.int32),
        to=put(to.reshape(-1, 3), np.int32), ts=put(ts, np.int32), tv=put(tv, np.float32),
        n=len(o), nt=len(ts))


def _call(lib, torch, d, h, out, n_tiles=None):
    stream = torch.cuda.current_stream(torch.device("cuda", 0))
    n = ctypes.c_uint64()
    nt = d["nt"] if n_tiles is None else n_tiles
    tp = (lambda t: t.data_ptr() if nt else None)
    st = lib.bs_dual_contour_noalloc(0, ctypes.c_void_p(stream.cuda_stream), d["o"].data_ptr(), d["v"].data_ptr(),
                                     d["m"].data_ptr(), d["n"], tp(d["to"]), tp(d["ts"]), tp(d["tv"]), nt, h,
                                     out.data_ptr() if out is not None else None,
                                     out.shape[0] if out is not None else 0, ctypes.byref(n))
    return st, n.value


def _check_twice(torch, vol, h):
    ref = bs.DualContouringMesher().with_voxel_size(h).mesh(vol).reshape(-1, 9)
    d = _device_arrays(torch, vol)
    torch.cuda.synchronize()
    lib = N.load()
    for _ in range(2):
        out = torch.full((len(ref) + 8, 9), float("nan"), dtype=torch.float32, device=torch.device("cuda", 0))
        st, n = _call(lib, torch, d, h, out)
        assert st == 0, N.STATUS.get(st)
        assert n == len(ref)
        got = out[:n].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    return ref, d


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    ctx = context()
    v, f = synthetic.config1()
    vol = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((v, f))
    ref, _ = _check_twice(torch, vol, 0.02)
    assert len(ref) > 1000


def test_noalloc_union_with_tiles_matches_allocating_entry_point_twice():
    """A boolean result with active tiles: with the exported tiles passed in,
    the triangles equal bs_dual_contour's bit for bit."""
    torch = pytest.importorskip("torch")
    va, fa = synthetic.icosphere(3, 0.6, 0.02, seed=11)
    vb, fb = synthetic.icosphere(3, 0.5, 0.02, seed=12)
    vb = vb + np.array([0.45, 0.1, -0.05], np.float32)
    ctx = context()
    a = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((va, fa))
    b = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((vb, fb))
    u = a.union(b)
    assert u.counts()["tiles"] > 0
    ref, d = _check_twice(torch, u, 0.02)
    assert len(ref) > 1000


def test_noalloc_rejects_too_many_leaves():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    small = torch.zeros(4096, dtype=torch.int32, device=dev)  # real buffers: never read past the size check
    lib = N.load()
    n = ctypes.c_uint64()
    p = small.data_ptr()
    st = lib.bs_dual_contour_noalloc(0, None, p, p, p, 1 << 40, None, None, None, 0, 0.02, p, 10, ctypes.byref(n))
    assert st == BS_ERR_CAPACITY
    st = lib.bs_dual_contour_noalloc(0, None, p, p, p, 1, p, p, p, 1 << 40, 0.02, p, 10, ctypes.byref(n))
    assert st == BS_ERR_CAPACITY


def test_noalloc_crossing_capacity_then_normal_call():
    """A checkerboard of signs over 300 fully active leaves has more than
    403,000 sign-change edges, beyond the 393,216 the static array holds: the
    call returns BS_ERR_CAPACITY before writing crossings, and the next call
    on a normal volume still matches bs_dual_contour bit for bit."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    org = np.array([(8 * i, 8 * j, 8 * k) for i in range(10) for j in range(6) for k in range(5)], np.int32)
    g = np.arange(512)
    par = ((g >> 6) + ((g >> 3) & 7) + (g & 7)) & 1
    vals = np.tile(np.where(par == 0, 0.5, -0.5).astype(np.float32), (len(org), 1))
    masks = np.full((len(org), 16), 0xFFFFFFFF, np.uint32)
    d = dict(o=torch.from_numpy(org).to(dev), v=torch.from_numpy(vals).to(dev),
             m=torch.from_numpy(masks.view(np.int32)).to(dev), to=None, ts=None, tv=None, n=len(org), nt=0)
    out = torch.zeros((16, 9), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    st, _ = _call(N.load(), torch, d, 0.1, out)
    assert st == BS_ERR_CAPACITY
    ctx = context()
    v, f = synthetic.config1()
    vol = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((v, f))
    _check_twice(torch, vol, 0.02)
