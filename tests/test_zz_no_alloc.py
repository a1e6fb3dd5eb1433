"""bs_dual_contour_noalloc: dual contouring for callers that cannot allocate
device memory (their host pre-allocates everything, or forbids driver
allocations while it runs).  The entry point works in a static device array;
this test checks, through the C ABI, that two calls in a row give exactly the
triangles of the allocating entry point bs_dual_contour (the tolerance of the
dual-contouring tests: bit-identical)."""
import ctypes

import numpy as np
import pytest

import baby_shark_gb300 as bs
from baby_shark_gb300 import _native as N
from baby_shark_gb300 import synthetic
from tests.gpu_common import context

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    ctx = context()
    v, f = synthetic.config1()
    vol = bs.MeshToVolume(ctx).with_voxel_size(0.02).with_narrow_band_width(3).convert((v, f))
    ref = bs.DualContouringMesher().with_voxel_size(0.02).mesh(vol).reshape(-1, 9)
    assert len(ref) > 1000
    o, val, m = vol.export()
    dev = torch.device("cuda", 0)
    d_o = torch.from_numpy(np.ascontiguousarray(o, np.int32)).to(dev)
    d_v = torch.from_numpy(np.ascontiguousarray(val, np.float32)).to(dev)
    d_m = torch.from_numpy(np.ascontiguousarray(m, np.uint32).view(np.int32)).to(dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize()
    lib = N.load()
    for _ in range(2):
        out = torch.full((len(ref) + 8, 9), float("nan"), dtype=torch.float32, device=dev)
        n = ctypes.c_uint64()
        st = lib.bs_dual_contour_noalloc(0, ctypes.c_void_p(stream.cuda_stream), d_o.data_ptr(), d_v.data_ptr(),
                                         d_m.data_ptr(), len(o), 0.02, out.data_ptr(), out.shape[0], ctypes.byref(n))
        assert st == 0, N.STATUS.get(st)
        assert n.value == len(ref)
        got = out[: n.value].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_noalloc_rejects_too_many_leaves():
    lib = N.load()
    n = ctypes.c_uint64()
    fake = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.bs_dual_contour_noalloc(0, None, fake, fake, fake, 4096, 0.02, fake, 10, ctypes.byref(n))
    assert st == 4  # BS_ERR_CAPACITY
