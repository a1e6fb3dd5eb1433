"""CPU-side checks of the C ABI library: it loads and exports every symbol
include/baby_shark_gb300.h declares (no compute is called without a GPU)."""
import ctypes
import glob
import os
import re

from baby_shark_gb300 import _native as N
from baby_shark_gb300 import build as bs_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(bs_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    path = bs_build.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    names = declared_symbols()
    assert names <= set(N.SIGNATURES), sorted(names - set(N.SIGNATURES))


def test_status_strings_without_gpu():
    lib = N.load()
    assert lib.bs_status_string(0) == b"ok"
    assert lib.bs_status_string(2) == b"empty input"


def test_params_default_matches_reference():
    lib = N.load()
    p = N.M2VParams()
    lib.bs_m2v_params_default(ctypes.byref(p))
    assert (p.voxel_size, p.band_width) == (1.0, 0)  # MeshToVolume::default (mesh_to_volume.rs:223-236)
    assert abs(p.wn_beta - 2.0) < 1e-7 and abs(p.wn_threshold - 0.2) < 1e-7  # mesh_to_volume.rs:264-266


def test_every_call_rejects_null_arguments_before_device_work():
    """Every status-returning entry point checks its handles, pointers and
    sizes before it touches a device: with null pointers and zero sizes it
    returns BS_ERR_INVALID_ARG (where the crate would panic on a missing
    object, the boundary reports a status)."""
    lib = N.load()
    checked = 0
    for name, (res, args) in N.SIGNATURES.items():
        if res is not N.i32 or name == "bs_mlp_num_params":
            continue
        vals = [0.0 if a in (ctypes.c_float, ctypes.c_double) else
                0 if a in (ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64) else None
                for a in args]
        assert getattr(lib, name)(*vals) == 1, name  # BS_ERR_INVALID_ARG
        checked += 1
    assert checked >= 50


def test_context_creation_without_a_device():
    import pytest
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = N.load()
    out = ctypes.c_void_p()
    assert lib.bs_ctx_create(0, None, ctypes.byref(out)) == 8  # BS_ERR_NO_DEVICE
    assert not out.value
