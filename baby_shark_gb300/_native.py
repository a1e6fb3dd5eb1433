"""ctypes binding of libbs_gb300.so (the C ABI in include/baby_shark_gb300.h).

The library is built in-tree by baby_shark_gb300.build; loading fails loudly
when it is missing — there is no CPU fallback.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbs_gb300.so")

BS_OK = 0
STATUS = {
    0: "BS_OK", 1: "BS_ERR_INVALID_ARG", 2: "BS_ERR_EMPTY", 3: "BS_ERR_OOM", 4: "BS_ERR_CAPACITY",
    5: "BS_ERR_TIMEOUT", 6: "BS_ERR_CUDA", 7: "BS_ERR_UNSUPPORTED", 8: "BS_ERR_NO_DEVICE",
}

# Every symbol the header declares: (restype, argtypes).
vp, u64, i32, f32 = C.c_void_p, C.c_uint64, C.c_int, C.c_float
PP = C.POINTER(C.c_void_p)


class M2VParams(C.Structure):
    _fields_ = [("voxel_size", C.c_float), ("band_width", C.c_int32), ("wn_beta", C.c_float),
                ("wn_threshold", C.c_float), ("wn_order", C.c_int32), ("wn_tree", C.c_int32)]


SIGNATURES = {
    "bs_ctx_create": (i32, [i32, vp, PP]),
    "bs_ctx_destroy": (i32, [vp]),
    "bs_ctx_stream": (vp, [vp]),
    "bs_ctx_synchronize": (i32, [vp]),
    "bs_ctx_kernel_launches": (u64, [vp]),
    "bs_ctx_last_error": (C.c_char_p, [vp]),
    "bs_status_string": (C.c_char_p, [i32]),
    "bs_ctx_set_stage_timing": (i32, [vp, i32]),
    "bs_ctx_stage_count": (i32, [vp, C.POINTER(C.c_int)]),
    "bs_ctx_stage_info": (i32, [vp, i32, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(u64)]),
    "bs_ctx_stage_reset": (i32, [vp]),
    "bs_ctx_last_stats": (i32, [vp, C.POINTER(u64)]),
    "bs_ctx_last_counters": (i32, [vp, C.POINTER(u64)]),
    "bs_autotune_mesh_to_volume": (i32, [vp, vp, u64, vp, u64, vp, vp, vp]),
    "bs_ctx_set_launch_shape": (i32, [vp, C.c_int32, C.c_int32, C.c_int32]),
    "bs_mlp_num_params": (i32, []),
    "bs_mlp_create": (i32, [vp, vp, f32, vp, vp, C.POINTER(vp)]),
    "bs_mlp_free": (i32, [vp]),
    "bs_mlp_get_params": (i32, [vp, vp, vp]),
    "bs_mlp_predict": (i32, [vp, vp, vp, u64, vp]),
    "bs_mlp_train": (i32, [vp, vp, vp, vp, u64, C.c_uint32, C.c_uint32, f32, f32, vp]),
    "bs_mlp_gradients": (i32, [vp, vp, vp, vp, u64, C.c_uint32, vp, vp]),
    "bs_mlp_classify": (i32, [vp, vp, vp, vp, vp, u64, f32, f32, f32, vp, C.POINTER(u64)]),
    "bs_volume_band_flags": (i32, [vp, vp, vp, u64, vp]),
    "bs_ctx_memory": (i32, [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
    "bs_ctx_memory_reset": (i32, [vp, C.c_int]),
    "bs_diag_fp32_peak": (i32, [vp, C.POINTER(C.c_double)]),
    "bs_diag_check_division": (i32, [vp, C.c_uint32, C.POINTER(u64), C.POINTER(u64)]),
    "bs_winding_numbers_exact": (i32, [vp, vp, u64, vp, u64, vp, u64, vp]),
    "bs_winding_numbers_build": (i32, [vp, vp, u64, vp, u64, i32, PP]),
    "bs_winding_numbers_build_ex": (i32, [vp, vp, u64, vp, u64, i32, i32, PP]),
    "bs_winding_numbers_approximate": (i32, [vp, vp, vp, u64, f32, vp]),
    "bs_winding_numbers_free": (i32, [vp]),
    "bs_m2v_params_default": (None, [C.POINTER(M2VParams)]),
    "bs_mesh_to_volume": (i32, [vp, vp, u64, vp, u64, C.POINTER(M2VParams), PP]),
    "bs_mesh_to_volume_device": (i32, [vp, vp, u64, vp, u64, C.POINTER(M2VParams), PP]),
    "bs_mesh_to_volume_batch": (i32, [vp, u64, vp, vp, vp, vp, C.POINTER(M2VParams), vp]),
    "bs_mesh_to_volume_batch_device": (i32, [vp, u64, vp, vp, vp, vp, C.POINTER(M2VParams), vp]),
    "bs_volume_create": (i32, [vp, f32, PP]),
    "bs_volume_free": (i32, [vp]),
    "bs_volume_voxel_size": (i32, [vp, C.POINTER(C.c_float)]),
    "bs_volume_clone": (i32, [vp, vp, PP]),
    "bs_volume_counts": (i32, [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
    "bs_volume_export": (i32, [vp, vp, vp, vp, vp]),
    "bs_volume_export_tiles": (i32, [vp, vp, vp, vp, vp]),
    "bs_volume_union": (i32, [vp, vp, vp, PP]),
    "bs_volume_subtract": (i32, [vp, vp, vp, PP]),
    "bs_volume_intersect": (i32, [vp, vp, vp, PP]),
    "bs_volume_offset": (i32, [vp, vp, f32]),
    "bs_volume_from_samples": (i32, [vp, f32, C.c_int64, vp, vp, vp, PP]),
    "bs_volume_from_samples_device": (i32, [vp, f32, C.c_int64, vp, vp, vp, PP]),
    "bs_volume_sphere": (i32, [vp, f32, f32, vp, PP]),
    "bs_volume_cuboid": (i32, [vp, f32, vp, vp, PP]),
    "bs_volume_iwp": (i32, [vp, f32, vp, vp, f32, PP]),
    "bs_marching_cubes": (i32, [vp, vp, f32, vp, u64, C.POINTER(u64)]),
    "bs_dual_contour_qef": (i32, [vp, vp, f32, vp, u64, C.POINTER(u64)]),
    "bs_dual_contour": (i32, [vp, vp, f32, vp, u64, C.POINTER(u64)]),
    "bs_dual_contour_noalloc": (i32, [i32, vp, vp, vp, vp, u64, vp, vp, vp, u64, f32, vp, u64, C.POINTER(u64)]),
    "bs_corner_table_from_soup": (i32, [vp, vp, u64, PP]),
    "bs_corner_table_from_dual_contour": (i32, [vp, vp, f32, PP]),
    "bs_corner_table_from_marching_cubes": (i32, [vp, vp, f32, PP]),
    "bs_corner_table_counts": (i32, [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
    "bs_corner_table_export": (i32, [vp, vp, vp, vp, vp, vp]),
    "bs_corner_table_free": (i32, [vp]),
}

_lib = None
_lock = threading.Lock()


class BsError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("%s%s" % (STATUS.get(status, status), (": " + msg) if msg else ""))


def load(path=None):
    """Loads the native library (raises if it is not built)."""
    global _lib
    with _lock:
        if _lib is None:
            p = path or LIB_PATH
            if not os.path.exists(p):
                raise RuntimeError("libbs_gb300.so is not built (run baby_shark_gb300.build.build())")
            L = C.CDLL(p)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status, ctx=None):
    if status != BS_OK:
        msg = ""
        if ctx is not None:
            msg = (load().bs_ctx_last_error(ctx) or b"").decode(errors="replace")
        raise BsError(status, msg)
