"""Helpers shared by the GPU parity tests: build/load the native library and
compare GPU volumes with oracle volumes leaf by leaf."""
import numpy as np

import baby_shark_gb300 as bs
from baby_shark_gb300 import build as bs_build

_ctx = None


def context():
    global _ctx
    if _ctx is None:
        bs_build.build()
        _ctx = bs.Context(0)
    return _ctx


def as_dict(origins, values, masks):
    return {tuple(int(c) for c in o): (v, m) for o, v, m in zip(origins, values, masks)}


def unpack_mask(m):
    """uint32[16] -> bool[512] (bit i&31 of word i>>5)."""
    bits = (m[:, None] >> np.arange(32, dtype=np.uint32)[None, :]) & 1
    return bits.reshape(-1).astype(bool)


def compare_volumes(gpu, ora, check_inactive=False):
    """Returns a report dict; exact comparison of leaf sets, masks, |values| and signs."""
    go, gv, gm = gpu
    oo, ov, om = ora
    gd, od = as_dict(go, gv, gm), as_dict(oo, ov, om)
    rep = {"gpu_leaves": len(gd), "oracle_leaves": len(od), "leaf_set_equal": set(gd) == set(od),
           "mask_mismatch_leaves": 0, "value_mismatch": 0, "sign_mismatch": 0, "active": 0,
           "inactive_mismatch": 0}
    for k in set(gd) & set(od):
        v1, m1 = gd[k]
        v2, m2 = od[k]
        if not np.array_equal(m1, m2):
            rep["mask_mismatch_leaves"] += 1
        act = unpack_mask(m2) & unpack_mask(m1)
        rep["active"] += int(act.sum())
        a1, a2 = v1[act], v2[act]
        rep["value_mismatch"] += int(np.sum(np.abs(a1).view(np.uint32) != np.abs(a2).view(np.uint32)))
        rep["sign_mismatch"] += int(np.sum(np.signbit(a1) != np.signbit(a2)))
        if check_inactive:
            ia = ~(unpack_mask(m2) | unpack_mask(m1))
            rep["inactive_mismatch"] += int(np.sum(v1[ia].view(np.uint32) != v2[ia].view(np.uint32)))
    return rep
