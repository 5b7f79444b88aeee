"""Loader of librg.so, the in-tree CUDA library of the explicit hot path.

The library is built by :func:`openradioss_gb300.build.build` (nvcc,
sm_103a).  Loading fails loudly when it is missing: the product has no CPU
path.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "librg.so")
HEADER = os.path.join(HERE, "..", "include", "rg_api.h")

_lib = None

# (name, restype, argtypes) for every entry point of include/rg_api.h
_vp, _ip, _dp = C.c_void_p, C.c_int, C.c_double
SIGNATURES = [
    ("rg_ctx_create", _ip, [_ip, C.POINTER(C.c_void_p)]),
    ("rg_ctx_destroy", _ip, [_vp]),
    ("rg_last_error", C.c_char_p, [_vp]),
    ("rg_set_precision", _ip, [_vp, _ip]),
    ("rg_mesh_upload", _ip, [_vp, _ip, _vp, _vp, _vp, _vp, _vp]),
    ("rg_hexa_group_add", _ip, [_vp, _ip, _vp, _ip, _vp, _vp, _vp, _vp, _ip, _ip, _ip]),
    ("rg_shell_group_add", _ip, [_vp, _ip, _vp, _ip, _vp, _vp, _vp, _vp, _vp, _ip, _ip]),
    ("rg_rwall_add", _ip, [_vp, _vp, _vp, _dp]),
    ("rg_rlink_add", _ip, [_vp, _ip, _vp, _ip, _ip]),
    ("rg_rlink_set_active", _ip, [_vp, _ip, _ip]),
    ("rg_set_shell_frame", _ip, [_vp, _ip]),
    ("rg_set_nodal_dt", _ip, [_vp, _dp, _dp]),
    ("rg_skyline_set", _ip, [_vp, _vp, _vp, _vp]),
    ("rg_finalize", _ip, [_vp, _dp, _dp, _dp, _dp]),
    ("rg_skyline_get", _ip, [_vp, _vp, _vp, _vp, _vp]),
    ("rg_cycle", _ip, [_vp, _ip]),
    ("rg_synchronize", _ip, [_vp]),
    ("rg_forint_step", _ip, [_vp, _vp, _vp, _vp, _dp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("rg_cycle_host", _ip, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("rg_host_register", _ip, [_vp, _vp, C.c_ulonglong]),
    ("rg_host_unregister", _ip, [_vp, _vp]),
    ("rg_download_nodes", _ip, [_vp, _vp, _vp, _vp, _vp]),
    ("rg_download_forces", _ip, [_vp, _vp, _vp, _vp]),
    ("rg_download_hexa_state", _ip, [_vp, _ip, _vp]),
    ("rg_download_shell_state", _ip, [_vp, _ip, _vp]),
    ("rg_get_time", _ip, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("rg_energy", _ip, [_vp, _vp, _vp, _vp, _vp]),
    ("rg_energy_balance", _ip, [_vp, _vp, _ip]),
    ("rg_set_dtmin", _ip, [_vp, _ip, _ip, _dp]),
    ("rg_set_parts", _ip, [_vp, _ip, _vp, _vp]),
    ("rg_part_count", _ip, [_vp, _vp]),
    ("rg_part_sums_due", _ip, [_vp]),
    ("rg_part_sums", _ip, [_vp, _vp, _ip]),
    ("rg_status", _ip, [_vp]),
    ("rg_snapshot_size", _ip, [_vp, _vp]),
    ("rg_snapshot", _ip, [_vp, _vp, C.c_ulonglong]),
    ("rg_restore", _ip, [_vp, _vp, C.c_ulonglong]),
    ("rg_info", _ip, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("rg_set_timing", _ip, [_vp, _ip]),
    ("rg_kernel_times", _ip, [_vp, _vp]),
    ("rg_time_cycles", _ip, [_vp, _ip, _vp]),
    ("rg_time_cycles_cold", _ip, [_vp, _ip, C.c_ulonglong, _vp]),
    ("rg_kinetic_energy_noalloc", _ip, [_ip, _ip, _vp, _vp, _vp]),
    ("rg_fp64_peak", _ip, [_ip, _vp]),
    ("rg_batch_create", _ip, [_ip, C.POINTER(C.c_void_p)]),
    ("rg_batch_destroy", _ip, [_vp]),
    ("rg_batch_last_error", C.c_char_p, [_vp]),
    ("rg_batch_add", _ip, [_vp, _vp, _ip]),
    ("rg_batch_remove", _ip, [_vp, _ip]),
    ("rg_batch_set_target", _ip, [_vp, _ip, _ip]),
    ("rg_batch_set_config", _ip, [_vp, _ip, _ip, _ip, _ip]),
    ("rg_batch_get_config", _ip, [_vp, _vp]),
    ("rg_batch_cycle", _ip, [_vp, _ip]),
    ("rg_batch_synchronize", _ip, [_vp]),
    ("rg_batch_time_cycles", _ip, [_vp, _ip, _vp]),
    ("rg_batch_progress", _ip, [_vp, _vp, _ip, _vp]),
    ("rg_batch_job_status", _ip, [_vp, _vp, _ip]),
    ("rg_batch_set_barrier_test", _ip, [_vp, C.c_uint, _ip, C.c_uint]),
    ("rg_batch_autotune", _ip, [_vp, _ip, _vp, _ip, _vp]),
]


def lib(path=None):
    """Load librg.so (building nothing): raises if it is absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB
    if not os.path.exists(p):
        raise RuntimeError("librg.so not found at %s: run openradioss_gb300.build.build() "
                           "(nvcc, sm_103a) first; there is no CPU fallback" % p)
    L = C.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = L
    return L
