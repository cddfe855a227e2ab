"""ctypes binding of libsphgpu.so (include/sph_gpu.h).

The library is built in-tree (mysph_gb300/build.py).  There is no CPU
fallback: if the library cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

from . import params as P

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libsphgpu.so"
HEADER = PKG.parent / "include" / "sph_gpu.h"

_lib: C.CDLL | None = None

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
vp = C.c_void_p
ctxp = C.c_void_p

SIGNATURES = {
    "sph_abi_version": (C.c_int, []),
    "sph_params_default": (C.c_int, [C.POINTER(P.SphParams)]),
    "sph_create": (C.c_int, [C.POINTER(P.SphParams), C.c_int64, C.POINTER(ctxp)]),
    "sph_destroy": (C.c_int, [ctxp]),
    "sph_set_params": (C.c_int, [ctxp, C.POINTER(P.SphParams)]),
    "sph_upload": (C.c_int, [ctxp, C.c_int64, C.c_int64] + [dp] * 8 + [ip] * 3 + [dp]),
    "sph_download": (C.c_int, [ctxp] + [dp] * 7),
    "sph_get_field": (C.c_int, [ctxp, C.c_int32, dp]),
    "sph_set_field": (C.c_int, [ctxp, C.c_int32, dp]),
    "sph_info": (C.c_int, [ctxp, i64p, i64p, i64p, dp]),
    "sph_nnps": (C.c_int, [ctxp]),
    "sph_neighbor_counts": (C.c_int, [ctxp, ip, i64p]),
    "sph_export_neighbors": (C.c_int, [ctxp, i64p, ip, C.c_int64]),
    "sph_density": (C.c_int, [ctxp, dp]),
    "sph_divergence": (C.c_int, [ctxp, dp, dp]),
    "sph_internal_force": (C.c_int, [ctxp, dp, dp, dp]),
    "sph_external_force": (C.c_int, [ctxp, dp]),
    "sph_arti_visc": (C.c_int, [ctxp, dp, dp]),
    "sph_arti_stress": (C.c_int, [ctxp, dp]),
    "sph_arti_heat": (C.c_int, [ctxp, dp]),
    "sph_energy": (C.c_int, [ctxp, C.c_int32, dp]),
    "sph_rates": (C.c_int, [ctxp, dp, dp, dp]),
    "sph_single_step": (C.c_int, [ctxp]),
    "sph_advance": (C.c_int, [ctxp, C.c_int64, dp, dp]),
    "sph_advance_async": (C.c_int, [ctxp, C.c_int64]),
    "sph_sync": (C.c_int, [ctxp, dp, dp]),
    "sph_statistics": (C.c_int, [ctxp, dp]),
    "sph_boundary": (C.c_int, [ctxp, dp]),
    "sph_courant_num": (C.c_int, [ctxp, C.c_int64, dp, dp, dp, dp]),
    "sph_step_host": (C.c_int, [ctxp, C.c_int64, dp, dp, dp, dp, dp]),
    "sph_batch_create": (C.c_int, [C.POINTER(P.SphParams), C.c_int32, C.c_int64, C.c_int64, C.POINTER(ctxp)]),
    "sph_batch_add": (C.c_int, [ctxp, C.POINTER(P.SphParams), C.c_int64, C.c_int64] + [dp] * 8 + [ip] * 3 + [dp, ip]),
    "sph_batch_remove": (C.c_int, [ctxp, C.c_int32]),
    "sph_batch_get_field": (C.c_int, [ctxp, C.c_int32, C.c_int32, dp]),
    "sph_batch_info": (C.c_int, [ctxp, C.c_int32, i64p, i64p, i64p, dp, dp, dp]),
    "sph_batch_capacity": (C.c_int, [ctxp, i64p, i64p, ip]),
    "sph_batch_slots": (C.c_int, [ctxp, ip, C.POINTER(C.c_uint8)]),
    "sph_upload_blocks": (C.c_int, [ctxp, C.c_int32, C.POINTER(P.SphBlock), C.c_int32]),
    "sph_batch_add_blocks": (C.c_int, [ctxp, C.POINTER(P.SphParams), C.c_int32, C.POINTER(P.SphBlock),
                                       C.c_int32, ip]),
    "sph_status": (C.c_int, [ctxp, C.c_char_p, C.c_size_t]),
    "sph_get_stream": (C.c_int, [ctxp, C.POINTER(vp)]),
    "sph_enable_stage_timing": (C.c_int, [ctxp, C.c_int32]),
    "sph_stage_times": (C.c_int, [ctxp, dp, i64p]),
    "sph_set_option": (C.c_int, [ctxp, C.c_int32, C.c_double]),
    "sph_launch_count": (C.c_int, [ctxp, i64p]),
    "sph_device_bytes": (C.c_int, [ctxp, i64p]),
    "sph_get_params": (C.c_int, [ctxp, C.POINTER(P.SphParams)]),
    "sph_state_bytes": (C.c_int, [ctxp, i64p]),
    "sph_state_save": (C.c_int, [ctxp, vp, C.c_int64]),
    "sph_state_load": (C.c_int, [vp, C.c_int64, C.POINTER(ctxp)]),
    "sph_sort_scratch_bytes": (C.c_int64, [C.c_int64, C.c_int32]),
    "sph_sort_pairs": (C.c_int, [vp, vp, vp, vp, C.c_int64, C.c_int32, vp, C.c_int64, vp]),
    "sph_sort_pairs_noalloc": (C.c_int, [vp, vp, vp, vp, C.c_int64, C.c_int32, vp]),
    "sph_probe_fp64_gflops": (C.c_int, [dp]),
    "sph_check_conversions": (C.c_int, [C.c_int64, C.c_uint64, i64p]),
}


def header_symbols() -> list[str]:
    """Every function declared in include/sph_gpu.h."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t)\s+(sph_\w+)\s*\(", text, re.M)))


def load(build_if_missing: bool = True) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not LIB_PATH.exists():
        raise RuntimeError(f"libsphgpu.so not found at {LIB_PATH}; run mysph_gb300/build.py")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class SphError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str = ""):
        self.status = status
        super().__init__(f"{where} failed with status {status}" + (f": {msg}" if msg else ""))
