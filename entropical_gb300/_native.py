"""ctypes binding of the C ABI declared in include/entropical_gb300.h.

The library is loaded from the package's own ``lib/`` directory. There is no
CPU fallback: if the compiled CUDA library is missing or no device is present,
every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import _build

_lock = threading.Lock()
_lib: C.CDLL | None = None

c_size_p = C.POINTER(C.c_size_t)
c_u32_p = C.POINTER(C.c_uint32)
c_f32_p = C.POINTER(C.c_float)
c_f64_p = C.POINTER(C.c_double)


class CallStats(C.Structure):
    _fields_ = [
        ("candidate_pairs", C.c_uint64),
        ("tiles", C.c_uint64),
        ("kernel_launches", C.c_uint32),
        ("instances", C.c_uint32),
        ("pair_kernel_ms", C.c_float),
        ("total_ms", C.c_float),
        ("candidate_pairs_by_dim", C.c_uint64 * 3),
        ("pair_kernel_ms_by_dim", C.c_float * 3),
        ("moment_target_ms", C.c_float),
        ("moment_edge_ms", C.c_float),
    ]


class Tuning(C.Structure):
    """ent_tuning: pair-kernel tile shapes."""
    _fields_ = [("targets_per_warp", C.c_uint32 * 3), ("cells_per_h", C.c_uint32),
                ("pair_variant", C.c_uint32), ("pair_variant_by_dim", C.c_uint32 * 3),
                ("cells_per_h3", C.c_uint32), ("moment_cells_per_h", C.c_uint32)]


class NativeError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"entropical_gb300 status {status}: {msg}")
        self.status = status


# name -> (restype, argtypes)
SIGNATURES: dict[str, tuple] = {
    "ent_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "ent_destroy": (None, [C.c_void_p]),
    "ent_status_string": (C.c_char_p, [C.c_int]),
    "ent_last_error": (C.c_char_p, [C.c_void_p]),
    "ent_last_stats": (C.c_int, [C.c_void_p, C.POINTER(CallStats)]),
    "ent_set_tuning": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ent_log64_selftest": (C.c_int, [C.c_void_p, c_f64_p, C.c_size_t, c_f64_p]),
    "ent_wait_selftest": (C.c_int, [C.c_void_p]),
    "ent_ilog_selftest": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_size_t,
                                    C.POINTER(C.c_int64)]),
    "ent_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32, C.c_uint32,
                               C.c_void_p]),
    "ent_autotune_cache_size": (C.c_size_t, [C.c_void_p]),
    "ent_get_tuning": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ent_densities": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_u32_p, c_f32_p,
                                c_u32_p, C.c_uint32, C.c_uint32, C.c_void_p, c_size_p]),
    "ent_densities_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_u32_p,
                                       c_f32_p, c_u32_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                       c_size_p]),
    "ent_densities_part_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t,
                                            c_u32_p, c_f32_p, c_u32_p, C.c_uint32, C.c_uint32,
                                            C.c_uint32, C.c_uint32, C.c_void_p, c_size_p,
                                            c_f64_p]),
    "ent_support_counts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_u32_p,
                                     c_f32_p, c_u32_p, C.c_uint32, C.c_void_p, c_size_p]),
    "ent_mi_all_pairs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_f32_p,
                                   C.c_uint32, c_f64_p, c_f64_p]),
    "ent_mi_all_pairs_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t,
                                          c_f32_p, C.c_uint32, c_f64_p, c_f64_p]),
    "ent_entropy_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32, c_f64_p]),
    "ent_mi_entropies_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_f32_p,
                                          C.POINTER(C.c_uint64), C.c_size_t, C.c_uint32,
                                          c_f64_p]),
    "ent_te_entropies_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_f32_p,
                                          c_u32_p, C.c_size_t, C.POINTER(C.c_uint64), C.c_size_t,
                                          C.c_uint32, c_f64_p]),
    "ent_reference_estimator": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t,
                                          c_f32_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                          c_f64_p]),
    "ent_dens_all": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_f32_p,
                               C.c_uint32, c_u32_p, C.c_uint32, C.c_void_p, c_size_p,
                               c_size_p]),
    "ent_coords_file_shape": (C.c_int, [C.c_char_p, c_size_p, c_size_p]),
    "ent_read_coords": (C.c_int, [C.c_char_p, c_size_p, C.c_size_t, C.c_char, C.c_void_p,
                                  C.c_size_t, C.c_size_t]),
    "ent_load_coords_device": (C.c_int, [C.c_void_p, C.c_char_p, c_size_p, C.c_size_t,
                                         C.c_void_p, C.c_size_t, C.c_size_t]),
    "ent_io_last_error": (C.c_char_p, []),
    "ent_xtc_file_shape": (C.c_int, [C.c_char_p, c_size_p, c_size_p]),
    "ent_load_xtc_device": (C.c_int, [C.c_void_p, C.c_char_p, c_size_p, C.c_size_t,
                                      C.c_void_p, C.c_size_t, C.c_size_t]),
    "ent_read_xtc": (C.c_int, [C.c_void_p, C.c_char_p, c_size_p, C.c_size_t, C.c_char,
                               C.c_void_p, C.c_size_t, C.c_size_t]),
    "ent_write_xtc": (C.c_int, [C.c_char_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_char,
                                C.c_float]),
    "ent_xtc_last_error": (C.c_char_p, []),
    "ent_te_all_pairs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_f32_p,
                                   c_u32_p, C.c_size_t, C.c_uint32, c_f64_p]),
    "ent_te_all_pairs_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t,
                                          c_f32_p, c_u32_p, C.c_size_t, C.c_uint32, c_f64_p]),
    "ent_neighbor_counts": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_float, C.c_uint32,
                                      C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]),
    "ent_hestimate_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32, c_f32_p,
                                      C.c_void_p]),
    "ent_hestimate_learned": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                        C.c_uint32, C.c_uint32, c_f32_p, C.c_void_p]),
    "ent_mlp_param_count": (C.c_size_t, []),
    "ent_mlp_create": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "ent_mlp_destroy": (None, [C.c_void_p]),
    "ent_mlp_set_params": (C.c_int, [C.c_void_p, c_f32_p, c_f32_p, c_f32_p]),
    "ent_mlp_get_params": (C.c_int, [C.c_void_p, c_f32_p, c_f32_p, c_f32_p]),
    "ent_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, c_f32_p, C.c_size_t, c_f32_p]),
    "ent_mlp_gradients": (C.c_int, [C.c_void_p, C.c_void_p, c_f32_p, c_f32_p, c_f32_p,
                                    C.c_size_t, c_f32_p, c_f32_p]),
    "ent_mlp_train_step": (C.c_int, [C.c_void_p, C.c_void_p, c_f32_p, c_f32_p, c_f32_p,
                                     C.c_size_t, C.c_float, c_f32_p]),
    "ent_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, c_f32_p]),
    "ent_density_1d_noalloc": (C.c_int, [C.c_void_p, C.c_size_t, C.c_float, C.c_void_p,
                                         C.c_void_p]),
    "ent_epa_convolution": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_float, c_f32_p]),
    "ent_hestimate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_u32_p,
                                C.c_size_t, C.c_uint32, c_f32_p, C.c_uint32, c_f32_p,
                                C.c_void_p]),
    "ent_hestimate_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_u32_p,
                                       C.c_size_t, C.c_uint32, c_f32_p, C.c_uint32, c_f32_p,
                                       C.c_void_p]),
}


class HestStats(C.Structure):
    """ent_hest_stats: per-column bandwidth-search statistics."""
    _fields_ = [
        ("h0", C.c_float),
        ("conv_evals", C.c_uint32),
        ("levels_skipped", C.c_uint32),
        ("warm_converged", C.c_uint32),
    ]


class Instance(C.Structure):
    """ent_instance: one entry of an uneven entropy batch."""
    _fields_ = [
        ("coords", C.c_void_p),
        ("n", C.c_uint64),
        ("d", C.c_uint32),
        ("h", C.c_float * 3),
    ]


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load (building first if needed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if not path.exists():
            if not build_if_missing:
                raise RuntimeError(f"entropical_gb300 native library missing: {path}")
            _build.build()
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def library_path() -> Path:
    return _build.lib_path()


def check(lib: C.CDLL, ctx: C.c_void_p | None, status: int) -> None:
    if status != 0:
        msg = ""
        if ctx is not None:
            raw = lib.ent_last_error(ctx)
            msg = raw.decode() if raw else ""
        if not msg:
            msg = lib.ent_status_string(status).decode()
        raise NativeError(status, msg)
