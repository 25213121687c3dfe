"""Loader of the native library (ctwin_gb300/_lib/libctwin_gb300.so).

There is no Python or CPU fallback: when the library is missing or has no
CUDA device to run on, the calls fail with CtwError.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libctwin_gb300.so")

_lock = threading.Lock()
_lib = None


class CtwResult(ctypes.Structure):
    """struct ctw_result of include/ctwin_gb300.h."""
    _fields_ = [("tag", ctypes.c_uint64), ("res64", ctypes.c_uint64), ("b", ctypes.c_uint32),
                ("log2_degree", ctypes.c_int32), ("is_prp", ctypes.c_uint8), ("gl_ok", ctypes.c_uint8),
                ("status", ctypes.c_int8), ("reserved", ctypes.c_uint8), ("slot", ctypes.c_int32),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double),
                ("squarings", ctypes.c_longlong)]


class CtwError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ctwin_gb300 error {code}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"native library not built: {LIB_PATH} (run ctwin_gb300.build)")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, u32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_longlong
        H = ctypes.c_void_p
        sigs = {
            "ctw_last_error": ([], ctypes.c_char_p),
            "ctw_version": ([], ctypes.c_char_p),
            "ctw_device_count": ([], i32),
            "ctw_prp_create": ([i32, i32, ctypes.POINTER(H)], i32),
            "ctw_prp_destroy": ([H], i32),
            "ctw_prp_set_csize": ([H, i32], i32),
            "ctw_prp_set_prime_count": ([H, i32], i32),
            "ctw_prp_prime_count": ([H], i32),
            "ctw_prp_two_primes": ([i32, i32, u32], i32),
            "ctw_prp_set_base": ([H, u32], i32),
            "ctw_prp_set_b": ([H, vp, i32], i32),
            "ctw_prp_set": ([H, u32], i32),
            "ctw_prp_copy": ([H, i32, i32], i32),
            "ctw_prp_square_dup": ([H, vp], i32),
            "ctw_prp_mul": ([H], i32),
            "ctw_prp_mul_regs": ([H, i32, i32, i32], i32),
            "ctw_prp_square_bits": ([H, vp, i32, i64, i32], i32),
            "ctw_prp_load_exponent": ([H, vp, i32], i32),
            "ctw_prp_square_resident": ([H, i64, i32], i32),
            "ctw_prp_get_digits": ([H, i32, vp], i32),
            "ctw_prp_is_prime": ([H, i32, vp, vp], i32),
            "ctw_prp_read_regs": ([H, i32, i32, vp], i32),
            "ctw_prp_write_regs": ([H, i32, i32, vp], i32),
            "ctw_prp_run": ([H, vp, i32, vp, vp, vp], i32),
            "ctw_prp_sync": ([H], i32),
            "ctw_prp_stream": ([H], vp),
            "ctw_prp_geometry": ([H, vp, vp, vp], i32),
            "ctw_prp_launches": ([H], i64),
            "ctw_prp_test_unreachable_barrier": ([H], i32),
            "ctw_imad_peak": ([], ctypes.c_double),
            "ctw_modmul_peak": ([i32], ctypes.c_double),
            "ctw_prp_mul_noalloc": ([i32, i32, vp, vp, vp, vp, i32, vp], i32),
            "ctw_sieve_run": ([i32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, i32, vp, vp], i32),
            "ctw_sieve_write_files": ([i32, ctypes.c_uint64, ctypes.c_uint64, vp, ctypes.c_uint64, ctypes.c_uint64,
                                       ctypes.c_char_p], i32),
            "ctw_sieve_launches": ([], i64),
            "ctw_mulmod64_peak": ([], ctypes.c_double),
            "ctw_sieve_factors": ([i32, ctypes.c_uint64, ctypes.c_uint64, i32, ctypes.c_uint64, vp, ctypes.c_uint64,
                                   vp], i32),
            "ctw_gfsieve_check": ([i32, ctypes.c_uint64, ctypes.c_uint64, i32, ctypes.c_char_p, vp, i32, vp], i32),
            "ctw_prp_create_split": ([i32, i32, i32, ctypes.POINTER(H)], i32),
            "ctw_prp_create_minus": ([i32, i32, ctypes.POINTER(H)], i32),
            "ctw_prp_shape": ([H, vp, vp, vp], i32),
            "ctw_prp_run_ex": ([H, vp, i32, i64, vp, vp, vp, vp, vp], i32),
            "ctw_prp_save_context": ([H, ctypes.c_char_p, i32, i32, ctypes.c_double], i32),
            "ctw_prp_read_context": ([H, ctypes.c_char_p, vp, vp, vp], i32),
            "ctw_context_bytes": ([i32, i32, i32], ctypes.c_size_t),
            "ctw_context_encode": ([i32, i32, i32, vp, i32, i32, ctypes.c_double, vp], i32),
            "ctw_context_decode": ([i32, i32, i32, vp, ctypes.c_size_t, vp, vp, vp, vp], i32),
            "ctw_cyclo_check_file": ([i32, ctypes.c_char_p, ctypes.c_char_p, i32, ctypes.c_double, vp, i32], i32),
            "ctw_prp_autotune": ([i32, i32, vp, vp, vp], i32),
            "ctw_prp_autotune_primes": ([i32, i32, i32, vp, vp, vp], i32),
            "ctw_pool_create": ([i32, i32, i32, i32, u32, i32, ctypes.POINTER(H)], i32),
            "ctw_pool_destroy": ([H], i32),
            "ctw_pool_create_minus": ([i32, i32, i32, u32, i32, ctypes.POINTER(H)], i32),
            "ctw_pool_slot_bytes": ([i32], ctypes.c_size_t),
            "ctw_pool_admit": ([H, u32, ctypes.c_uint64], i32),
            "ctw_pool_admit_many": ([H, vp, vp, i32, i32], i32),
            "ctw_pool_run": ([H, i32], i32),
            "ctw_pool_collect": ([H, i32], i32),
            "ctw_pool_results": ([H, vp, i32], i32),
            "ctw_pool_info": ([H, vp, vp, vp, vp, vp, vp, vp], i32),
            "ctw_pool_read_slot": ([H, i32, i32, vp], i32),
            "ctw_pool_set_prime_count": ([H, i32], i32),
            "ctw_pool_prime_count": ([H], i32),
            "ctw_pool_stream": ([H], vp),
            "ctw_pool_schedule": ([i32, u32, i32, vp, i32, vp], i32),
            "ctw_batch_create": ([vp, i32, ctypes.POINTER(H)], i32),
            "ctw_batch_run": ([H, i32], i32),
            "ctw_batch_destroy": ([H], i32),
            "ctw_batch_stream": ([H], vp),
            "ctw_batch_launches": ([H], i64),
            "ctw_batch_set_ctas_per_sm": ([H, i32], i32),
            "ctw_server_create": ([ctypes.c_size_t, i32, u32, i32, i32, ctypes.POINTER(H)], i32),
            "ctw_server_submit": ([H, i32, u32, ctypes.c_uint64], i32),
            "ctw_server_prepare": ([H, i32, i32], i32),
            "ctw_server_set_grid_lane": ([H, i32], i32),
            "ctw_server_set_grid_lanes": ([H, i32], i32),
            "ctw_server_poll": ([H, vp, i32, i32], i32),
            "ctw_server_stats": ([H, vp, vp, vp, vp, vp], i32),
            "ctw_server_clock": ([H], ctypes.c_double),
            "ctw_server_destroy": ([H], i32),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
        return _lib


def check(rc: int) -> None:
    if rc != 0:
        raise CtwError(rc, lib().ctw_last_error().decode(errors="replace"))


def ptr(a) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None
