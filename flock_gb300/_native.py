"""ctypes binding of libflock_gb300.so (the C ABI of include/flock_gb300.h).

The library is built in-tree by ``__graft_entry__.build()`` into ``flock_gb300/_lib``.
There is no fallback: if the library is missing or fails to load, every entry point
raises ``NativeLibraryError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libflock_gb300.so")

#: Exported symbols, in declaration order of include/flock_gb300.h.
EXPORTS = (
    "flock_gb300_input_record_bytes",
    "flock_gb300_setup_new",
    "flock_gb300_setup_free",
    "flock_gb300_setup_info",
    "flock_gb300_prove_fast",
    "flock_gb300_prove_fast_device",
    "flock_gb300_setup_stream",
    "flock_gb300_set_stage_timing",
    "flock_gb300_last_stage_ms",
    "flock_gb300_stage_name",
    "flock_gb300_last_transfer_bytes",
    "flock_gb300_launch_count",
    "flock_gb300_last_phase_ms",
    "flock_gb300_commit_cap_noalloc",
    "flock_gb300_estimate_device_bytes",
    "flock_gb300_prove_batch",
    "flock_gb300_server_new",
    "flock_gb300_server_submit",
    "flock_gb300_server_poll",
    "flock_gb300_server_prove_batch",
    "flock_gb300_union_setup_new",
    "flock_gb300_union_setup_free",
    "flock_gb300_prove_union",
    "flock_gb300_mixed_proof_io",
    "flock_gb300_f128_mul_rate",
    "flock_gb300_f128_table_mix_rate",
    "flock_gb300_proof_io",
    "flock_gb300_server_free",
    "flock_gb300_free",
    "flock_gb300_device_count",
    "flock_gb300_last_error",
)

BLAKE3, SHA256, KECCAK = 0, 1, 2
OK, EINVAL, ECUDA, EINTERNAL, PENDING = 0, 1, 2, 3, 4


class Request(ctypes.Structure):
    _fields_ = [("hash_kind", ctypes.c_int), ("n_blocks", ctypes.c_uint64), ("inputs", ctypes.c_void_p),
                ("domain", ctypes.c_char_p), ("domain_len", ctypes.c_size_t)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("bundle", ctypes.POINTER(ctypes.c_uint8)), ("bundle_len", ctypes.c_size_t),
                ("latency_ms", ctypes.c_double)]


class NativeLibraryError(RuntimeError):
    """The CUDA library is not built or cannot be loaded."""


class FlockError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


_lock = threading.Lock()
_lib = None


def load() -> ctypes.CDLL:
    """Load (once) and return the library, declaring every signature."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise NativeLibraryError(
                f"{LIB_PATH} is missing: build the CUDA extension with __graft_entry__.build()"
            )
        try:
            lib = ctypes.CDLL(LIB_PATH)
        except OSError as e:  # pragma: no cover - depends on the machine
            raise NativeLibraryError(f"cannot load {LIB_PATH}: {e}") from e
        c = ctypes
        lib.flock_gb300_input_record_bytes.argtypes = [c.c_int]
        lib.flock_gb300_input_record_bytes.restype = c.c_size_t
        lib.flock_gb300_setup_new.argtypes = [c.c_int, c.c_uint64, c.POINTER(c.c_void_p)]
        lib.flock_gb300_setup_new.restype = c.c_int
        lib.flock_gb300_setup_free.argtypes = [c.c_void_p]
        lib.flock_gb300_setup_free.restype = None
        lib.flock_gb300_setup_info.argtypes = [c.c_void_p, c.POINTER(c.c_uint32), c.POINTER(c.c_uint32),
                                               c.POINTER(c.c_uint32), c.c_char_p]
        lib.flock_gb300_setup_info.restype = c.c_int
        lib.flock_gb300_prove_fast.argtypes = [
            c.c_void_p, c.c_void_p, c.c_size_t, c.c_char_p, c.c_size_t,
            c.POINTER(c.POINTER(c.c_uint8)), c.POINTER(c.c_size_t),
        ]
        lib.flock_gb300_prove_fast.restype = c.c_int
        lib.flock_gb300_prove_fast_device.argtypes = lib.flock_gb300_prove_fast.argtypes
        lib.flock_gb300_prove_fast_device.restype = c.c_int
        lib.flock_gb300_setup_stream.argtypes = [c.c_void_p, c.POINTER(c.c_void_p)]
        lib.flock_gb300_setup_stream.restype = c.c_int
        lib.flock_gb300_set_stage_timing.argtypes = [c.c_void_p, c.c_uint32]
        lib.flock_gb300_set_stage_timing.restype = c.c_int
        lib.flock_gb300_last_stage_ms.argtypes = [c.c_void_p, c.POINTER(c.c_double), c.POINTER(c.c_uint32), c.c_int]
        lib.flock_gb300_last_stage_ms.restype = c.c_int
        lib.flock_gb300_stage_name.argtypes = [c.c_int]
        lib.flock_gb300_stage_name.restype = c.c_char_p
        lib.flock_gb300_last_transfer_bytes.argtypes = [c.c_void_p, c.POINTER(c.c_uint64), c.POINTER(c.c_uint64)]
        lib.flock_gb300_last_transfer_bytes.restype = c.c_int
        lib.flock_gb300_launch_count.argtypes = []
        lib.flock_gb300_launch_count.restype = c.c_uint64
        lib.flock_gb300_last_phase_ms.argtypes = [c.c_void_p, c.POINTER(c.c_double)]
        lib.flock_gb300_last_phase_ms.restype = c.c_int
        lib.flock_gb300_commit_cap_noalloc.argtypes = [c.c_int, c.c_void_p, c.c_uint64, c.c_char_p, c.c_size_t,
                                                       c.POINTER(c.c_size_t), c.c_void_p]
        lib.flock_gb300_commit_cap_noalloc.restype = c.c_int
        lib.flock_gb300_estimate_device_bytes.argtypes = [c.c_int, c.c_uint64, c.POINTER(c.c_uint64)]
        lib.flock_gb300_estimate_device_bytes.restype = c.c_int
        lib.flock_gb300_prove_batch.argtypes = [c.POINTER(Request), c.c_size_t, c.c_int, c.c_uint64, c.POINTER(Result)]
        lib.flock_gb300_prove_batch.restype = c.c_int
        lib.flock_gb300_server_new.argtypes = [c.c_uint64, c.c_int, c.POINTER(c.c_void_p)]
        lib.flock_gb300_server_new.restype = c.c_int
        lib.flock_gb300_server_submit.argtypes = [c.c_void_p, c.POINTER(Request), c.POINTER(c.c_uint64)]
        lib.flock_gb300_server_submit.restype = c.c_int
        lib.flock_gb300_server_poll.argtypes = [c.c_void_p, c.c_uint64, c.c_int, c.POINTER(Result)]
        lib.flock_gb300_server_poll.restype = c.c_int
        lib.flock_gb300_server_prove_batch.argtypes = [c.c_void_p, c.POINTER(Request), c.c_size_t, c.POINTER(Result)]
        lib.flock_gb300_server_prove_batch.restype = c.c_int
        lib.flock_gb300_proof_io.argtypes = [c.c_int, c.c_uint64, c.c_char_p, c.c_size_t,
                                             c.POINTER(c.POINTER(c.c_uint8)), c.POINTER(c.c_size_t)]
        lib.flock_gb300_proof_io.restype = c.c_int
        lib.flock_gb300_union_setup_new.argtypes = [c.POINTER(c.c_int), c.c_size_t, c.c_uint32,
                                                    c.POINTER(c.c_void_p), c.POINTER(c.c_int)]
        lib.flock_gb300_union_setup_new.restype = c.c_int
        lib.flock_gb300_union_setup_free.argtypes = [c.c_void_p]
        lib.flock_gb300_union_setup_free.restype = None
        lib.flock_gb300_prove_union.argtypes = [c.c_void_p, c.POINTER(c.c_uint64), c.POINTER(c.c_void_p), c.c_char_p,
                                                c.c_size_t, c.POINTER(c.POINTER(c.c_uint8)), c.POINTER(c.c_size_t)]
        lib.flock_gb300_prove_union.restype = c.c_int
        lib.flock_gb300_mixed_proof_io.argtypes = [c.c_void_p, c.POINTER(c.c_uint64), c.c_char_p, c.c_size_t,
                                                   c.POINTER(c.POINTER(c.c_uint8)), c.POINTER(c.c_size_t)]
        lib.flock_gb300_mixed_proof_io.restype = c.c_int
        lib.flock_gb300_f128_mul_rate.argtypes = [c.c_int, c.POINTER(c.c_double)]
        lib.flock_gb300_f128_mul_rate.restype = c.c_int
        lib.flock_gb300_f128_table_mix_rate.argtypes = [c.c_int, c.POINTER(c.c_double)]
        lib.flock_gb300_f128_table_mix_rate.restype = c.c_int
        lib.flock_gb300_server_free.argtypes = [c.c_void_p]
        lib.flock_gb300_server_free.restype = None
        lib.flock_gb300_free.argtypes = [c.POINTER(c.c_uint8)]
        lib.flock_gb300_free.restype = None
        lib.flock_gb300_device_count.argtypes = []
        lib.flock_gb300_device_count.restype = c.c_int
        lib.flock_gb300_last_error.argtypes = []
        lib.flock_gb300_last_error.restype = c.c_char_p
        _lib = lib
        return lib


def check(code: int) -> None:
    if code != OK:
        msg = load().flock_gb300_last_error().decode("utf-8", "replace")
        raise FlockError(code, msg)
