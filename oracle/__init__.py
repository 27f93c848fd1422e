"""ORACLE — test infrastructure only.

ctypes wrapper over oracle/_build/liboracle.so, the CPU restatement of the reference's
prove_fast (cpu_backend.h). Only the tests, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` use it, always as the checker or the timed CPU reference,
never as the product path.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run __graft_entry__.build()")
        lib = ctypes.CDLL(LIB_PATH)
        c = ctypes
        lib.oracle_prove_fast.argtypes = [c.c_int, c.c_uint64, c.c_void_p, c.c_char_p, c.c_size_t,
                                          c.POINTER(c.POINTER(c.c_uint8)), c.POINTER(c.c_size_t)]
        lib.oracle_prove_fast.restype = c.c_int
        lib.oracle_free.argtypes = [c.POINTER(c.c_uint8)]
        lib.oracle_registry_digest.argtypes = [c.c_int, c.c_uint64, c.c_char_p]
        lib.oracle_registry_digest.restype = c.c_int
        lib.oracle_last_error.restype = c.c_char_p
        lib.oracle_last_phase_ms.argtypes = [c.POINTER(c.c_double)]
        lib.oracle_verify.argtypes = [c.c_int, c.c_uint64, c.c_char_p, c.c_size_t, c.c_char_p, c.c_size_t,
                                      c.c_char_p, c.c_size_t]
        lib.oracle_verify.restype = c.c_int
        lib.oracle_prove_union.argtypes = [c.POINTER(c.c_int), c.c_size_t, c.c_uint32, c.POINTER(c.c_uint64),
                                           c.POINTER(c.c_void_p), c.c_char_p, c.c_size_t,
                                           c.POINTER(c.POINTER(c.c_uint8)), c.POINTER(c.c_size_t)]
        lib.oracle_prove_union.restype = c.c_int
        lib.oracle_mixed_proof_io.argtypes = [c.POINTER(c.c_int), c.c_size_t, c.c_uint32, c.POINTER(c.c_uint64),
                                              c.c_char_p, c.c_size_t, c.POINTER(c.POINTER(c.c_uint8)),
                                              c.POINTER(c.c_size_t)]
        lib.oracle_mixed_proof_io.restype = c.c_int
        lib.oracle_verify_union.argtypes = [c.POINTER(c.c_int), c.c_size_t, c.c_uint32, c.POINTER(c.c_uint64),
                                            c.c_char_p, c.c_size_t, c.c_char_p, c.c_size_t, c.c_char_p, c.c_size_t]
        lib.oracle_verify_union.restype = c.c_int
        _lib = lib
    return _lib


def prove_fast_bytes(kind: int, inputs, domain: bytes) -> bytes:
    """Oracle prove_fast over a numpy structured array of records; returns the bundle."""
    import numpy as np

    lib = load()
    arr = np.ascontiguousarray(inputs)
    out = ctypes.POINTER(ctypes.c_uint8)()
    n = ctypes.c_size_t()
    rc = lib.oracle_prove_fast(kind, arr.shape[0], arr.ctypes.data, domain, len(domain), ctypes.byref(out),
                               ctypes.byref(n))
    if rc != 0:
        raise RuntimeError(lib.oracle_last_error().decode())
    try:
        return ctypes.string_at(out, n.value)
    finally:
        lib.oracle_free(out)


def last_phase_ms() -> dict:
    v = (ctypes.c_double * 6)()
    load().oracle_last_phase_ms(v)
    return dict(zip(("witness", "commit", "zerocheck", "lincheck", "open", "total"), list(v)))


def registry_digest(kind: int, n_blocks: int) -> bytes:
    lib = load()
    buf = ctypes.create_string_buffer(32)
    if lib.oracle_registry_digest(kind, n_blocks, buf) != 0:
        raise RuntimeError(lib.oracle_last_error().decode())
    return buf.raw


def verify(kind: int, n_blocks: int, bundle: bytes, domain: bytes) -> tuple:
    """Replays the transcript of a bundle and checks every relation of the reference
    verifier (oracle/verifier.h). Returns (accepted, reason)."""
    lib = load()
    reason = ctypes.create_string_buffer(256)
    rc = lib.oracle_verify(kind, n_blocks, bundle, len(bundle), domain, len(domain), reason, 256)
    if rc == 2:
        raise RuntimeError(reason.value.decode())
    return rc == 0, reason.value.decode()


def _union_args(kinds, counts):
    n = len(kinds)
    return (ctypes.c_int * n)(*kinds), n, (ctypes.c_uint64 * n)(*counts)


def prove_union_bytes(kinds, nu: int, counts, records, domain: bytes) -> bytes:
    """Oracle prove_fast_ligerito_union of a registry given in slot order (k_log
    descending), declared counts and per-slot record arrays; returns the bundle."""
    import numpy as np

    lib = load()
    k, n, c = _union_args(kinds, counts)
    arrs = [np.ascontiguousarray(r) for r in records]
    ptrs = (ctypes.c_void_p * n)(*[a.ctypes.data if a.size else 0 for a in arrs])
    out = ctypes.POINTER(ctypes.c_uint8)()
    ln = ctypes.c_size_t()
    if lib.oracle_prove_union(k, n, nu, c, ptrs, domain, len(domain), ctypes.byref(out), ctypes.byref(ln)) != 0:
        raise RuntimeError(lib.oracle_last_error().decode())
    try:
        return ctypes.string_at(out, ln.value)
    finally:
        lib.oracle_free(out)


def mixed_proof_io(kinds, nu: int, counts, bundle: bytes) -> bytes:
    """MixedProofBundleLigerito::to_bytes of a union bundle."""
    lib = load()
    k, n, c = _union_args(kinds, counts)
    out = ctypes.POINTER(ctypes.c_uint8)()
    ln = ctypes.c_size_t()
    if lib.oracle_mixed_proof_io(k, n, nu, c, bundle, len(bundle), ctypes.byref(out), ctypes.byref(ln)) != 0:
        raise RuntimeError(lib.oracle_last_error().decode())
    try:
        return ctypes.string_at(out, ln.value)
    finally:
        lib.oracle_free(out)


def verify_union(kinds, nu: int, counts, bundle: bytes, domain: bytes) -> tuple:
    """The restated verifier on a union bundle (registry in slot order, declared counts).
    Returns (accepted, reason)."""
    lib = load()
    k, n, c = _union_args(kinds, counts)
    reason = ctypes.create_string_buffer(256)
    rc = lib.oracle_verify_union(k, n, nu, c, bundle, len(bundle), domain, len(domain), reason, 256)
    if rc == 2:
        raise RuntimeError(reason.value.decode())
    return rc == 0, reason.value.decode()
