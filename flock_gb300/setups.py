"""Host mirror of the reference's prove_fast interface.

    Blake3Setup(n).prove_fast(inputs, domain)       blake3.rs:1589-1652, 1669-1685
    Sha256HybridSetup(n).prove_fast(inputs, domain) sha2.rs:1185-1268, 1289-1306
    KeccakSetup(n).prove_fast(inputs, domain)       keccak.rs:847-909, 922-938

(crates/flock-prover/src/r1cs_hashes/). The reference passes a challenger built as
``FsChallenger::new(domain)``; here the domain bytes are passed and the transcript is
built inside the library. Inputs are numpy structured arrays (see ``*_DTYPE``) or raw
bytes of ``n`` packed records. Like the reference's ``assert_eq!(blocks.len(),
self.n_blocks)``, a wrong count is an error (``FlockError`` with code EINVAL).
"""
from __future__ import annotations

import ctypes
from typing import Union

import numpy as np

from . import _native
from .bundle import ProofBundle

#: Compression {cv[8], m[16], counter, block_len, flags} (blake3.rs:1232)
BLAKE3_DTYPE = np.dtype([("cv", "<u4", 8), ("m", "<u4", 16), ("counter", "<u8"),
                         ("block_len", "<u4"), ("flags", "<u4")])
#: {h[8], w[16]} (sha2.rs:1332)
SHA256_DTYPE = np.dtype([("h", "<u4", 8), ("w", "<u4", 16)])
#: 25 lanes, bit j of lane i = state bit 64 i + j
KECCAK_DTYPE = np.dtype([("lanes", "<u8", 25)])

Inputs = Union[bytes, bytearray, memoryview, np.ndarray]


class _Setup:
    KIND = -1
    DTYPE: np.dtype = None

    def __init__(self, n_blocks: int):
        lib = _native.load()
        h = ctypes.c_void_p()
        _native.check(lib.flock_gb300_setup_new(self.KIND, int(n_blocks), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.n_blocks = int(n_blocks)
        m, lanes, kc = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        dig = ctypes.create_string_buffer(32)
        _native.check(lib.flock_gb300_setup_info(h, ctypes.byref(m), ctypes.byref(lanes), ctypes.byref(kc), dig))
        self.m = m.value
        self.lanes = lanes.value
        self.log_code_len = kc.value
        self.registry_digest = dig.raw

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.flock_gb300_setup_free(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _buffer(self, inputs: Inputs):
        if isinstance(inputs, np.ndarray):
            if inputs.dtype != self.DTYPE:
                raise TypeError(f"inputs must have dtype {self.DTYPE}")
            arr = np.ascontiguousarray(inputs)
            n = arr.shape[0]
            return arr, arr.ctypes.data, n
        b = bytes(inputs)
        rec = self.DTYPE.itemsize
        if len(b) % rec:
            raise ValueError(f"input bytes are not a whole number of {rec}-byte records")
        buf = ctypes.create_string_buffer(b, len(b))
        return buf, ctypes.addressof(buf), len(b) // rec

    def prove_fast_bytes(self, inputs: Inputs, domain: bytes) -> bytes:
        """prove_fast; returns the raw proof bundle."""
        if self._h is None:
            raise RuntimeError("setup is closed")
        keep, ptr, n = self._buffer(inputs)
        out = ctypes.POINTER(ctypes.c_uint8)()
        out_len = ctypes.c_size_t()
        _native.check(self._lib.flock_gb300_prove_fast(self._h, ptr, n, domain, len(domain),
                                                       ctypes.byref(out), ctypes.byref(out_len)))
        try:
            return ctypes.string_at(out, out_len.value)
        finally:
            self._lib.flock_gb300_free(out)
        del keep

    def prove_fast_device_bytes(self, d_inputs: int, n_inputs: int, domain: bytes) -> bytes:
        """prove_fast from input records already in device memory (raw device pointer)."""
        if self._h is None:
            raise RuntimeError("setup is closed")
        out = ctypes.POINTER(ctypes.c_uint8)()
        out_len = ctypes.c_size_t()
        _native.check(self._lib.flock_gb300_prove_fast_device(self._h, ctypes.c_void_p(d_inputs), n_inputs, domain,
                                                              len(domain), ctypes.byref(out), ctypes.byref(out_len)))
        try:
            return ctypes.string_at(out, out_len.value)
        finally:
            self._lib.flock_gb300_free(out)

    def stream_handle(self) -> int:
        """The cudaStream_t (as an integer) every kernel of this setup runs on."""
        h = ctypes.c_void_p()
        _native.check(self._lib.flock_gb300_setup_stream(self._h, ctypes.byref(h)))
        return h.value or 0

    def set_stage_timing(self, stages=True) -> None:
        """Record CUDA events around stages: True = all, False/None = none, or an
        iterable of stage names."""
        if stages is True:
            mask = 0xFFFFFFFF
        elif not stages:
            mask = 0
        else:
            names = [self._lib.flock_gb300_stage_name(i).decode() for i in range(32)]
            mask = 0
            for s in stages:
                mask |= 1 << names.index(s)
        _native.check(self._lib.flock_gb300_set_stage_timing(self._h, mask))

    def last_stage_ms(self) -> dict:
        """{stage: (device ms, kernel launches)} of the last prove (stage timing enabled)."""
        ms = (ctypes.c_double * 32)()
        ln = (ctypes.c_uint32 * 32)()
        n = self._lib.flock_gb300_last_stage_ms(self._h, ms, ln, 32)
        if n < 0:
            _native.check(n)
        return {self._lib.flock_gb300_stage_name(i).decode(): (ms[i], ln[i]) for i in range(n)}

    def last_transfer_bytes(self) -> tuple:
        h2d, d2h = ctypes.c_uint64(), ctypes.c_uint64()
        _native.check(self._lib.flock_gb300_last_transfer_bytes(self._h, ctypes.byref(h2d), ctypes.byref(d2h)))
        return h2d.value, d2h.value

    def prove_fast(self, inputs: Inputs, domain: bytes) -> ProofBundle:
        return ProofBundle.parse(self.prove_fast_bytes(inputs, domain))

    def last_phase_ms(self) -> dict:
        v = (ctypes.c_double * 8)()
        _native.check(self._lib.flock_gb300_last_phase_ms(self._h, v))
        return dict(zip(("witness", "commit", "zerocheck", "lincheck", "open", "total", "assist", "assist_wait"),
                        list(v)))


class Blake3Setup(_Setup):
    KIND = _native.BLAKE3
    DTYPE = BLAKE3_DTYPE


class Sha256HybridSetup(_Setup):
    KIND = _native.SHA256
    DTYPE = SHA256_DTYPE


class KeccakSetup(_Setup):
    KIND = _native.KECCAK
    DTYPE = KECCAK_DTYPE


SETUPS = {_native.BLAKE3: Blake3Setup, _native.SHA256: Sha256HybridSetup, _native.KECCAK: KeccakSetup}


class UnionSetup:
    """Mixed multi-type union proofs: ``UnionSetup(types, nu).prove(counts, records, domain)``
    mirrors ``prover::prove_fast_ligerito_union(&UnionInstance::new(&Registry::new(types,
    nu), counts), ...)`` (crates/flock-prover/src/prover.rs:587-620). ``slot_kinds`` is the
    registry's slot order (k_log descending); ``counts`` and ``records`` follow it, each
    count at most ``2**nu`` (zero allowed)."""

    def __init__(self, types, nu: int):
        lib = _native.load()
        n = len(types)
        kinds = (ctypes.c_int * n)(*types)
        order = (ctypes.c_int * n)()
        h = ctypes.c_void_p()
        _native.check(lib.flock_gb300_union_setup_new(kinds, n, nu, ctypes.byref(h), order))
        self._h, self._lib, self.nu = h, lib, nu
        self.slot_kinds = list(order)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.flock_gb300_union_setup_free(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _counts(self, counts):
        if len(counts) != len(self.slot_kinds):
            raise ValueError("one count per registry slot")
        return (ctypes.c_uint64 * len(counts))(*[int(c) for c in counts])

    def prove_bytes(self, counts, records, domain: bytes) -> bytes:
        """The union proof bundle (the prove_fast bundle format)."""
        if self._h is None:
            raise RuntimeError("setup is closed")
        arrs = []
        for kind, c, r in zip(self.slot_kinds, counts, records):
            a = np.ascontiguousarray(r)
            if a.dtype != SETUPS[kind].DTYPE or a.shape[0] != int(c):
                raise TypeError(f"slot records must be {int(c)} records of dtype {SETUPS[kind].DTYPE}")
            arrs.append(a)
        ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data if a.size else None for a in arrs])
        out = ctypes.POINTER(ctypes.c_uint8)()
        out_len = ctypes.c_size_t()
        _native.check(self._lib.flock_gb300_prove_union(self._h, self._counts(counts), ptrs, domain, len(domain),
                                                        ctypes.byref(out), ctypes.byref(out_len)))
        try:
            return ctypes.string_at(out, out_len.value)
        finally:
            self._lib.flock_gb300_free(out)

    def prove(self, counts, records, domain: bytes) -> ProofBundle:
        return ProofBundle.parse(self.prove_bytes(counts, records, domain))

    def mixed_proof_io(self, counts, bundle: bytes) -> bytes:
        """MixedProofBundleLigerito::to_bytes of a bundle of this registry (built-in tiers)."""
        out = ctypes.POINTER(ctypes.c_uint8)()
        out_len = ctypes.c_size_t()
        _native.check(self._lib.flock_gb300_mixed_proof_io(self._h, self._counts(counts), bundle, len(bundle),
                                                           ctypes.byref(out), ctypes.byref(out_len)))
        try:
            return ctypes.string_at(out, out_len.value)
        finally:
            self._lib.flock_gb300_free(out)
