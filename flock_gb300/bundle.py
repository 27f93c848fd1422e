"""Proof bundles returned by prove_fast.

Layout (little-endian): u64 proof_len | bincode(R1csProofMergedLigerito) | u64 cap_len |
cap_len x 32-byte Merkle cap | ab_value (16 B) | c_value (16 B).

``digest()`` is SHA-256 over proof || cap || ab_value || c_value, the byte-identity
digest of crates/flock-prover/tests/union_m6_fixtures.rs:166-180.
"""
from __future__ import annotations

import hashlib
import struct
from dataclasses import dataclass
from typing import List


@dataclass(frozen=True)
class ProofBundle:
    proof: bytes
    cap: List[bytes]
    ab_value: bytes
    c_value: bytes

    @classmethod
    def parse(cls, blob: bytes) -> "ProofBundle":
        (plen,) = struct.unpack_from("<Q", blob, 0)
        o = 8
        proof = bytes(blob[o:o + plen])
        o += plen
        (clen,) = struct.unpack_from("<Q", blob, o)
        o += 8
        cap = [bytes(blob[o + 32 * i:o + 32 * i + 32]) for i in range(clen)]
        o += 32 * clen
        ab, c = bytes(blob[o:o + 16]), bytes(blob[o + 16:o + 32])
        if o + 32 != len(blob):
            raise ValueError("malformed proof bundle")
        return cls(proof, cap, ab, c)

    def to_bytes(self) -> bytes:
        return (struct.pack("<Q", len(self.proof)) + self.proof + struct.pack("<Q", len(self.cap))
                + b"".join(self.cap) + self.ab_value + self.c_value)

    def to_proof_io(self, hash_kind: int, n_blocks: int) -> bytes:
        """The reference's proof file / wire bytes ("FLOCK" v21, flavor R1cs:
        bincode(Commitment { cap, params }, proof); crates/flock-prover/src/proof_io.rs:238-252)
        for the setup of (hash_kind, n_blocks). Host-only conversion in the C library."""
        import ctypes

        from . import _native

        lib = _native.load()
        blob = self.to_bytes()
        out = ctypes.POINTER(ctypes.c_uint8)()
        n = ctypes.c_size_t()
        _native.check(lib.flock_gb300_proof_io(hash_kind, n_blocks, blob, len(blob), ctypes.byref(out), ctypes.byref(n)))
        try:
            return ctypes.string_at(out, n.value)
        finally:
            lib.flock_gb300_free(out)

    def digest(self) -> bytes:
        h = hashlib.sha256()
        h.update(self.proof)
        for x in self.cap:
            h.update(x)
        h.update(self.ab_value)
        h.update(self.c_value)
        return h.digest()
