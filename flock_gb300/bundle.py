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

    def digest(self) -> bytes:
        h = hashlib.sha256()
        h.update(self.proof)
        for x in self.cap:
            h.update(x)
        h.update(self.ab_value)
        h.update(self.c_value)
        return h.digest()
