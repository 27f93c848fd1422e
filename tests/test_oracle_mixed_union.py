"""The oracle's mixed multi-type union proofs against the reference's four pinned digests
(crates/flock-prover/tests/union_m6_fixtures.rs:196-281): a BLAKE3 + SHA-256 registry at
nu = 10 with full, partial, equal-small and zero-count utilisation, digested over the
proof-IO wire bytes (MixedProofBundleLigerito::to_bytes) and the two claim values."""
import hashlib

import pytest

import oracle
from flock_gb300 import BLAKE3, SHA256, ProofBundle, inputs


def mixed_digest(bundle: bytes, wire: bytes) -> str:
    pb = ProofBundle.parse(bundle)
    h = hashlib.sha256(wire)
    for v in (pb.ab_value, pb.c_value):
        h.update(v)
    return h.hexdigest()


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_oracle_reproduces_mixed_union_digest(anchors, idx):
    mx = anchors["mixed"]
    fx = mx["fixtures"][idx]
    n_sha2, n_b3 = fx["counts"]
    seed = mx["seed_base"] ^ (n_sha2 << 16) ^ n_b3
    sha, b3 = inputs.mixed_fixture(n_sha2, n_b3, seed)
    kinds = [SHA256, BLAKE3]  # slot order: k_log descending
    dom = anchors["domain"].encode()
    bundle = oracle.prove_union_bytes(kinds, mx["nu"], [n_sha2, n_b3], [sha, b3], dom)
    wire = oracle.mixed_proof_io(kinds, mx["nu"], [n_sha2, n_b3], bundle)
    assert wire[:7] == b"FLOCK\x15\x04"
    assert mixed_digest(bundle, wire) == fx["digest"], fx["name"]
