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


@pytest.mark.parametrize("idx", [1, 3])
def test_restated_verifier_accepts_union_proofs_and_rejects_tampering(anchors, idx):
    """The restated verifier replays a union bundle: per-slot const-pin challenges with
    their count-derived targets, the per-slot matrix discharge under the slot prefix
    weights, and the general jagged multipoint assist of the compacted stack."""
    mx = anchors["mixed"]
    n_sha2, n_b3 = mx["fixtures"][idx]["counts"]
    sha, b3 = inputs.mixed_fixture(n_sha2, n_b3, mx["seed_base"] ^ (n_sha2 << 16) ^ n_b3)
    kinds, counts, dom = [SHA256, BLAKE3], [n_sha2, n_b3], anchors["domain"].encode()
    bundle = oracle.prove_union_bytes(kinds, mx["nu"], counts, [sha, b3], dom)
    ok, why = oracle.verify_union(kinds, mx["nu"], counts, bundle, dom)
    assert ok, why
    for pos in (100, len(bundle) // 2, len(bundle) - 40):
        bad = bytearray(bundle)
        bad[pos] ^= 0x04
        assert not oracle.verify_union(kinds, mx["nu"], counts, bytes(bad), dom)[0]
    # the same bytes under different declared counts are a different statement
    other = [n_sha2 + 1, n_b3] if n_sha2 < 1024 else [n_sha2, n_b3 - 1]
    assert not oracle.verify_union(kinds, mx["nu"], other, bundle, dom)[0]
