"""The oracle's verifier (oracle/verifier.h) on CPU: it accepts the pinned anchor proofs
(byte-identical to the reference's), accepts a Keccak proof, and rejects tampered bundles,
a wrong transcript domain and swapped claim values."""
import random

import pytest

import oracle
from flock_gb300 import BLAKE3, KECCAK, SHA256, inputs

KINDS = {"blake3": BLAKE3, "sha256": SHA256}


@pytest.fixture(scope="module")
def keccak_bundle():
    recs = inputs.batch(KECCAK, 64, 5)
    return oracle.prove_fast_bytes(KECCAK, recs, b"verifier-test")


@pytest.mark.parametrize("idx", [0, 1])
def test_verifier_accepts_anchor_proofs(anchors, idx):
    entry = anchors["prove_fast"][idx]
    recs = inputs.blake3_fixture(entry["n_blocks"], entry["seed"]) if entry["kind"] == "blake3" else \
        inputs.sha256_batch(entry["n_blocks"], entry["seed"])
    dom = anchors["domain"].encode()
    blob = oracle.prove_fast_bytes(KINDS[entry["kind"]], recs, dom)
    ok, why = oracle.verify(KINDS[entry["kind"]], entry["n_blocks"], blob, dom)
    assert ok, why


def test_verifier_accepts_keccak(keccak_bundle):
    ok, why = oracle.verify(KECCAK, 64, keccak_bundle, b"verifier-test")
    assert ok, why


def test_verifier_rejects_bit_flips(keccak_bundle):
    rng = random.Random(11)
    b = keccak_bundle
    n = 120
    for i in range(n):
        pos = (i * len(b)) // n + rng.randrange(len(b) // n)
        bb = bytearray(b)
        bb[pos] ^= 1 << rng.randrange(8)
        ok, why = oracle.verify(KECCAK, 64, bytes(bb), b"verifier-test")
        assert not ok, f"flip at byte {pos} accepted"


def test_verifier_rejects_wrong_domain_and_swapped_claims(keccak_bundle):
    ok, why = oracle.verify(KECCAK, 64, keccak_bundle, b"verifier-tesT")
    assert not ok
    b = bytearray(keccak_bundle)
    ab, c = bytes(b[-32:-16]), bytes(b[-16:])
    b[-32:-16], b[-16:] = c, ab
    ok, why = oracle.verify(KECCAK, 64, bytes(b), b"verifier-test")
    assert not ok and why.startswith("claims")


def test_verifier_rejects_truncation_and_wrong_statement(keccak_bundle):
    ok, why = oracle.verify(KECCAK, 64, keccak_bundle[:-1], b"verifier-test")
    assert not ok and why.startswith("bundle")
    ok, why = oracle.verify(KECCAK, 128, keccak_bundle, b"verifier-test")
    assert not ok
