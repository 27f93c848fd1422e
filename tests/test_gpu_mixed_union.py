"""Mixed multi-type union proofs on the GPU (flock_gb300_prove_union): the reference's four
pinned BLAKE3 + SHA-256 nu = 10 digests through the proof-IO wire bytes
(crates/flock-prover/tests/union_m6_fixtures.rs:196-281), byte identity with the oracle,
and unions with Keccak-f slots and partial counts, whose proofs the restated verifier
accepts."""
import hashlib

import pytest

import flock_gb300
import oracle
from flock_gb300 import BLAKE3, KECCAK, SHA256, FlockError, ProofBundle, inputs

pytestmark = pytest.mark.gpu


def mixed_digest(bundle: bytes, wire: bytes) -> str:
    pb = ProofBundle.parse(bundle)
    h = hashlib.sha256(wire)
    h.update(pb.ab_value)
    h.update(pb.c_value)
    return h.hexdigest()


@pytest.fixture(scope="module")
def b3sha2_nu10(anchors):
    with flock_gb300.UnionSetup([BLAKE3, SHA256], anchors["mixed"]["nu"]) as u:
        yield u


@pytest.mark.parametrize("idx", [0, 1, 2, 3])
def test_gpu_reproduces_mixed_union_digest(anchors, b3sha2_nu10, idx):
    mx = anchors["mixed"]
    fx = mx["fixtures"][idx]
    n_sha2, n_b3 = fx["counts"]
    sha, b3 = inputs.mixed_fixture(n_sha2, n_b3, mx["seed_base"] ^ (n_sha2 << 16) ^ n_b3)
    u = b3sha2_nu10
    assert u.slot_kinds == [SHA256, BLAKE3]
    dom = anchors["domain"].encode()
    bundle = u.prove_bytes([n_sha2, n_b3], [sha, b3], dom)
    wire = u.mixed_proof_io([n_sha2, n_b3], bundle)
    assert mixed_digest(bundle, wire) == fx["digest"], fx["name"]
    assert bundle == oracle.prove_union_bytes([SHA256, BLAKE3], mx["nu"], [n_sha2, n_b3], [sha, b3], dom)
    # the same counts again (cached prover) and fresh inputs stay identical to the oracle
    again = u.prove_bytes([n_sha2, n_b3], [sha, b3], dom)
    assert again == bundle


@pytest.mark.parametrize("types,nu,counts", [
    ([KECCAK, SHA256, BLAKE3], 6, [64, 23, 5]),
    ([BLAKE3, KECCAK], 8, [0, 200]),
    ([SHA256, KECCAK], 7, [128, 128]),
])
def test_union_with_keccak_matches_oracle(types, nu, counts):
    with flock_gb300.UnionSetup(types, nu) as u:
        recs = [inputs.batch(k, c, 900 + i) if c else inputs.batch(k, 8, 1)[:0]
                for i, (k, c) in enumerate(zip(u.slot_kinds, counts))]
        dom = b"gpu-union-%d" % nu
        bundle = u.prove_bytes(counts, recs, dom)
        assert bundle == oracle.prove_union_bytes(u.slot_kinds, nu, counts, recs, dom)
        ok, why = oracle.verify_union(u.slot_kinds, nu, counts, bundle, dom)
        assert ok, why
        with pytest.raises(FlockError):
            u.mixed_proof_io(counts, bundle)  # not a built-in tier


def test_union_rejects_bad_arguments():
    with pytest.raises(FlockError):
        flock_gb300.UnionSetup([BLAKE3, BLAKE3], 6)
    with flock_gb300.UnionSetup([BLAKE3, SHA256], 6) as u:
        with pytest.raises(FlockError):
            u.prove_bytes([70, 0], [inputs.batch(SHA256, 70, 1), inputs.batch(BLAKE3, 8, 1)[:0]], b"x")
