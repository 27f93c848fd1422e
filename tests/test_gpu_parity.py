"""GPU prove_fast (through the C ABI) against the oracle and the pinned digests."""
import pytest

import oracle
import flock_gb300
from flock_gb300 import BLAKE3, KECCAK, SHA256, FlockError, ProofBundle, inputs

pytestmark = pytest.mark.gpu
DOMAIN = b"flock-m6-fixture-v0"


@pytest.fixture(scope="module")
def setups():
    cache = {}

    def get(kind, n):
        if (kind, n) not in cache:
            cache[(kind, n)] = flock_gb300.SETUPS[kind](n)
        return cache[(kind, n)]

    yield get
    for s in cache.values():
        s.close()


def test_blake3_anchor(setups, anchors):
    e = anchors["prove_fast"][0]
    inp = inputs.blake3_fixture(e["n_blocks"], e["seed"])
    blob = setups(BLAKE3, e["n_blocks"]).prove_fast_bytes(inp, DOMAIN)
    assert ProofBundle.parse(blob).digest().hex() == e["digest"]
    assert blob == oracle.prove_fast_bytes(BLAKE3, inp, DOMAIN)


def test_sha256_anchor(setups, anchors):
    e = anchors["prove_fast"][1]
    inp = inputs.sha256_batch(e["n_blocks"], e["seed"])
    blob = setups(SHA256, e["n_blocks"]).prove_fast_bytes(inp, DOMAIN)
    assert ProofBundle.parse(blob).digest().hex() == e["digest"]
    assert blob == oracle.prove_fast_bytes(SHA256, inp, DOMAIN)


@pytest.mark.parametrize("kind,n,seed", [
    (KECCAK, 64, 11), (KECCAK, 128, 12),
    (BLAKE3, 512, 21), (BLAKE3, 1024, 22),
    (SHA256, 256, 31), (SHA256, 512, 32),
])
def test_random_batches_match_oracle(setups, kind, n, seed):
    inp = inputs.batch(kind, n, seed)
    dom = b"flock-gb300-parity"
    assert setups(kind, n).prove_fast_bytes(inp, dom) == oracle.prove_fast_bytes(kind, inp, dom)


def test_two_calls_in_a_row_are_identical(setups):
    s = setups(SHA256, 256)
    a = inputs.batch(SHA256, 256, 5)
    b = inputs.batch(SHA256, 256, 6)
    pa = s.prove_fast_bytes(a, b"x")
    pb = s.prove_fast_bytes(b, b"x")
    assert pa != pb
    assert s.prove_fast_bytes(a, b"x") == pa
    assert s.prove_fast_bytes(b, b"x") == pb


def test_domain_separation_and_empty_domain(setups):
    s = setups(BLAKE3, 256)
    a = inputs.batch(BLAKE3, 256, 1)
    assert s.prove_fast_bytes(a, b"") != s.prove_fast_bytes(a, b"d")
    assert s.prove_fast_bytes(a, b"") == oracle.prove_fast_bytes(BLAKE3, a, b"")


def test_wrong_input_count_is_rejected(setups):
    s = setups(BLAKE3, 256)
    with pytest.raises(FlockError) as ei:
        s.prove_fast_bytes(inputs.batch(BLAKE3, 128, 1), b"d")
    assert ei.value.code == flock_gb300._native.EINVAL
