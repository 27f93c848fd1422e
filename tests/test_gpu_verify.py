"""Proofs made by the CUDA path, from the parity sizes up to the benchmark workloads
(BLAKE3 2^12, SHA-256 2^16, Keccak-f 2^18), are accepted by the oracle's verifier,
which replays the transcript and checks every sumcheck, opening and Merkle relation."""
import pytest

import flock_gb300
import oracle
from flock_gb300 import BLAKE3, KECCAK, SHA256, inputs

pytestmark = pytest.mark.gpu

CASES = [(BLAKE3, 1 << 8), (SHA256, 1 << 7), (KECCAK, 1 << 6), (BLAKE3, 1 << 12), (SHA256, 1 << 14),
         (KECCAK, 1 << 13), (SHA256, 1 << 16), (KECCAK, 1 << 18)]


@pytest.mark.parametrize("kind,n", CASES)
def test_gpu_proof_is_accepted(kind, n):
    recs = inputs.batch(kind, n, 77)
    dom = b"gpu-verify-%d-%d" % (kind, n)
    with flock_gb300.SETUPS[kind](n) as s:
        blob = s.prove_fast_bytes(recs, dom)
    ok, why = oracle.verify(kind, n, blob, dom)
    assert ok, why
    bad = bytearray(blob)
    bad[len(bad) // 3] ^= 0x10
    assert not oracle.verify(kind, n, bytes(bad), dom)[0]
