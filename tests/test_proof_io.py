"""The reference proof-file format of a bundle (flock_gb300_proof_io; host-only, so this
runs without a GPU): "FLOCK" | 21 | flavor 2 | bincode(Commitment { cap, PcsParams }, proof)."""
import struct

import pytest

import oracle
from flock_gb300 import KECCAK, SHA256, ProofBundle, inputs


@pytest.mark.parametrize("kind,n", [(KECCAK, 64), (SHA256, 128)])
def test_proof_io_layout(kind, n):
    blob = oracle.prove_fast_bytes(kind, inputs.batch(kind, n, 3), b"proof-io")
    b = ProofBundle.parse(blob)
    io = b.to_proof_io(kind, n)
    assert io[:5] == b"FLOCK" and io[5] == 21 and io[6] == 2
    o = 7
    (ncap,) = struct.unpack_from("<Q", io, o)
    o += 8
    assert [io[o + 32 * i:o + 32 * i + 32] for i in range(ncap)] == b.cap
    o += 32 * ncap
    m, rate, log_batch = struct.unpack_from("<QQQ", io, o)
    o += 24
    (profile,) = struct.unpack_from("<I", io, o)
    o += 4
    tag = io[o]
    o += 1
    lanes = None
    if tag == 1:
        (lanes,) = struct.unpack_from("<Q", io, o)
        o += 8
    (merkle,) = struct.unpack_from("<I", io, o)
    o += 4
    assert rate == 1 and profile == 0 and merkle == 0 and tag in (0, 1)
    assert lanes is None or 1 <= lanes < (1 << log_batch)
    assert m >= 7 + log_batch
    assert io[o:] == b.proof


def test_proof_io_rejects_malformed_bundles():
    import flock_gb300

    blob = oracle.prove_fast_bytes(KECCAK, inputs.batch(KECCAK, 64, 3), b"proof-io")
    with pytest.raises(flock_gb300.FlockError):
        ProofBundle(blob[8:20], [], b"\0" * 16, b"\0" * 16).to_proof_io(KECCAK, 100)
