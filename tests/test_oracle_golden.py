"""The oracle against the reference's own pinned vectors (CPU)."""
import ctypes

import pytest

import oracle
from flock_gb300 import BLAKE3, SHA256, ProofBundle, inputs

KINDS = {"blake3": BLAKE3, "sha256": SHA256}


def fixture_inputs(entry):
    if entry["kind"] == "blake3":
        return inputs.blake3_fixture(entry["n_blocks"], entry["seed"])
    return inputs.sha256_batch(entry["n_blocks"], entry["seed"])


@pytest.mark.parametrize("idx", [0, 1])
def test_oracle_reproduces_anchor_digest(anchors, idx):
    entry = anchors["prove_fast"][idx]
    blob = oracle.prove_fast_bytes(KINDS[entry["kind"]], fixture_inputs(entry), anchors["domain"].encode())
    assert ProofBundle.parse(blob).digest().hex() == entry["digest"]


@pytest.mark.parametrize("which", [0, 1])
def test_registry_digest_kats(anchors, which):
    lib = oracle.load()
    buf = ctypes.create_string_buffer(32)
    lib.oracle_registry_digest_kat.argtypes = [ctypes.c_int, ctypes.c_char_p]
    assert lib.oracle_registry_digest_kat(which, buf) == 0
    assert buf.raw.hex() == anchors["registry"][which]["digest"]


def test_fixture_generator_is_splitmix64():
    # first draws of SplitMix64 from seed 0: the published reference sequence
    # 0xe220a8397b1dcdaf, 0x6e789e6aa1b965f4 (low 32 bits kept)
    assert list(inputs.splitmix_u32(0, 2)) == [0x7B1DCDAF, 0xA1B965F4]


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("seed", [1, 2])
def test_block_r1cs_is_satisfied(kind, seed):
    """a = A z, b = B z (materialised matrices, or the Keccak walker's transpose
    identity) and a AND b = z on a seeded block of every hash encoder."""
    lib = oracle.load()
    out = (ctypes.c_uint64 * 4)()
    lib.oracle_r1cs_check.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    assert lib.oracle_r1cs_check(kind, seed, out) == 0
    assert list(out)[:3] == [0, 0, 0]
    if kind == 2:
        assert out[3] == 1  # Keccak-f[1600] of the zero state, lane 0 = 0xf1258f7940e1dde7
