"""Seeded synthetic hash inputs.

``splitmix_u32`` is the SplitMix64 stream the reference's fixtures draw from
(crates/flock-prover/tests/union_m6_fixtures.rs:100-121): state += 0x9E3779B97F4A7C15,
then the standard mix; each draw keeps the low 32 bits.
"""
from __future__ import annotations

import numpy as np

from .setups import BLAKE3_DTYPE, KECCAK_DTYPE, SHA256_DTYPE

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix_u32(seed: int, n: int) -> np.ndarray:
    """n successive 32-bit SplitMix64 outputs from `seed` (vectorised)."""
    with np.errstate(over="ignore"):
        k = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def blake3_fixture(n: int, seed: int, flags: int = 11) -> np.ndarray:
    """cv[8], m[16], counter = (hi << 32) | lo from two more draws, block_len 64
    (the union_m6_fixtures.rs:100-121 generator)."""
    d = splitmix_u32(seed, 26 * n).reshape(n, 26)
    out = np.zeros(n, dtype=BLAKE3_DTYPE)
    out["cv"] = d[:, :8]
    out["m"] = d[:, 8:24]
    out["counter"] = (d[:, 24].astype(np.uint64) << np.uint64(32)) | d[:, 25].astype(np.uint64)
    out["block_len"] = 64
    out["flags"] = flags
    return out


def blake3_batch(n: int, seed: int) -> np.ndarray:
    """Benchmark batch: cv[8], m[16] uniform from the seed, counter = index, block_len 64, flags 0."""
    d = splitmix_u32(seed, 24 * n).reshape(n, 24)
    out = np.zeros(n, dtype=BLAKE3_DTYPE)
    out["cv"] = d[:, :8]
    out["m"] = d[:, 8:]
    out["counter"] = np.arange(n, dtype=np.uint64)
    out["block_len"] = 64
    out["flags"] = 0
    return out


def sha256_batch(n: int, seed: int) -> np.ndarray:
    """h[8], w[16] uniform from the seed (also the SHA-256 fixture generator)."""
    d = splitmix_u32(seed, 24 * n).reshape(n, 24)
    out = np.zeros(n, dtype=SHA256_DTYPE)
    out["h"] = d[:, :8]
    out["w"] = d[:, 8:]
    return out


def keccak_batch(n: int, seed: int) -> np.ndarray:
    """25 uniform u64 lanes per state (two draws per lane, high word first)."""
    d = splitmix_u32(seed, 50 * n).reshape(n, 25, 2).astype(np.uint64)
    out = np.zeros(n, dtype=KECCAK_DTYPE)
    out["lanes"] = (d[:, :, 0] << np.uint64(32)) | d[:, :, 1]
    return out


def _blake3_from_draws(d: np.ndarray, flags: int) -> np.ndarray:
    n = d.shape[0]
    out = np.zeros(n, dtype=BLAKE3_DTYPE)
    out["cv"] = d[:, :8]
    out["m"] = d[:, 8:24]
    out["counter"] = (d[:, 24].astype(np.uint64) << np.uint64(32)) | d[:, 25].astype(np.uint64)
    out["block_len"] = 64
    out["flags"] = flags
    return out


def mixed_fixture(n_sha2: int, n_blake3: int, seed: int):
    """One SplitMix64 stream from `seed`: n_sha2 SHA-256 records (h[8], w[16]) first, then
    n_blake3 BLAKE3 records (cv[8], m[16], counter = (hi << 32) | lo, block_len 64,
    flags 11) — the mixed-union fixture generator of union_m6_fixtures.rs:226-268."""
    d = splitmix_u32(seed, 24 * n_sha2 + 26 * n_blake3)
    sha = np.zeros(n_sha2, dtype=SHA256_DTYPE)
    if n_sha2:
        s = d[:24 * n_sha2].reshape(n_sha2, 24)
        sha["h"] = s[:, :8]
        sha["w"] = s[:, 8:]
    b3 = _blake3_from_draws(d[24 * n_sha2:].reshape(n_blake3, 26), 11) if n_blake3 else np.zeros(0, dtype=BLAKE3_DTYPE)
    return sha, b3


def batch(kind: int, n: int, seed: int) -> np.ndarray:
    return (blake3_batch, sha256_batch, keccak_batch)[kind](n, seed)
