"""flock_gb300 — GB300-native prove_fast for Flock's hash-batch R1CS proofs.

The compute path is the in-tree CUDA library ``_lib/libflock_gb300.so`` (sm_103a); this
package is the host-side mirror of the reference's Setup / prove_fast interface.
"""
from ._native import BLAKE3, KECCAK, SHA256, FlockError, NativeLibraryError, load
from .bundle import ProofBundle
from .setups import (BLAKE3_DTYPE, KECCAK_DTYPE, SHA256_DTYPE, SETUPS, Blake3Setup, KeccakSetup,
                     Sha256HybridSetup, UnionSetup)
from . import inputs
from .serving import ProofServer, prove_batch

__all__ = [
    "BLAKE3", "SHA256", "KECCAK", "FlockError", "NativeLibraryError", "load", "ProofBundle",
    "Blake3Setup", "Sha256HybridSetup", "KeccakSetup", "SETUPS", "UnionSetup",
    "BLAKE3_DTYPE", "SHA256_DTYPE", "KECCAK_DTYPE", "inputs", "ProofServer", "prove_batch",
]
