"""The C-ABI library loads and exports every declared symbol; host-side helpers (CPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

import flock_gb300
from flock_gb300 import _native, inputs
from flock_gb300.bundle import ProofBundle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "flock_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(flock_gb300_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = flock_gb300.load()
    names = declared_functions()
    assert len(names) >= 9
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(_native.EXPORTS) == names


def test_record_sizes_match_dtypes():
    lib = flock_gb300.load()
    assert lib.flock_gb300_input_record_bytes(0) == flock_gb300.BLAKE3_DTYPE.itemsize == 112
    assert lib.flock_gb300_input_record_bytes(1) == flock_gb300.SHA256_DTYPE.itemsize == 96
    assert lib.flock_gb300_input_record_bytes(2) == flock_gb300.KECCAK_DTYPE.itemsize == 200
    assert lib.flock_gb300_input_record_bytes(7) == 0


def test_setup_rejects_bad_arguments_without_touching_the_gpu():
    lib = flock_gb300.load()
    h = ctypes.c_void_p()
    assert lib.flock_gb300_setup_new(5, 256, ctypes.byref(h)) == _native.EINVAL
    assert b"hash kind" in lib.flock_gb300_last_error()
    assert lib.flock_gb300_setup_new(0, 100, ctypes.byref(h)) == _native.EINVAL
    assert lib.flock_gb300_setup_new(0, 4, ctypes.byref(h)) == _native.EINVAL
    assert lib.flock_gb300_prove_fast(None, None, 0, None, 0, None, None) == _native.EINVAL


def test_bundle_roundtrip():
    b = ProofBundle(b"\x01\x02\x03", [bytes(range(32)), bytes(32)], bytes(16), bytes(range(16)))
    assert ProofBundle.parse(b.to_bytes()) == b
    with pytest.raises(ValueError):
        ProofBundle.parse(b.to_bytes() + b"\x00")


def test_batch_generators_shapes():
    assert inputs.blake3_batch(8, 1)["counter"].tolist() == list(range(8))
    assert (inputs.blake3_batch(8, 1)["flags"] == 0).all()
    k = inputs.keccak_batch(4, 3)
    assert k.dtype == flock_gb300.KECCAK_DTYPE and k.shape == (4,)
    assert not np.array_equal(inputs.sha256_batch(4, 1), inputs.sha256_batch(4, 2))
