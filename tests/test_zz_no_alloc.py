"""flock_gb300_commit_cap_noalloc (static scratch, no device allocation by the library)
against the cap in the bundle of the allocating entry point flock_gb300_prove_fast, for
all three hashes up to the largest accepted batch of each (codewords of 2^13 rows:
2^11 BLAKE3, 2^10 SHA-256, 2^9 Keccak-f), and the rejection of the next size up.
Collected last (file name) so it also runs after every other test in one process."""
import ctypes

import numpy as np
import pytest

import flock_gb300
from flock_gb300 import BLAKE3, KECCAK, SHA256, inputs

pytestmark = pytest.mark.gpu


def noalloc_cap(kind, recs):
    import torch

    lib = flock_gb300.load()
    dev = torch.from_numpy(np.frombuffer(recs.tobytes(), dtype=np.uint8).copy()).to("cuda:0")
    out = ctypes.create_string_buffer(1 << 16)
    n = ctypes.c_size_t()
    rc = lib.flock_gb300_commit_cap_noalloc(kind, ctypes.c_void_p(dev.data_ptr()), len(recs), out, len(out),
                                             ctypes.byref(n), None)
    torch.cuda.synchronize()
    if rc != 0:
        raise flock_gb300.FlockError(rc, lib.flock_gb300_last_error().decode())
    return [out.raw[i:i + 32] for i in range(0, n.value, 32)]


@pytest.mark.parametrize("kind,n,seed", [(BLAKE3, 256, 3), (SHA256, 128, 4), (BLAKE3, 2048, 5), (SHA256, 1024, 6),
                                         (KECCAK, 64, 7), (KECCAK, 512, 8)])
def test_noalloc_cap_matches_prove_fast_twice(kind, n, seed):
    recs = inputs.batch(kind, n, seed)
    with flock_gb300.SETUPS[kind](n) as setup:
        bundle = setup.prove_fast(recs, b"noalloc")
    first = noalloc_cap(kind, recs)
    second = noalloc_cap(kind, recs)
    assert first == bundle.cap
    assert second == bundle.cap


@pytest.mark.parametrize("kind,n", [(BLAKE3, 4096), (SHA256, 2048), (KECCAK, 1024)])
def test_noalloc_rejects_batches_beyond_the_static_scratch(kind, n):
    with pytest.raises(flock_gb300.FlockError) as ei:
        noalloc_cap(kind, inputs.batch(kind, n, 1))
    assert ei.value.code == flock_gb300._native.EINVAL
    assert "static scratch" in str(ei.value)
