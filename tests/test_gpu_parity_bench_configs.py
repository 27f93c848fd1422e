"""Byte identity of GPU proofs with the oracle at the benchmark workloads.

The GPU bundle (proof bytes, Merkle cap and both claims) must equal the oracle's for
  * BLAKE3 2^12 (m = 26, counter = index, flags 0),
  * SHA-256 2^16 (m = 31),
  * Keccak-f[1600] 2^15 (m = 31),
each of which runs its own Ligerito level ladder. The lockstep harness
(tests/native/lockstep.cu) is also run at BLAKE3 2^12: it drives the CUDA backend and the
oracle side by side through one prove and names the first step whose returned values
differ, so a divergence points at its kernel.
"""
import os
import subprocess

import pytest

import flock_gb300
import oracle
from flock_gb300 import BLAKE3, KECCAK, SHA256, inputs

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DOMAIN = b"flock-gb300-bench-parity"


@pytest.mark.parametrize("kind,n,seed", [
    (BLAKE3, 1 << 12, 0x5EED),
    (SHA256, 1 << 16, 0x5EED),
    (KECCAK, 1 << 15, 0x5EED),
])
def test_benchmark_workload_bundle_matches_oracle(kind, n, seed):
    recs = inputs.batch(kind, n, seed)
    with flock_gb300.SETUPS[kind](n) as s:
        gpu = s.prove_fast_bytes(recs, DOMAIN)
        again = s.prove_fast_bytes(recs, DOMAIN)
    ref = oracle.prove_fast_bytes(kind, recs, DOMAIN)
    assert gpu == again
    assert len(gpu) == len(ref)
    if gpu != ref:
        first = next(i for i in range(len(gpu)) if gpu[i] != ref[i])
        pytest.fail(f"GPU bundle differs from the oracle's at byte {first} of {len(gpu)}")


def _build_lockstep() -> str:
    import __graft_entry__ as g

    out_dir = os.path.join(ROOT, "tests", "native", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "lockstep")
    src = os.path.join(ROOT, "tests", "native", "lockstep.cu")
    objs = [os.path.join(g.OBJ_DIR, f)
            for f in ("witness.o", "commit.o", "sumcheck.o", "rounds.o", "backend.o", "host_accel.o")]
    deps = [src] + objs + g._headers() + [os.path.join(ROOT, "oracle", "cpu_backend.h")]
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(p) for p in deps):
        g._run([g._nvcc(), *g.NVCC_FLAGS, src, *objs, "-o", exe, "-lpthread"])
    return exe


def test_lockstep_blake3_4096():
    exe = _build_lockstep()
    r = subprocess.run([exe, str(BLAKE3), str(1 << 12), "0x5EED"], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=900)
    assert r.returncode == 0 and "LOCKSTEP OK" in r.stdout, r.stdout[-3000:]
