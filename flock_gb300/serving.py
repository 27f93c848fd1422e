"""Batched and served proving (flock_gb300_prove_batch / flock_gb300_server_*).

Independent proofs run concurrently on the device, each on its own stream and buffers,
admitted against a device-memory budget; every bundle is byte-identical to the one a
single ``Setup.prove_fast`` call returns for the same request.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np

from . import _native
from .bundle import ProofBundle
from .setups import SETUPS

GiB = 1 << 30
# Concurrent provers. Two keep one GB300 busy on the mixed-size workload (one proof's host
# round trips and assist overlap the other's kernels); more contend for the device and the
# host cores without adding throughput (measured: 2 -> 1.36x one-at-a-time, 3 -> 1.08x).
DEFAULT_WORKERS = 2


@dataclass
class Outcome:
    bundle: ProofBundle
    latency_ms: float


@dataclass
class RawOutcome:
    """An Outcome whose bundle is left as the wire bytes (no parsing)."""
    bundle_bytes: bytes
    latency_ms: float


def _request(kind: int, recs, domain: bytes, keep: list) -> _native.Request:
    arr = np.ascontiguousarray(recs)
    if arr.dtype != SETUPS[kind].DTYPE:
        raise TypeError(f"inputs for kind {kind} must have dtype {SETUPS[kind].DTYPE}")
    keep.append(arr)
    keep.append(domain)
    return _native.Request(kind, arr.shape[0], arr.ctypes.data, domain, len(domain))


def _take(lib, res: _native.Result, raw: bool = False):
    try:
        blob = ctypes.string_at(res.bundle, res.bundle_len)
    finally:
        lib.flock_gb300_free(res.bundle)
    if raw:
        return RawOutcome(blob, res.latency_ms)
    return Outcome(ProofBundle.parse(blob), res.latency_ms)


def _run_batch(call, requests, raw: bool):
    lib = _native.load()
    keep: list = []
    n = len(requests)
    reqs = (_native.Request * n)(*[_request(k, r, d, keep) for k, r, d in requests])
    results = (_native.Result * n)()
    rc = call(lib, reqs, n, results)
    outs = [_take(lib, results[i], raw) if results[i].status == _native.OK else None for i in range(n)]
    _native.check(rc)
    return outs


def estimate_device_bytes(kind: int, n_blocks: int) -> int:
    """Device bytes one prover of this shape holds (the admission figure of the batch and
    serving entry points)."""
    lib = _native.load()
    out = ctypes.c_uint64()
    _native.check(lib.flock_gb300_estimate_device_bytes(kind, n_blocks, ctypes.byref(out)))
    return out.value


def prove_batch(requests: Sequence[Tuple[int, np.ndarray, bytes]], workers: int = DEFAULT_WORKERS,
                hbm_budget_bytes: int = 64 * GiB, raw: bool = False) -> List[Outcome]:
    """Proves [(kind, records, domain), ...] concurrently; results in request order. The
    provers are created for this call and released at its end (ProofServer.prove_batch
    keeps them)."""
    return _run_batch(lambda lib, reqs, n, res: lib.flock_gb300_prove_batch(reqs, n, workers, hbm_budget_bytes, res),
                      requests, raw)


class ProofServer:
    """submit() returns a ticket at once; result(ticket) waits for that proof."""

    def __init__(self, hbm_budget_bytes: int = 64 * GiB, workers: int = DEFAULT_WORKERS):
        self._lib = _native.load()
        h = ctypes.c_void_p()
        _native.check(self._lib.flock_gb300_server_new(hbm_budget_bytes, workers, ctypes.byref(h)))
        self._h = h

    def submit(self, kind: int, records: np.ndarray, domain: bytes) -> int:
        keep: list = []
        req = _request(kind, records, domain, keep)
        t = ctypes.c_uint64()
        _native.check(self._lib.flock_gb300_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        return t.value

    def result(self, ticket: int, wait_ms: int = -1, raw: bool = False):
        """The Outcome of a finished ticket, or None while it runs (wait_ms >= 0)."""
        res = _native.Result()
        rc = self._lib.flock_gb300_server_poll(self._h, ticket, wait_ms, ctypes.byref(res))
        if rc == _native.PENDING:
            return None
        _native.check(rc)
        if res.status != _native.OK:
            raise _native.FlockError(res.status, self._lib.flock_gb300_last_error().decode())
        return _take(self._lib, res, raw)

    def prove_batch(self, requests: Sequence[Tuple[int, np.ndarray, bytes]], raw: bool = False) -> List[Outcome]:
        """prove_batch on this server's cached provers."""
        return _run_batch(lambda lib, reqs, n, res: lib.flock_gb300_server_prove_batch(self._h, reqs, n, res),
                          requests, raw)

    def close(self) -> None:
        if self._h:
            self._lib.flock_gb300_server_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
