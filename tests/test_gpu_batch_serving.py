"""Batched and served proving: every bundle equals the one-call prove_fast bundle for the
same request, alone and in the mix."""
import random

import pytest

import flock_gb300
from flock_gb300 import BLAKE3, KECCAK, SHA256, inputs

pytestmark = pytest.mark.gpu


def single(kind, n, recs, dom):
    with flock_gb300.SETUPS[kind](n) as s:
        return s.prove_fast_bytes(recs, dom)


def mixed_requests(count, seed):
    rng = random.Random(seed)
    reqs = []
    for i in range(count):
        kind = rng.choice([BLAKE3, SHA256, KECCAK])
        lo = {BLAKE3: 8, SHA256: 7, KECCAK: 6}[kind]
        n = 1 << rng.randint(lo, lo + 2)
        reqs.append((kind, inputs.batch(kind, n, 1000 + i), b"mix-%d" % i))
    return reqs


def test_batch_matches_single_proofs():
    reqs = mixed_requests(10, 7)
    outs = flock_gb300.prove_batch(reqs, workers=4)
    for (kind, recs, dom), out in zip(reqs, outs):
        assert out.bundle.to_bytes() == single(kind, len(recs), recs, dom)


def test_batch_under_a_tight_budget_still_matches():
    reqs = mixed_requests(6, 9)
    outs = flock_gb300.prove_batch(reqs, workers=3, hbm_budget_bytes=1 << 30)
    for (kind, recs, dom), out in zip(reqs, outs):
        assert out.bundle.to_bytes() == single(kind, len(recs), recs, dom)


def test_server_results_alone_and_in_the_mix():
    reqs = mixed_requests(12, 11)
    with flock_gb300.ProofServer(workers=4) as srv:
        tickets = [srv.submit(k, r, d) for k, r, d in reqs]
        outs = [srv.result(t) for t in tickets]
        # the same request again, alone
        k, r, d = reqs[3]
        alone = srv.result(srv.submit(k, r, d))
    for (kind, recs, dom), out in zip(reqs, outs):
        assert out.bundle.to_bytes() == single(kind, len(recs), recs, dom)
        assert out.latency_ms > 0
    assert alone.bundle.to_bytes() == outs[3].bundle.to_bytes()


def test_server_rejects_bad_requests():
    with flock_gb300.ProofServer(workers=1) as srv:
        with pytest.raises(flock_gb300.FlockError):
            srv.submit(BLAKE3, inputs.batch(BLAKE3, 100, 1), b"x")


def test_batch_of_fresh_provers_at_larger_sizes():
    """Every prover in the batch is new (its first prove allocates and uploads level
    twiddles while other provers run): the uploads must be ordered on the prover's stream."""
    reqs = [(SHA256, inputs.batch(SHA256, 1 << 12, 50 + i), b"fresh-%d" % i) for i in range(2)]
    reqs += [(KECCAK, inputs.batch(KECCAK, 1 << 11, 60 + i), b"fresh-k%d" % i) for i in range(2)]
    reqs += [(BLAKE3, inputs.batch(BLAKE3, 1 << 12, 70 + i), b"fresh-b%d" % i) for i in range(2)]
    outs = flock_gb300.prove_batch(reqs, workers=6)
    for (kind, recs, dom), out in zip(reqs, outs):
        assert out.bundle.to_bytes() == single(kind, len(recs), recs, dom)


def test_server_batches_reuse_cached_provers():
    """Two batches on one server: the second runs on the provers the first left cached,
    alongside a submitted request; every result equals its single prove."""
    reqs = mixed_requests(8, 13)
    with flock_gb300.ProofServer(workers=3) as srv:
        first = srv.prove_batch(reqs, raw=True)
        k, r, d = reqs[0]
        ticket = srv.submit(k, r, d)
        second = srv.prove_batch(reqs[::-1], raw=True)[::-1]
        extra = srv.result(ticket)
    for (kind, recs, dom), a, b in zip(reqs, first, second):
        want = single(kind, len(recs), recs, dom)
        assert a.bundle_bytes == want and b.bundle_bytes == want
    assert extra.bundle.to_bytes() == first[0].bundle_bytes


def test_large_request_is_admitted_while_small_ones_keep_arriving():
    """Aging: a Keccak-f 2^18 request whose prover fits the budget only when no small
    prover is busy is admitted after a few small requests overtake it, although small
    requests keep arriving, and its bundle equals the single prove."""
    from flock_gb300.serving import estimate_device_bytes

    big_kind, big_n = KECCAK, 1 << 18
    small_kind, small_n = SHA256, 1 << 15
    need_big = estimate_device_bytes(big_kind, big_n)
    need_small = estimate_device_bytes(small_kind, small_n)
    big = inputs.batch(big_kind, big_n, 5)
    small = [inputs.batch(small_kind, small_n, 100 + i) for i in range(3)]
    max_small = 60
    submitted, small_tickets = 0, []
    with flock_gb300.ProofServer(hbm_budget_bytes=need_big + need_small // 2, workers=2) as srv:
        for _ in range(4):
            small_tickets.append((submitted, srv.submit(small_kind, small[submitted % 3], b"s%d" % submitted)))
            submitted += 1
        t_big = srv.submit(big_kind, big, b"big")
        out_big = None
        while out_big is None:
            assert submitted < max_small, "the large request was starved by the stream of small ones"
            small_tickets.append((submitted, srv.submit(small_kind, small[submitted % 3], b"s%d" % submitted)))
            submitted += 1
            out_big = srv.result(t_big, wait_ms=10, raw=True)
        outs = [(i, srv.result(t, raw=True)) for i, t in small_tickets[:6]]
    assert out_big.bundle_bytes == single(big_kind, big_n, big, b"big")
    with flock_gb300.SETUPS[small_kind](small_n) as s:
        for i, o in outs:
            assert o.bundle_bytes == s.prove_fast_bytes(small[i % 3], b"s%d" % i)
