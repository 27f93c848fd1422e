"""Benchmark: proved hashes per second of prove_fast on one GB300.

Default workload: prove_fast of a Keccak-f[1600] batch of 2^18 permutations (m = 34, 42
commit lanes; the largest single-GPU configuration), seeded synthetic inputs (25 uniform
u64 lanes). One step = one full prove (witness generation through proof bytes) of one
batch. At N = 1 the BLAKE3 2^12 and SHA-256 2^16 workloads are measured the same way in
the same run and reported under "other_workloads" of the one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload keccak|sha256|blake3]
    python bench.py --impl reference ...   # the CPU restatement, timed on the host cores

value : inputs already resident in HBM (flock_gb300_prove_fast_device), CUDA events on
        the library's stream around K proves, k hashes/s over all ranks.
e2e   : the public host-buffer call (Setup.prove_fast: host->device copy of the inputs
        and the proof bytes back inside the timed region).
roofline : the stage with the most device time in the timed region, its algorithmic
        bytes per launch over its CUDA-event duration, against the measured HBM copy
        bandwidth.
Multi-GPU: replicas only (each rank proves its own batch; no collective on the data path).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k hashes/s proved per GB300 vs host CPU prove_fast; p50/p99 served proof latency"
UNIT = "k hashes/s"
WORKLOADS = {
    # name: (kind, batch, description)
    "blake3": (0, 1 << 12, "prove_fast BLAKE3 batch 2^12 (counter=index, block_len 64, flags 0)"),
    "sha256": (1, 1 << 16, "prove_fast SHA-256 batch 2^16"),
    "keccak": (2, 1 << 18, "prove_fast Keccak-f[1600] batch 2^18"),
}
HEADLINE = "keccak"
# CPU sample per workload: the largest batch of the same hash whose oracle prove (all host
# threads) stays within a few seconds, so that warm-up + best of 3 and the reference arm's
# W + K steps end within minutes: the configured batch for BLAKE3 2^12 and SHA-256 2^16
# (about 0.1 s and 2 s per prove on 16 Grace cores), half of it for Keccak-f 2^18 (about
# 6.5 s per prove at 2^17).
CPU_SAMPLE = {"blake3": 1 << 12, "sha256": 1 << 16, "keccak": 1 << 17}
# The reference's own published CPU rates for the configured batches (k hashes/s;
# README.md:50-64, AMD Threadripper 7970X, best of 3 after a verified warm-up).
PUBLISHED_CPU = {
    "blake3": {"batch": 4096, "one_thread": 54.0, "threads_32": 227.1, "source": "README.md:56"},
    "sha256": {"batch": 65536, "one_thread": 32.0, "threads_32": 271.3, "source": "README.md:53"},
    "keccak": {"batch": 262144, "one_thread": 17.6, "threads_32": 164.3, "source": "README.md:64"},
}
DOMAIN = b"flock-gb300-bench"
SEED = 0x5EED


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def algorithmic_bytes(stage: str, m: int, lanes: int, k_code: int, n: int, kind: int) -> float | None:
    """Algorithmic bytes of one prove's `stage` (summed over its launches): the data the
    stage must read and write at least once."""
    W = 1 << (m - 7)           # F128 words of z, a, b
    code_words = lanes << k_code
    rec = (112, 96, 200)[kind]
    table = {
        "witness": n * rec + 3 * 16 * W,
        "l0_fill": 16 * lanes * (1 << (k_code - 1)) + 16 * code_words,
        "l0_ntt": 2 * 16 * code_words,
        "l0_merkle": 16 * code_words + 32 * (2 * (1 << k_code) - 1),
        "zc_round1": 3 * 16 * W,
        "zc_fold_skip": 2 * 16 * W + 2 * 32 * W,
        "mo_build_w": 16 * W + 16 * W,
        # folds: each round reads both vectors and writes both halves
        "zc_folds": sum(2 * 16 * (3 * (1 << (m - 6 - i)) // 2) for i in range(1, m - 6)),
        "mo_rounds": sum(2 * 16 * (3 * (W >> i) // 2) for i in range(0, m - 8)),
    }
    return table.get(stage)


def algorithmic_muls(stage: str, lanes: int, k_code: int) -> float | None:
    """GF(2^128) products one prove's `stage` must compute (the multiply-bound stages):
    the additive NTT does one product per butterfly, lanes * 2^(k_code-1) butterflies in
    each of its k_code - 1 layers (the first layer of the rate-1/2 code is a copy)."""
    table = {"l0_ntt": lanes * (1 << (k_code - 1)) * (k_code - 1)}
    return table.get(stage)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        mx = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()) if rows else None}


# ------------------------------------------------------------------ CPU baseline (oracle)
def host_threads() -> int:
    """Threads the oracle's host pool runs a prove on: its workers plus the caller."""
    c = os.cpu_count() or 1
    return min(c - 2, 15) + 1 if c > 2 else 1


def cpu_sample_rate(workload: str, rounds: int = 3) -> dict:
    """The oracle's prove_fast of the sample batch, each prove spread over the host thread
    pool: one warm-up prove whose bundle the restated verifier accepts, then the best of
    `rounds` timed proves (the reference's hash_throughput.rs:64-83 method); k hashes/s."""
    import oracle
    from flock_gb300 import inputs

    kind = WORKLOADS[workload][0]
    n = CPU_SAMPLE[workload]
    oracle.registry_digest(kind, n)  # statement set-up outside the timed region
    recs = inputs.batch(kind, n, SEED + 1000)
    warm = oracle.prove_fast_bytes(kind, recs, DOMAIN)
    ok, why = oracle.verify(kind, n, warm, DOMAIN)
    if not ok:
        raise SystemExit(f"oracle warm-up proof rejected by the verifier: {why}")
    best = None
    for _ in range(rounds):
        t0 = time.perf_counter()
        out = oracle.prove_fast_bytes(kind, recs, DOMAIN)
        dt = time.perf_counter() - t0
        if out != warm:
            raise SystemExit("oracle proves of the same inputs differ")
        best = dt if best is None else min(best, dt)
    return {"value": n / best / 1e3, "unit": UNIT, "cores": host_threads(), "kind": "port",
            "sample": f"oracle prove_fast of a {workload} batch of {n} compressions (seed {SEED + 1000}) on the host "
                      f"thread pool; one verified warm-up, best of {rounds}",
            "same_config": n == WORKLOADS[workload][1], "sample_batch": n,
            "published_reference": PUBLISHED_CPU[workload]}


# ------------------------------------------------------------------ distributed helpers
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = os.environ.get("FLOCK_GB300_DIST_BACKEND") or ("nccl" if torch.cuda.is_available() else "gloo")
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ arms
def run_reference(args, world, rank):
    if rank != 0:
        return 0
    wl = args.workload
    W, K = args.warmup, args.steps
    n = args.batch or CPU_SAMPLE[wl]
    import oracle
    from flock_gb300 import inputs

    kind = WORKLOADS[wl][0]
    threads = host_threads()
    oracle.registry_digest(kind, n)
    recs = inputs.batch(kind, n, SEED + 1000)
    times = []
    first = None
    for step in range(W + K):
        t0 = time.perf_counter()
        out = oracle.prove_fast_bytes(kind, recs, DOMAIN)
        dt = time.perf_counter() - t0
        if first is None:
            first = out
            ok, why = oracle.verify(kind, n, out, DOMAIN)
            if not ok:
                raise SystemExit(f"oracle proof rejected by the verifier: {why}")
        elif out != first:
            raise SystemExit("oracle proves of the same inputs differ")
        if step >= W:
            times.append(dt)
    total = sum(times)
    value = K * n / total / 1e3
    same = n == WORKLOADS[wl][1]
    sample = (f"each step: one oracle prove_fast (C++ restatement of the reference's prove_fast) of a {wl} batch of "
              f"{n} compressions{'' if same else ' (the configured batch is ' + str(WORKLOADS[wl][1]) + ')'}, "
              f"spread over {threads} host threads; the first proof is checked by the restated verifier")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "gf2_128", "data": "synthetic (seeded SplitMix64 inputs)",
        "config": {"workload": WORKLOADS[wl][2] + ("" if same else f" (CPU sample: batch {n})"), "hash": wl,
                   "batch": n, "configured_batch": WORKLOADS[wl][1], "same_config": same, "threads": threads},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "same_config": same, "published_reference": PUBLISHED_CPU[wl]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, world, rank, local):
    line = measure(args.workload, args, world, rank, local)
    if rank != 0:
        return 0
    if world == 1 and not args.batch and not args.no_other_workloads:
        others = {}
        for wl in sorted(WORKLOADS):
            if wl == args.workload:
                continue
            o = measure(wl, args, world, rank, local)
            others[wl] = {k: o[k] for k in ("value", "unit", "ms_per_step", "config", "latency_ms", "e2e",
                                            "roofline", "stages_ms_per_prove", "host_phase_ms", "gpu_launches",
                                            "clocks", "cpu_baseline")}
        line["other_workloads"] = others
    print(json.dumps(line), flush=True)
    return 0


def measure(wl, args, world, rank, local):
    """One workload's bench line: K device-resident proves, K host-buffer proves, the
    roofline stage and (rank 0, N = 1) the CPU baseline."""
    import numpy as np
    import torch

    import flock_gb300
    from flock_gb300 import inputs

    kind, n, desc = WORKLOADS[wl]
    if args.batch:
        n = args.batch
    torch.cuda.set_device(local)
    setup = flock_gb300.SETUPS[kind](n)
    host = inputs.batch(kind, n, SEED + rank)
    dev = torch.from_numpy(np.frombuffer(host.tobytes(), dtype=np.uint8).copy()).to(f"cuda:{local}")
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(setup.stream_handle(), device=f"cuda:{local}")
    lib = flock_gb300.load()

    def prove_dev():
        return setup.prove_fast_device_bytes(dev.data_ptr(), n, DOMAIN)

    # warm-up (also a parity check of the two entry points)
    for _ in range(args.warmup):
        a = prove_dev()
    b = setup.prove_fast_bytes(host, DOMAIN)
    if a != b:
        raise SystemExit("device-input and host-input proves differ")
    bundle_len = len(b)

    # ---- stage breakdown of one prove (outside the timed region): picks the roofline kernel
    setup.set_stage_timing(True)
    prove_dev()
    calib = setup.last_stage_ms()
    phases_calib = setup.last_phase_ms()
    ranked = sorted(calib.items(), key=lambda kv: -kv[1][0])
    dominant = next((k for k, _ in ranked if algorithmic_bytes(k, setup.m, setup.lanes, setup.log_code_len, n, kind)),
                    ranked[0][0])

    # ---- integer-pipe peak: throughput of the device GF(2^128) product (its own launch)
    import ctypes
    mul_peak = ctypes.c_double()
    flock_gb300._native.check(lib.flock_gb300_f128_mul_rate(256, ctypes.byref(mul_peak)))
    mul_peak = mul_peak.value
    mix_peak = ctypes.c_double()
    flock_gb300._native.check(lib.flock_gb300_f128_table_mix_rate(256, ctypes.byref(mix_peak)))
    mix_peak = mix_peak.value

    # ---- value: inputs resident in HBM; events only around the roofline stage
    setup.set_stage_timing([dominant])
    L2_BYTES = 129 << 20
    working_set = 3 * 16 * (1 << (setup.m - 7))
    flush = torch.zeros(512 << 18, dtype=torch.int32, device=f"cuda:{local}") if working_set < 2 * L2_BYTES else None
    dom_ms, dom_launches = 0.0, 0
    step_ms = []
    barrier(world)
    torch.cuda.synchronize()
    launches0 = lib.flock_gb300_launch_count()
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            if flush is not None:  # working set below 2x L2: evict it between steps
                with torch.cuda.stream(stream):
                    flush.add_(1)
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            prove_dev()
            s1.record(stream)
            d_ms, d_l = setup.last_stage_ms()[dominant]
            dom_ms += d_ms
            dom_launches += d_l
            step_ms.append((s0, s1))
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = lib.flock_gb300_launch_count() - launches0  # this library's kernels only
    phases = setup.last_phase_ms()
    barrier(world)
    per_step = [a.elapsed_time(b) for a, b in step_ms]
    # with flushes, the timed region is the sum of the steps (flush kernels excluded)
    ms = allmax(world, sum(per_step) if flush is not None else ev0.elapsed_time(ev1))
    setup.set_stage_timing(False)
    value = world * n * args.steps / (ms / 1e3) / 1e3

    # ---- e2e: host buffers through the public call
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        setup.prove_fast_bytes(host, DOMAIN)
    e1.record(stream)
    torch.cuda.synchronize()
    h2d, d2h = setup.last_transfer_bytes()
    barrier(world)
    e2e_ms = allmax(world, e0.elapsed_time(e1))
    e2e = world * n * args.steps / (e2e_ms / 1e3) / 1e3

    # ---- roofline of the stage with the most device time
    peak, peak_src = peaks()
    m, lanes = setup.m, setup.lanes
    alg = algorithmic_bytes(dominant, m, lanes, setup.log_code_len, n, kind)
    roof = None
    if alg and dom_launches:
        per_prove_ms = dom_ms / args.steps
        achieved = alg / (per_prove_ms / 1e3) / 1e9
        traffic = None
        tf = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tf):
            try:
                traffic = json.load(open(tf)).get(wl, {}).get(dominant) if not args.batch else None
            except Exception:
                traffic = None
        roof = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "traffic_scope": "DRAM bytes per launch (profiles/traffic.json)" if traffic else None,
                "algorithmic_bytes_per_launch": alg / max(1.0, dom_launches / args.steps), "algorithmic_bytes": alg,
                "launches_per_prove": dom_launches / args.steps, "device_ms_per_prove": per_prove_ms,
                "peak_source": f"{peak_src} hbm_gbs", "share_of_step": per_prove_ms / (ms / args.steps)}
        muls = algorithmic_muls(dominant, lanes, setup.log_code_len)
        if muls:
            rate = muls / (per_prove_ms / 1e3)
            roof["mul_pipe"] = {"achieved": rate, "peak": mix_peak, "unit": "F128 mul/s", "frac": rate / mix_peak,
                                "algorithmic_muls": muls,
                                "peak_source": "measured live: flock_gb300_f128_table_mix_rate (products by a block "
                                               "constant, half from shared-memory byte tables, half integer-multiply)",
                                "peak_multiply_only": mul_peak,
                                "frac_of_multiply_only": rate / mul_peak}
    if rank != 0:
        setup.close()
        return None

    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample_rate(wl, rounds=3)
    per_step.sort()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "gf2_128", "data": "synthetic (seeded SplitMix64 inputs)",
        "config": {"workload": desc, "hash": wl, "batch": n, "m": m, "lanes": lanes,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": ("flushed between steps (512 MiB write, outside the step events)" if flush is not None else
                          "no flush: every step streams z, a, b and the codeword, each larger than L2"),
                   "seed": SEED},
        "latency_ms": {"p50": per_step[len(per_step) // 2], "p99": per_step[min(len(per_step) - 1,
                                                                             int(0.99 * len(per_step)))]},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "bundle_bytes": bundle_len},
        "roofline": roof,
        "stages_ms_per_prove": {k: round(v[0], 4) for k, v in ranked},
        "host_phase_ms": {k: round(v, 3) for k, v in phases.items()},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    setup.close()
    return line


def mixed_workload(count: int, seed: int, lo_log: int, hi_log: int):
    """Seeded mixed requests: hash uniform over the three kinds, batch 2^U(lo..hi) compressions
    (kept at or above each hash's smallest full-utilisation batch)."""
    import random

    from flock_gb300 import inputs

    rng = random.Random(seed)
    out = []
    floor = {0: 8, 1: 7, 2: 6}
    for i in range(count):
        kind = rng.randrange(3)
        lg = max(floor[kind], int(round(rng.uniform(lo_log, hi_log))))
        out.append((kind, inputs.batch(kind, 1 << lg, seed * 1000 + i), b"flock-gb300-mixed-%d" % i))
    return out


def run_batched(args):
    """64 mixed proofs: batched (concurrent provers) against one-proof-at-a-time on the
    same GPU, identical bundles required."""
    import flock_gb300

    reqs = mixed_workload(args.count, SEED, 10, args.max_log)
    hashes = sum(len(r) for _, r, _ in reqs)
    # plain path: one setup per shape, proofs one after another
    setups = {}
    for kind, recs, dom in reqs:
        setups.setdefault((kind, len(recs)), flock_gb300.SETUPS[kind](len(recs)))
    for (kind, n), st in setups.items():  # warm-up: device buffers and level twiddles
        st.prove_fast_bytes(next(r for k, r, _ in reqs if k == kind and len(r) == n), b"warm")
    # device-busy fraction of the plain run: kernel time inside the stages (CUDA events
    # around every stage; includes the device idle time inside a stage's round trips, so
    # an upper bound) over the wall time
    for st in setups.values():
        st.set_stage_timing(True)
    t0 = time.perf_counter()
    plain = []
    stage_ms = 0.0
    for k, r, d in reqs:
        st = setups[(k, len(r))]
        plain.append(st.prove_fast_bytes(r, d))
        stage_ms += sum(v[0] for v in st.last_stage_ms().values())
    t_plain = time.perf_counter() - t0
    for st in setups.values():
        st.set_stage_timing(False)
    t0 = time.perf_counter()
    plain_untimed = [setups[(k, len(r))].prove_fast_bytes(r, d) for k, r, d in reqs]
    t_plain = time.perf_counter() - t0
    for st in setups.values():
        st.close()
    if plain_untimed != plain:
        raise SystemExit("plain proves differ between runs")
    if args.plain_only:
        print(json.dumps({"mode": "batched-plain", "plain_value": hashes / t_plain / 1e3, "unit": UNIT,
                          "plain_s": t_plain, "stage_event_ms": stage_ms, "n_proofs": len(reqs)}), flush=True)
        return 0
    with flock_gb300.ProofServer(workers=args.workers) as srv:
        srv.prove_batch(reqs, raw=True)  # warm-up: the server's provers for every shape of the batch
        t0 = time.perf_counter()
        outs = srv.prove_batch(reqs, raw=True)
        t_batch = time.perf_counter() - t0
    same = all(o.bundle_bytes == p for o, p in zip(outs, plain))
    lat = sorted(o.latency_ms for o in outs)
    line = {"metric": METRIC, "mode": "batched", "value": hashes / t_batch / 1e3, "unit": UNIT,
            "plain_value": hashes / t_plain / 1e3, "speedup_vs_plain": t_plain / t_batch, "identical_bundles": same,
            "plain_stage_event_busy_upper_bound": stage_ms / 1e3 / t_plain,
            "n_proofs": len(reqs), "hashes": hashes, "workers": args.workers,
            "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
            "config": {"workload": f"{len(reqs)} proofs, hash uniform over BLAKE3/SHA-256/Keccak-f, batch 2^U(10..{args.max_log})",
                       "seed": SEED}, "data": "synthetic (seeded SplitMix64 inputs)", "n_gpus": 1}
    print(json.dumps(line), flush=True)
    return 0


def run_served(args):
    """Poisson arrivals through the serving loop at each rate of --rates (proofs/s); p50/p99
    latency and throughput per rate, for the served form (--workers provers) and the plain
    one-proof-at-a-time form (the same engine with one prover) on the same stream. Every
    served bundle is checked against the plain one of the same request."""
    import random

    import flock_gb300

    reqs = mixed_workload(args.count, SEED + 1, 10, args.max_log)
    hashes = sum(len(r) for _, r, _ in reqs)
    rates = [float(x) for x in (args.rates.split(",") if args.rates else [args.rate])]

    def serve(workers, rate):
        rng = random.Random(SEED)
        with flock_gb300.ProofServer(workers=workers, hbm_budget_bytes=args.hbm_budget_gib << 30) as srv:
            # warm-up: one request of every shape of the stream (provers, buffers, twiddles)
            seen = {}
            for k, r, d in reqs:
                seen.setdefault((k, len(r)), (k, r, d))
            srv.prove_batch(list(seen.values()), raw=True)
            tickets = []
            t0 = time.perf_counter()
            t_next = t0
            for k, r, d in reqs:
                now = time.perf_counter()
                if t_next > now:
                    time.sleep(t_next - now)
                tickets.append(srv.submit(k, r, d))
                t_next += rng.expovariate(rate)
            outs = [srv.result(t, raw=True) for t in tickets]
            t_all = time.perf_counter() - t0
        lat = sorted(o.latency_ms for o in outs)
        return outs, {"value": hashes / t_all / 1e3, "wall_s": t_all,
                      "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                                     "max": lat[-1]}}

    points = []
    for rate in rates:
        outs, served = serve(args.workers, rate)
        plain_outs, plain = serve(1, rate)
        same = all(a.bundle_bytes == b.bundle_bytes for a, b in zip(outs, plain_outs))
        points.append({"offered_rate_proofs_per_s": rate, "served": served, "plain_one_prover": plain,
                       "identical_bundles": same})
    line = {"metric": METRIC, "mode": "served", "unit": UNIT, "n_proofs": len(reqs), "hashes": hashes,
            "workers": args.workers, "hbm_budget_gib": args.hbm_budget_gib, "rates": points,
            "config": {"workload": f"{len(reqs)} Poisson arrivals, hash uniform, batch 2^U(10..{args.max_log})",
                       "seed": SEED}, "data": "synthetic (seeded SplitMix64 inputs)", "n_gpus": 1}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=HEADLINE)
    ap.add_argument("--batch", type=int, default=0, help="override the batch size (parity-test sizes)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="measure the chosen workload only (no other_workloads in the line)")
    ap.add_argument("--mode", choices=["plain", "batched", "served"], default="plain",
                    help="plain: the contract line; batched / served: the mixed-workload lines")
    ap.add_argument("--count", type=int, default=64, help="proofs in the batched / served workload")
    ap.add_argument("--max-log", type=int, default=16, help="largest batch 2^max_log in the mixed workloads")
    ap.add_argument("--workers", type=int, default=2)
    ap.add_argument("--rate", type=float, default=200.0, help="served mode: Poisson arrival rate (proofs/s)")
    ap.add_argument("--rates", default="", help="served mode: comma-separated arrival rates to sweep")
    ap.add_argument("--hbm-budget-gib", type=int, default=200, help="served mode: device-memory budget")
    ap.add_argument("--plain-only", action="store_true", help="batched mode: the plain run only")
    args = ap.parse_args()
    if args.mode != "plain":
        import __graft_entry__

        __graft_entry__.build()
        return run_batched(args) if args.mode == "batched" else run_served(args)
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_init()
    if args.impl == "reference":
        rc = run_reference(args, world, rank)
    else:
        import __graft_entry__

        if rank == 0:
            __graft_entry__.build()
        barrier(world)
        if rank != 0:
            __graft_entry__.build()
        rc = run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
