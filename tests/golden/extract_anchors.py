"""Regenerates anchors.json from the reference's own test sources (read as text).

The digests are the reference's pinned values; nothing is recomputed here. Run with the
reference checkout as the first argument:
    python tests/golden/extract_anchors.py <reference-root>
"""
import json
import os
import re
import sys


def main(root: str) -> None:
    fx = open(os.path.join(root, "crates/flock-prover/tests/union_m6_fixtures.rs")).read()
    body = fx[fx.index("fn m6_single_slot_merged_anchor_proof_bytes_pinned"):]
    digests = re.findall(r'const EXPECTED: &str = "([0-9a-f]{64})"', body)[:2]
    seeds = [int(s.replace("_", ""), 16) for s in re.findall(r"Rng::new\((0x[0-9A-Fa-f_]+)\)", body)[:2]]
    counts = [int(n) for n in re.findall(r"let n_blocks = (\d+)usize", body)[:2]]
    sched = open(os.path.join(root, "crates/flock-core/src/schedule.rs")).read()
    sb = sched[sched.index("fn boolean_only_digest_is_byte_identical"):]
    reg = re.findall(r'"([0-9a-f]{64})"', sb)[:2]
    # mixed two-slot union fixtures: (label, [n_sha2, n_blake3], digest) of
    # m6_merged_union_proof_bytes_pinned, digested over MixedProofBundleLigerito::to_bytes
    mb = fx[fx.index("fn m6_merged_union_proof_bytes_pinned"):fx.index("fn m6_single_slot_merged_anchor_proof_bytes_pinned")]
    mixed = [{"name": lab, "counts": [int(a), int(b)], "digest": d}
             for lab, a, b, d in re.findall(r'\(\s*"([^"]+)",\s*\[(\d+),\s*(\d+)\],\s*"([0-9a-f]{64})",?\s*\)', mb)]
    nu = int(re.search(r"let nu = (\d+)usize;", mb).group(1))
    seed_base = int(re.search(r"Rng::new\((0x[0-9A-Fa-f_]+) \^", mb).group(1).replace("_", ""), 16)
    here = os.path.dirname(os.path.abspath(__file__))
    path = os.path.join(here, "anchors.json")
    data = json.load(open(path))
    data["mixed"] = {
        "source": "crates/flock-prover/tests/union_m6_fixtures.rs:196-281 (m6_merged_union_proof_bytes_pinned)",
        "registry": "BLAKE3 + SHA-256, slot order SHA-256 then BLAKE3 (MixedRegistryId::Blake3Sha2Nu10, code 2)",
        "nu": nu,
        "seed": "seed_base ^ (n_sha2 << 16) ^ n_blake3; SHA-256 records (h[8], w[16]) first, then BLAKE3 "
                "records (cv[8], m[16], counter=(hi<<32)|lo, block_len 64, flags 11) from the same stream",
        "seed_base": seed_base,
        "digest_over": "SHA-256 of MixedProofBundleLigerito::to_bytes || ab.lo || ab.hi || c.lo || c.hi",
        "fixtures": mixed,
    }
    for entry, d, s, n in zip(data["prove_fast"], digests, seeds, counts):
        entry["digest"], entry["seed"], entry["n_blocks"] = d, s, n
    for entry, d in zip(data["registry"], reg):
        entry["digest"] = d
    json.dump(data, open(path, "w"), indent=2)
    print(json.dumps(data, indent=2))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else ".")
