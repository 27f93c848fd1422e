"""Generate ligerito_configs.h from the reference's embedded Ligerito security configs.

The prove_fast path reads one security configuration per committed size m and profile
(crates/flock-core/configs/ligerito/m<NN>_<profile>.toml, looked up by
crates/flock-core/src/pcs/ligerito.rs:540-600 and converted to prover parameters by
ligerito.rs:2070-2140). These are protocol parameters, so this script copies the
fields the prover and verifier consume into a C++ table. Run it with the path of the
reference's config directory; the output header is committed.
"""
import re
import sys
from pathlib import Path

FIELDS = ["log_inv_rate", "log_msg_cols", "k_recursive", "queries", "grinding_bits",
          "fold_grinding_bits", "claim_batch_grinding_bits", "consistency_batch_grinding_bits",
          "ood_samples"]


def parse(text):
    top, levels, cur = {}, [], None
    for line in text.splitlines():
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        if line == "[[levels]]":
            cur = {}
            levels.append(cur)
            continue
        if line.startswith("["):
            cur = {}
            continue
        m = re.match(r"(\w+)\s*=\s*(.+)", line)
        if not m:
            continue
        key, val = m.group(1), m.group(2).strip().strip('"')
        (cur if cur is not None else top)[key] = val
    return top, levels


def main(cfg_dir, out_path):
    rows = []
    for m in range(22, 36):
        p = Path(cfg_dir) / f"m{m}_fast.toml"
        if not p.exists():
            continue
        top, levels = parse(p.read_text())
        assert top["hash"] == "sha256", p
        lv = []
        for L in levels:
            lv.append("{" + ", ".join(str(int(L.get(f, 0))) for f in FIELDS) + "}")
        rows.append(f"  {{{m}, {int(top['log_n'])}, {int(top['initial_k'])}, {len(levels)}, {{{', '.join(lv)}}}}},")
    body = "\n".join(rows)
    Path(out_path).write_text(f"""// Generated by gen_ligerito_configs.py from the reference's Fast-profile Ligerito
// security configurations (crates/flock-core/configs/ligerito/m22_fast.toml ..
// m35_fast.toml). Do not edit by hand.
#pragma once
#include <cstdint>

namespace flock {{

struct LigeritoLevelParams {{
  uint32_t log_inv_rate, log_msg_cols, k_recursive, queries, grinding_bits, fold_grinding_bits,
      claim_batch_grinding_bits, consistency_batch_grinding_bits, ood_samples;
}};
struct LigeritoFastConfig {{
  uint32_t m, log_n, initial_k, n_levels;
  LigeritoLevelParams levels[8];
}};

inline const LigeritoFastConfig* ligerito_fast_configs(int* count) {{
  static const LigeritoFastConfig table[] = {{
{body}
  }};
  *count = (int)(sizeof(table) / sizeof(table[0]));
  return table;
}}

}}  // namespace flock
""")


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
