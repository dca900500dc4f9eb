"""Generates tests/golden/reference_energies.json from ExaChem's own CPU (T)
(oracle/_ref: exachem/cc/ccsd_t/ccsd_t_all_fused_cpu.hpp compiled unmodified against
oracle/ref_shim) on seeded synthetic inputs (exachem_gb300.generator).

Run where the reference tree is present:  python tests/golden/make_golden.py
The JSON keeps the generator parameters, the tile layout, E[T], E(T), the reference's
own op count (fused_common.hpp:34-128) and its task count for each case.

It also records the op counts the reference's CI outputs hold for (T) runs
(ci/reference_output/*ccsd_t*.json, field total_num_ops) with the orbital counts
and tile size of those runs, which pin the task enumeration and equation enabling.
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from exachem_gb300.generator import generate, tiles_uniform  # noqa: E402

CASES = [
    # name, o, v, seed, occ_tiles, vir_tiles, t2_scale
    ("cfg0_o8_v40_ts16", 8, 40, 0, tiles_uniform(8, 16), tiles_uniform(40, 16), 1.0),
    ("o6_v24_ts5", 6, 24, 0, tiles_uniform(6, 5), tiles_uniform(24, 5), 1.0),
    ("o5_v17_ts3", 5, 17, 7, tiles_uniform(5, 3), tiles_uniform(17, 3), 1.0),
    ("o3_v7_ts2", 3, 7, 5, tiles_uniform(3, 2), tiles_uniform(7, 2), 1.0),
    ("o8_v40_ragged", 8, 40, 11, [3, 5], [7, 13, 20], 1.0),
    ("o6_v20_t2x2.5", 6, 20, 12, [6], [8, 12], 2.5),
    ("o2_v2", 2, 2, 2, [2], [2], 1.0),
    ("o1_v3_zero", 1, 3, 1, [1], [3], 1.0),
    ("o4_v12_ts16", 4, 12, 0, [4], [12], 1.0),
    ("o7_v9_ts4", 7, 9, 3, tiles_uniform(7, 4), tiles_uniform(9, 4), 1.0),
]

# (T) runs in the reference's CI outputs: file, line of total_num_ops, o, v, tile size
CI_OPS = [
    ("ci/reference_output/butanol2_pt.sto-3g.ccsd_t.json", 262, 21, 14, 40, 30952040112),
    ("ci/reference_output/uracil.cc-pvdz.ccsd_t.json", 383, 29, 103, 40, 62789556886348),
    ("ci/reference_output/seh2.cc-pvdz.ccsd_t.json", 263, 9, 36, 40, 52991044992),
]


def main(reference: str | None = None):
    reference = reference or os.environ.get("CCSDT_REFERENCE")
    if not reference:
        sys.exit("give the reference tree as the first argument or in CCSDT_REFERENCE")
    out = {"generator": "exachem_gb300.generator.generate", "cases": [], "ci_ops": []}
    for name, o, v, seed, ot, vt, sc in CASES:
        d = generate(o, v, seed, t2_scale=sc)
        t0 = time.time()
        r = oracle.reference_energy(d, ot, vt)
        out["cases"].append(dict(name=name, o=o, v=v, seed=seed, occ_tiles=ot, vir_tiles=vt, t2_scale=sc,
                                 e_bracket_T=r["e_bracket_T"], e_paren_T=r["e_paren_T"], ref_ops=r["ops"],
                                 ref_tasks=r["tasks"]))
        print(f"{name}: E(T) = {r['e_paren_T']:.16e}  ({time.time() - t0:.1f} s)")
    for f, line, o, v, ts, want in CI_OPS:
        text = (Path(reference) / f).read_text().splitlines()
        assert str(want) in text[line - 1], (f, line, text[line - 1])
        out["ci_ops"].append(dict(file=f, line=line, o=o, v=v, ts=ts, total_num_ops=want))
    (Path(__file__).parent / "reference_energies.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main(*sys.argv[1:])
