"""Generates tests/golden/open_shell_energies.json from ExaChem's own CPU (T) run unrestricted
(oracle/_ref, ref_ccsd_t_energy_so: ccsd_t_all_fused_cpu.hpp compiled unmodified against
oracle/ref_shim, is_restricted = false) on seeded open-shell systems
(oracle.spin_orbital_oracle.open_shell_system with exact = True: every input is exact in FP64, so
the arrays regenerate bit for bit on any machine).

Run where the reference tree is present:  python tests/golden/make_open_shell_golden.py
The JSON keeps the generator parameters, the alpha / beta tile lists, exact checksums of the
generated t2 and v2iabc, E[T], E(T) and the reference's task count for each case, and the op
counts the reference's CI outputs hold for unrestricted (T) runs (total_num_ops), which pin the
unrestricted task enumeration and spin filters.
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle.spin_orbital_oracle import golden_checksums, open_shell_system  # noqa: E402

CASES = [
    # name, oa, ob, va, vb, nq, seed, tiles (occ_a, occ_b, virt_a, virt_b)
    ("os_o4_3_v12_14", 4, 3, 12, 14, 8, 51, ([2, 2], [3], [5, 7], [6, 8])),
    ("os_o4_1_v10_16", 4, 1, 10, 16, 6, 55, ([4], [1], [10], [16])),
    ("os_o5_4_v20_24", 5, 4, 20, 24, 10, 52, ([3, 2], [4], [8, 8, 4], [10, 14])),
    ("os_o6_2_v30_36_ragged", 6, 2, 30, 36, 9, 54, ([5, 1], [2], [7, 13, 10], [11, 25])),
    ("os_o8_6_v40_44", 8, 6, 40, 44, 12, 53, ([4, 4], [3, 3], [16, 16, 8], [20, 24])),
]


# unrestricted (T) runs in the reference's CI outputs: file, line of total_num_ops, alpha / beta
# occupied and virtual counts (nelectrons_alpha / _beta, nbf - those), tile size, the value
CI_OPS = [
    ("ci/reference_output/ch4.def2-tzvp.ccsd_t.json", 484, 6, 4, 49, 51, 28, 37432196256),
]


def main(reference: str | None = None):
    reference = reference or os.environ.get("CCSDT_REFERENCE")
    if not reference:
        sys.exit("give the reference tree as the first argument or in CCSDT_REFERENCE")
    out = {"generator": "oracle.spin_orbital_oracle.open_shell_system(exact=True)", "cases": [], "ci_ops": []}
    for f, line, oa, ob, va, vb, ts, want in CI_OPS:
        text = (Path(reference) / f).read_text().splitlines()
        assert str(want) in text[line - 1], (f, line, text[line - 1])
        out["ci_ops"].append(dict(file=f, line=line, oa=oa, ob=ob, va=va, vb=vb, ts=ts, total_num_ops=want))
    for name, oa, ob, va, vb, nq, seed, tiles in CASES:
        arrs = open_shell_system(oa, ob, va, vb, nq, seed, exact=True)
        t0 = time.time()
        e4, e5, tasks = oracle.ref_energy_spin_orbital(tiles, np.concatenate(arrs[:2]), *arrs[2:],
                                                       is_restricted=False)
        out["cases"].append(dict(name=name, oa=oa, ob=ob, va=va, vb=vb, nq=nq, seed=seed,
                                 tiles=[list(t) for t in tiles], checksums=golden_checksums(arrs),
                                 e_bracket_T=e4, e_paren_T=e5, ref_tasks=tasks))
        print(f"{name}: E(T) = {e5:.16e}  ({time.time() - t0:.1f} s, {tasks} tasks)")
    path = ROOT / "tests" / "golden" / "open_shell_energies.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {path}")


if __name__ == "__main__":
    main(*sys.argv[1:])
