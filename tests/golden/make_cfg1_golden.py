"""Generates tests/golden/cfg1_energy.json: the whole closed-shell (T) at o=21, v=180, seed 1
(the drop-in configuration: tiles of 40, ragged last virtual tile of 20) from the oracle's C
restatement (oracle/ccsdt_oracle.c, every triplet i <= j <= k, compensated sums), which matches
ExaChem's own CPU (T) (oracle/_ref) to 1e-14 relative on the systems of reference_energies.json.
The reference's own CPU kernel is not run at this size: it materialises two ts^6 t3 blocks per
task (ccsd_t_all_fused_cpu.hpp:103-108) and does 7.5x the arithmetic of the spatial formulation.

Also records the per-triplet energies of an evenly spread sample, for quicker checks.  Runs on
the CPU (about half an hour on 8 cores):
    python tests/golden/make_cfg1_golden.py
"""
from __future__ import annotations

import json
import math
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from exachem_gb300.generator import generate, tiles_uniform  # noqa: E402

O, V, SEED, TS = 21, 180, 1, 40


def main():
    d = generate(O, V, SEED)
    tri = np.array([(i, j, k) for i in range(O) for j in range(i, O) for k in range(j, O)], dtype=np.int32)
    t0 = time.time()
    e4, e5 = oracle.triplets(d, tri)
    secs = time.time() - t0
    tot4, tot5 = math.fsum(e4), math.fsum(e5)   # correctly rounded totals
    samp = [int(x) for x in np.linspace(0, len(tri) - 1, 24).round()]
    out = {"generator": "exachem_gb300.generator.generate", "o": O, "v": V, "seed": SEED,
           "occ_tiles": tiles_uniform(O, TS), "vir_tiles": tiles_uniform(V, TS),
           "e_bracket_T": tot4, "e_paren_T": tot5, "n_triplets": int(len(tri)),
           "oracle": "oracle/ccsdt_oracle.c (oracle_triplets), math.fsum over triplets",
           "oracle_threads": oracle.num_threads(), "oracle_seconds": secs,
           "sample": [{"tri": [int(x) for x in tri[s]], "e_bracket_T": float(e4[s]), "e_paren_T": float(e5[s])}
                      for s in samp]}
    path = ROOT / "tests" / "golden" / "cfg1_energy.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"E[T] = {tot4:.16e}  E(T) = {tot5:.16e}  ({secs:.0f} s) -> {path}")


if __name__ == "__main__":
    main()
