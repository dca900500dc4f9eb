"""bench.py's JSON lines: the contract's keys, the whole call covered by the timed steps (no
projection in split mode), and the reference arm's bounded CPU sample."""
import json
import subprocess
import sys

import pytest

from conftest import ROOT

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "dtype", "data", "config", "cpu_baseline", "e2e")


def _run(args, timeout=900):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], check=True, capture_output=True, text=True,
                         timeout=timeout, cwd=ROOT)
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_reference_arm_small_shape(built):
    """--impl reference on the CPU: one JSON line, the reference's keys, a bounded per-step sample
    projected to the whole call, the same workload name as the GPU arm."""
    line = _run(["--impl", "reference", "--o", "6", "--v", "40", "--steps", "2", "--warmup", "1"])
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is False
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["workload"] == "closed-shell (T) o=6 v=40 seed=3 ragged tiles"


@pytest.mark.gpu
def test_split_bench_covers_every_triplet(built):
    """The split-precision bench line at a small shape: the K steps partition every triplet
    (timed_fraction 1, no projection), e2e includes the upload, the parity sample against the
    FP64 path holds S = 3 to 1e-6 relative, and the (T)-equivalent throughput is reported."""
    line = _run(["--o", "8", "--v", "40", "--steps", "3", "--warmup", "3", "--sample", "6", "--cpu-sample", "1"])
    for k in KEYS + ("roofline", "gpu_launches", "clocks", "throughput", "energy_sample"):
        assert k in line, k
    cfg = line["config"]
    assert cfg["timed_fraction"] == 1.0 and cfg["projection"] is None
    assert cfg["triplets_timed"] == cfg["triplets_total"] == 8 * 9 * 10 // 6 - 8
    assert line["e2e"]["value"] >= line["value"] > 0 and line["e2e"]["upload_s"] > 0
    assert line["gpu_launches"] > 0 and line["throughput"]["ref_equiv_tflops"] > 0
    assert line["energy_sample"]["vs_fp64"]["S=3"]["rel_error_of_sum"] <= 1e-6
