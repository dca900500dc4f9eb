"""The drop-in adapter (include/exachem_compat/ccsd_t_fused_driver.hpp) fed spin-orbital
tiled tensors the way ExaChem holds them: the gather must reproduce the closed-shell
spatial arrays bit for bit (CPU), and the full call must reproduce the reference's E(T)
(GPU)."""
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_close

KEYS = ["eps_occ", "eps_vir", "t1", "t2", "oovv", "ooov", "ovvv"]


def _compile(tmp_path, link_lib=False):
    exe = tmp_path / "compat_driver"
    cmd = ["g++", "-O2", "-std=c++17", str(ROOT / "tests" / "compat" / "compat_driver.cpp"), "-o", str(exe),
           "-I", str(ROOT / "include"), "-I", str(ROOT / "oracle"), "-I", str(ROOT / "oracle" / "ref_shim")]
    if link_lib:
        lib = ROOT / "exachem_gb300" / "_build"
        cmd += ["-L", str(lib), "-lccsdt_gb300", f"-Wl,-rpath,{lib}"]
    else:
        cmd += ["-DCCSDT_NO_LINK"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _write(path, d, ot, vt):
    with open(path, "wb") as f:
        np.array([d["o"], d["v"], len(ot), len(vt)] + list(ot) + list(vt), dtype=np.int32).tofile(f)
        for k in KEYS:
            np.ascontiguousarray(d[k], dtype=np.float64).tofile(f)


def _read(path, d, extra=0):
    raw = np.fromfile(path, dtype=np.float64)
    out, off = {}, 0
    for k in KEYS:
        n = d[k].size
        out[k] = raw[off:off + n].reshape(d[k].shape)
        off += n
    return out, raw[off:off + extra]


def test_adapter_gather_is_exact(tmp_path, built):
    from exachem_gb300.generator import generate
    exe = _compile(tmp_path, link_lib=True)
    for (o, v, seed, ot, vt) in [(5, 11, 3, [2, 3], [4, 4, 3]), (4, 9, 8, [4], [9])]:
        d = generate(o, v, seed)
        _write(tmp_path / "in.bin", d, ot, vt)
        subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
        got, _ = _read(tmp_path / "out.bin", d)
        for k in KEYS:
            assert np.array_equal(got[k], d[k]), k


@pytest.mark.gpu
def test_adapter_full_call_matches_reference_golden(tmp_path, built, golden):
    from exachem_gb300.generator import generate
    exe = _compile(tmp_path, link_lib=True)
    c = next(c for c in golden["cases"] if c["name"] == "o8_v40_ragged")
    d = generate(c["o"], c["v"], c["seed"])
    _write(tmp_path / "in.bin", d, c["occ_tiles"], c["vir_tiles"])
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "--run"], check=True)
    _, e = _read(tmp_path / "out.bin", d, extra=2)
    assert rel_close(e[0], c["e_bracket_T"], 1e-12) and rel_close(e[1], c["e_paren_T"], 1e-12)


@pytest.mark.gpu
def test_adapter_tiled_call_matches_reference_golden(tmp_path, built, golden):
    """The drop-in path proper: the adapter reads every block with Tensor::get and hands the blocks
    to the device-side retile (ccsdt_upload_blocks) - no host gather of the four-index arrays."""
    from exachem_gb300.generator import generate
    exe = _compile(tmp_path, link_lib=True)
    c = next(c for c in golden["cases"] if c["name"] == "o8_v40_ragged")
    d = generate(c["o"], c["v"], c["seed"])
    _write(tmp_path / "in.bin", d, c["occ_tiles"], c["vir_tiles"])
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "--run-tiled"], check=True)
    _, e = _read(tmp_path / "out.bin", d, extra=2)
    assert rel_close(e[0], c["e_bracket_T"], 1e-12) and rel_close(e[1], c["e_paren_T"], 1e-12)
