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


def _cholesky_case(o, v, nq, seed):
    """The generator's amplitudes with integrals from random spatial Cholesky vectors L[p][q][Q]
    (symmetric in p, q; occupied orbitals first)."""
    from exachem_gb300.generator import generate
    d = generate(o, v, seed)
    rng = np.random.default_rng(seed + 500)
    L = rng.normal(0.0, 0.05, size=(o + v, o + v, nq))
    L = 0.5 * (L + L.transpose(1, 0, 2))
    Lov, Loo, Lvv = L[:o, o:], L[:o, :o], L[o:, o:]
    d["oovv"] = np.einsum("iaQ,jbQ->ijab", Lov, Lov)
    d["ooov"] = np.einsum("ijQ,kaQ->ijka", Loo, Lov)
    d["ovvv"] = np.einsum("iaQ,bcQ->iabc", Lov, Lvv)
    return d, L


def _write_chol(path, L, ci_tiles):
    with open(path, "wb") as f:
        np.array([L.shape[2], len(ci_tiles)] + list(ci_tiles), dtype=np.int32).tofile(f)
        np.ascontiguousarray(L, dtype=np.float64).tofile(f)


def test_adapter_cholesky_gather_is_exact(tmp_path, built):
    """gather_cholesky reads the alpha-alpha blocks of a tiled spin-orbital cholVpr {MO, MO, CI}
    back into the spatial vectors bit for bit."""
    exe = _compile(tmp_path, link_lib=True)
    o, v, ot, vt, ci = 5, 11, [2, 3], [4, 4, 3], [3, 4]
    d, L = _cholesky_case(o, v, sum(ci), 21)
    _write(tmp_path / "in.bin", d, ot, vt)
    _write_chol(tmp_path / "chol.bin", L, ci)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "--chol", str(tmp_path / "chol.bin")],
                   check=True)
    nq = sum(ci)
    _, extra = _read(tmp_path / "out.bin", d, extra=(o * o + o * v + v * v) * nq)
    Loo = extra[:o * o * nq].reshape(o, o, nq)
    Lov = extra[o * o * nq:(o * o + o * v) * nq].reshape(o, v, nq)
    Lvv = extra[(o * o + o * v) * nq:].reshape(v, v, nq)
    assert np.array_equal(Loo, L[:o, :o]) and np.array_equal(Lov, L[:o, o:]) and np.array_equal(Lvv, L[o:, o:])


@pytest.mark.gpu
@pytest.mark.parametrize("slabs", [None, "4"])
def test_adapter_cholesky_call_matches_oracle(tmp_path, built, slabs):
    """The Cholesky route end to end: cholVpr blocks -> gather_cholesky -> ccsdt_upload_cholesky
    (integral blocks built on the GPU) -> E[T], E(T) against the oracle on the same integrals; with
    EXACHEM_GB300_OVVV_SLABS the adapter takes the Cholesky-direct mode ((ia|bc) formed slab by slab
    into a cache of that many slabs) and must give the same energies."""
    import os
    import oracle
    exe = _compile(tmp_path, link_lib=True)
    o, v, ot, vt, ci = 8, 40, [4, 4], [16, 12, 12], [10, 14]
    d, L = _cholesky_case(o, v, sum(ci), 22)
    _write(tmp_path / "in.bin", d, ot, vt)
    _write_chol(tmp_path / "chol.bin", L, ci)
    env = {k: x for k, x in os.environ.items() if k != "EXACHEM_GB300_OVVV_SLABS"}
    if slabs:
        env["EXACHEM_GB300_OVVV_SLABS"] = slabs
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "--chol", str(tmp_path / "chol.bin"),
                    "--run"], check=True, env=env)
    nq = sum(ci)
    _, extra = _read(tmp_path / "out.bin", d, extra=(o * o + o * v + v * v) * nq + 2)
    e4, e5 = oracle.energy(d)
    assert rel_close(extra[-2], e4, 1e-12) and rel_close(extra[-1], e5, 1e-12)


SO_KEYS = ["eps_occ", "eps_vir", "t1", "t2", "v2ijab", "v2ijka", "v2iabc"]


def _so_allowed(oa, ob, va, vb):
    """Spin-allowed masks of t1 {V,O}, t2 {V,V,O,O}, v2ijab {O,O,V,V}, v2ijka {O,O,O,V},
    v2iabc {O,V,V,V}: the spins of the first half of the indices sum to those of the second."""
    so = np.array([0] * oa + [1] * ob)
    sv = np.array([0] * va + [1] * vb)

    def rule(*sp):
        g = np.meshgrid(*sp, indexing="ij")
        if len(g) == 2:
            return g[0] == g[1]
        return g[0] + g[1] == g[2] + g[3]
    return [rule(sv, so), rule(sv, sv, so, so), rule(so, so, sv, sv), rule(so, so, so, sv), rule(so, sv, sv, sv)]


def _write_so(path, tiles, arrs):
    with open(path, "wb") as f:
        dims = [sum(t) for t in tiles]
        np.array(dims + [len(t) for t in tiles] + [x for t in tiles for x in t], dtype=np.int32).tofile(f)
        np.concatenate([arrs[0], arrs[1]]).astype(np.float64).tofile(f)
        for a in arrs[2:]:
            np.ascontiguousarray(a, dtype=np.float64).tofile(f)


def _read_so(path, arrs, extra=0):
    raw = np.fromfile(path, dtype=np.float64)
    out, off = [], 0
    for a in arrs:
        out.append(raw[off:off + a.size].reshape(a.shape))
        off += a.size
    return out, raw[off:off + extra]


def test_adapter_open_shell_gather_is_exact(tmp_path, built):
    """gather_spin_orbital reads every spin-allowed block of the open-shell tensors bit for bit
    and never asks for a spin-forbidden one: the harness's tensors throw on such a get, as a
    block-sparse TAMM tensor has no such blocks (and their elements are NaN here besides)."""
    from oracle.spin_orbital_oracle import open_shell_system
    exe = _compile(tmp_path, link_lib=True)
    for (oa, ob, va, vb, tiles, seed) in [(3, 2, 5, 6, ([2, 1], [2], [3, 2], [4, 2]), 3),
                                          (4, 1, 3, 7, ([4], [1], [2, 1], [3, 3, 1]), 4)]:
        arrs = list(open_shell_system(oa, ob, va, vb, 5, seed))
        poisoned = arrs[:2] + [np.where(m, a, np.nan) for m, a in zip(_so_allowed(oa, ob, va, vb), arrs[2:])]
        _write_so(tmp_path / "so.bin", tiles, poisoned)
        subprocess.run([str(exe), "--so", str(tmp_path / "so.bin"), str(tmp_path / "out.bin")], check=True)
        got, _ = _read_so(tmp_path / "out.bin", arrs)
        for name, g, a in zip(SO_KEYS, got, arrs):
            assert np.array_equal(g, a), name


@pytest.mark.gpu
def test_adapter_open_shell_call_matches_oracle(tmp_path, built):
    """The open-shell drop-in end to end: tiled spin-orbital tensors -> gather_spin_orbital ->
    ccsdt_energy_spin_orbital -> E[T], E(T) against the spin-orbital oracle."""
    from oracle.spin_orbital_oracle import energy_spin_orbital, open_shell_system
    exe = _compile(tmp_path, link_lib=True)
    oa, ob, va, vb, tiles = 5, 3, 9, 11, ([3, 2], [3], [5, 4], [6, 5])
    arrs = list(open_shell_system(oa, ob, va, vb, 8, 31))
    _write_so(tmp_path / "so.bin", tiles, arrs)
    subprocess.run([str(exe), "--so", str(tmp_path / "so.bin"), str(tmp_path / "out.bin"), "--run"], check=True)
    _, extra = _read_so(tmp_path / "out.bin", arrs, extra=2)
    e4, e5 = energy_spin_orbital(*arrs)
    assert rel_close(extra[0], e4, 1e-12) and rel_close(extra[1], e5, 1e-12)


def test_adapter_reads_the_closed_shell_ccsd_amplitudes(tmp_path, built):
    """gather_cs_amplitudes takes the closed-shell CCSD's t1_aa {v_alpha, o_alpha} and t2_abab
    {v_alpha, v_beta, o_alpha, o_beta} (ccsd_util.cpp:550-575) as they are - no expansion to the
    spin-orbital d_t1 / d_t2 (cd_ccsd_cs_ann.cpp:932-975) - into the same spatial arrays."""
    from exachem_gb300.generator import generate
    exe = _compile(tmp_path, link_lib=True)
    o, v, ot, vt = 5, 11, [2, 3], [4, 4, 3]
    d = generate(o, v, 17)
    _write(tmp_path / "in.bin", d, ot, vt)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "--cs"], check=True)
    raw = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    off = 0
    for k in ["eps_occ", "eps_vir", "t1", "t2"]:
        got = raw[off:off + d[k].size].reshape(d[k].shape)
        off += d[k].size
        assert np.array_equal(got, d[k]), k


def test_adapter_execute_compiles_with_the_reference_signature(tmp_path, built):
    """CCSD_T_Fused_Driver<T>::execute - the drop-in itself, compiled only inside an ExaChem build
    (EXACHEM_GB300_WITH_TAMM) - compiles and links for T = double against stand-ins for the types
    of the reference's signature, restricted and open-shell branches included; and the options it
    reads from the environment (EXACHEM_GB300_MODE / SLICES / BUDGET / AUTOTUNE / GRAPH)."""
    exe = tmp_path / "execute_compile"
    lib = ROOT / "exachem_gb300" / "_build"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-Wno-unused-parameter",
                    str(ROOT / "tests" / "compat" / "execute_compile.cpp"), "-o", str(exe),
                    "-I", str(ROOT / "include"), "-I", str(ROOT / "oracle" / "ref_shim"),
                    "-L", str(lib), "-lccsdt_gb300", f"-Wl,-rpath,{lib}"], check=True, capture_output=True, text=True)
    subprocess.run([str(exe)], check=True)
    import os
    env = {k: v for k, v in os.environ.items() if not k.startswith("EXACHEM_GB300_")}

    def opts(**kw):
        out = subprocess.run([str(exe), "--opts"], check=True, capture_output=True, text=True,
                             env=env | {f"EXACHEM_GB300_{k}": v for k, v in kw.items()}).stdout.split()
        return int(out[0]), int(out[1]), float(out[2]), int(out[3]), int(out[4]), int(out[5])
    assert opts() == (0, 3, 1e-8, 1, 0, 0)                               # fp64 drop-in, autotune on, no graph
    assert opts(MODE="ozaki", SLICES="4", GRAPH="1") == (1, 4, 1e-8, 1, 1, 0)
    assert opts(MODE="learned", BUDGET="1e-9", AUTOTUNE="0") == (2, 5, 1e-9, 0, 0, 0)
    assert opts(MODE="ozaki", SLICES="2", P_STORAGE="ff")[5] == 1
    assert opts(MODE="ozaki", SLICES="2", P_STORAGE="f32")[5] == 2
    for bad in ({"EXACHEM_GB300_MODE": "int4"}, {"EXACHEM_GB300_P_STORAGE": "fp16"}):
        assert subprocess.run([str(exe), "--opts"], env=env | bad, capture_output=True).returncode != 0
