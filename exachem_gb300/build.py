"""Builds the in-tree shared library exachem_gb300/_build/libccsdt_gb300.so with nvcc
(sm_103a only) and, for tests, the CPU oracle under oracle/."""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libccsdt_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

CU_SOURCES = ["ccsdt_capi.cu", "split.cu", "persist.cu", "noalloc.cu", "mlp.cu", "learned.cu", "retile.cu",
              "cholesky.cu", "pz_launch_a.cu", "pz_launch_b.cu", "pz_launch_c.cu", "spin_orbital.cu"]
CPP_SOURCES = ["refcount.cpp"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def sources() -> list[Path]:
    out = []
    for s in CU_SOURCES + CPP_SOURCES:
        p = CSRC / s
        if p.exists():
            out.append(p)
    return out


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "ccsdt.h"]
    srcs = sources()
    nvcc = _nvcc()
    objs, jobs = [], []
    for s in srcs:
        o = BUILD / (s.name + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            if s.suffix == ".cu":
                cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
            else:
                cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-c", str(s), "-o", str(o)]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                sys.stdout.write(r.stdout + r.stderr)
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    return LIB


def build_oracle(reference: str | None = None) -> None:
    """The oracle is test infrastructure: the C restatement always, and the reference's
    own CPU (T) (oracle/_ref) only where the reference tree is present."""
    oracle = ROOT / "oracle"
    _run(["make", "-C", str(oracle), "port"])
    ref = reference or os.environ.get("CCSDT_REFERENCE")
    if not ref:
        print("oracle/_ref not rebuilt: CCSDT_REFERENCE (the reference source tree) is not set", file=sys.stderr)
    elif os.path.isdir(os.path.join(ref, "exachem", "cc", "ccsd_t")):
        _run(["make", "-C", str(oracle), "ref", f"REFERENCE={ref}"])
    else:
        print(f"oracle/_ref not rebuilt: {ref} holds no exachem/cc/ccsd_t", file=sys.stderr)


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
    build_oracle()
