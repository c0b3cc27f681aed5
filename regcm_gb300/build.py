"""Build the in-tree libraries: libmoloch_gb300.so (CUDA, sm_103a) and the CPU
oracle used by the tests.  Translation units compile in parallel; outputs go
to regcm_gb300/_build/ and oracle/_build/ (both git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fno-fast-math", "-ffp-contract=off"]

CU_SOURCES = ["mlc_sound.cu", "mlc_advect.cu", "mlc_end.cu", "mlc_context.cu", "mlc_noalloc.cu",
              "mlc_peak.cu"]
CPP_SOURCES = ["mlc_setup.cpp", "mlc_restart.cpp"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False, extra_nvcc=(), out_name: str = "libmoloch_gb300.so") -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    tag = "" if out_name == "libmoloch_gb300.so" else Path(out_name).stem + "_"
    jobs = []
    for src in CU_SOURCES:
        obj = OUT / (tag + src.replace(".cu", ".o"))
        if _stale(obj, [CSRC / src, *headers, Path(__file__)]):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *extra_nvcc, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = OUT / (tag + src.replace(".cpp", ".o"))
        if _stale(obj, [CSRC / src, *headers, Path(__file__)]):
            jobs.append(["g++", *CXX_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            if lg.strip():
                print(lg)
    objs = [OUT / (tag + s.replace(".cu", ".o")) for s in CU_SOURCES] + \
           [OUT / (tag + s.replace(".cpp", ".o")) for s in CPP_SOURCES]
    lib = OUT / out_name
    if _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    return lib


def build_oracle() -> Path:
    _run(["make", "-s", "-C", str(ORACLE)])
    return ORACLE / "_build" / "libmoloch_oracle.so"


def build_all(verbose: bool = False):
    lib = build_library(verbose=verbose)
    orc = build_oracle()
    return lib, orc


if __name__ == "__main__":
    lib, orc = build_all(verbose="-v" in sys.argv)
    print(lib)
    print(orc)
