"""In-tree native build of the entropical GB300 library (sm_103a only).

Compiles every ``csrc/*.cu`` translation unit with nvcc in parallel and links
``lib/libentropical_gb300.so``; compiles the C++ drop-in shim
(``shim/densities_gb300.cpp``, ``shim/coords_file_gb300.cpp``) into ``lib/libentropical_shim.so``. No cmake,
no torch extension machinery: plain nvcc/g++ invocations, so the same recipe
runs on the x86_64 build host and on the aarch64 GPU hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
OBJ = LIB / "obj"
SHIM = PKG / "shim"
ROOT = PKG.parent
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]

LIB_NAME = "libentropical_gb300.so"
SHIM_NAME = "libentropical_shim.so"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the entropical GB300 library needs the CUDA toolkit")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def lib_path() -> Path:
    return LIB / LIB_NAME


def shim_path() -> Path:
    return LIB / SHIM_NAME


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the CUDA library (and the C++ shim); return the library path."""
    nvcc = _nvcc()
    OBJ.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "entropical_gb300.h"]
    sources = sorted(CSRC.glob("*.cu"))
    jobs = []
    for src in sources:
        obj = OBJ / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    objs = [OBJ / (s.stem + ".o") for s in sources]
    out = lib_path()
    if force or _stale(out, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart"])
    shim_srcs = [SHIM / "densities_gb300.cpp", SHIM / "coords_file_gb300.cpp"]
    if all(p.exists() for p in shim_srcs):
        sout = shim_path()
        deps = [*shim_srcs, SHIM / "densities_gb300.hpp", SHIM / "coords_file_gb300.hpp",
                INCLUDE / "entropical_gb300.h", out]
        if force or _stale(sout, deps):
            _run(["g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-I", str(INCLUDE), "-I", str(SHIM),
                  *map(str, shim_srcs), "-o", str(sout), "-L", str(LIB), "-lentropical_gb300",
                  "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", out)
    return out
