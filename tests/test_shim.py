"""The C++ drop-in shim keeps the reference's density interface: the
reference's own estimator sources compile and link against it unchanged
(CPU, where the reference sources are present), and a driver calling it the
way mi.cpp does reproduces the reference's MI output (GPU)."""
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT

from oracle import oracle as O  # noqa: E402

REF = O.reference_dir() or Path("reference-sources-not-present")
SHIM = ROOT / "entropical_gb300" / "shim"
LIB = ROOT / "entropical_gb300" / "lib"


def _build_lib():
    from entropical_gb300 import _build
    _build.build()


@pytest.mark.skipif(not (REF / "mi.cpp").exists(), reason="reference sources not present")
def test_reference_estimators_link_against_shim():
    _build_lib()
    with tempfile.TemporaryDirectory() as td:
        # the reference includes "densities_cuda.hpp"; point it at the shim
        Path(td, "densities_cuda.hpp").write_text('#include "densities_gb300.hpp"\n')
        objs = []
        for src in ["mi.cpp", "transs.cpp", "autoent.cpp", "kldiv.cpp", "negs.cpp", "dens.cpp",
                    "hestimate.cpp", "tools.cpp"]:
            o = Path(td, src + ".o")
            defs = [] if src == "hestimate.cpp" else ["-DUSE_CUDA"]
            subprocess.run(["g++", "-std=c++11", "-O1", "-fPIC", "-w", *defs, "-include", "cmath",
                            "-I", td, "-I", str(SHIM), "-I", str(ROOT / "oracle" / "stub"),
                            "-I", str(REF), "-c", str(REF / src), "-o", str(o)], check=True)
            objs.append(str(o))
        subprocess.run(["g++", "-shared", "-o", str(Path(td, "libestimators.so"), ), *objs,
                        "-L", str(LIB), "-lentropical_shim", "-lentropical_gb300",
                        "-Wl,--no-undefined", "-fopenmp"], check=True)


@pytest.mark.gpu
def test_mi_driver_matches_reference(golden):
    _build_lib()
    with tempfile.TemporaryDirectory() as td:
        exe = Path(td, "mi_driver")
        subprocess.run(["g++", "-std=c++14", "-O2", str(ROOT / "tests" / "cpp" / "mi_driver.cpp"),
                        "-I", str(SHIM), "-I", str(ROOT / "include"), "-L", str(LIB),
                        "-lentropical_shim", "-lentropical_gb300", f"-Wl,-rpath,{LIB}",
                        "-o", str(exe)], check=True)
        x = golden["est_x"].astype(np.float32)
        h = golden["est_h"].astype(np.float32)
        fin, fout = Path(td, "in.bin"), Path(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([x.shape[1], x.shape[0]], np.int32).tofile(f)
            x.tofile(f)
            h.tofile(f)
        subprocess.run([str(exe), str(fin), str(fout)], check=True)
        mi = np.fromfile(fout, np.float32).reshape(x.shape[0], x.shape[0])
        ref = golden["est_mi"]
        # the reference prints 6 significant digits
        assert np.allclose(mi, ref, rtol=2e-5, atol=1e-5)


def _build_abi_driver(td) -> Path:
    _build_lib()
    exe = Path(td, "abi_driver")
    subprocess.run(["g++", "-std=c++14", "-O2", "-Wall", "-Werror",
                    str(ROOT / "tests" / "cpp" / "abi_driver.cpp"), "-I", str(ROOT / "include"),
                    "-L", str(LIB), "-lentropical_gb300", f"-Wl,-rpath,{LIB}", "-o", str(exe)],
                   check=True)
    return exe


def test_abi_driver_compiles():
    """The C header is usable from C++ as a plain C ABI (no CUDA headers)."""
    with tempfile.TemporaryDirectory() as td:
        assert _build_abi_driver(td).exists()


@pytest.mark.gpu
def test_abi_driver_matches_python_path(golden):
    """C++ through the C ABI: file reader, autotuner, the reference's MI formula
    and the resubstitution MI batch give the Python mirror's numbers and the
    reference's MI output."""
    from entropical_gb300 import Context
    from entropical_gb300.densities import REF_MI
    x = golden["est_x"].astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        exe = _build_abi_driver(td)
        txt = Path(td, "coords.txt")
        np.savetxt(txt, x.T, fmt="%.9g")
        out = Path(td, "out.bin")
        subprocess.run([str(exe), str(txt), "0.4", str(out)], check=True)
        v = np.fromfile(out, np.float64)
        m = int(v[0])
        mi_ref = v[1:1 + m * m].reshape(m, m)
        mi = v[1 + m * m:1 + 2 * m * m].reshape(m, m)
        hx = v[1 + 2 * m * m:]
    h = np.full(m, 0.4, np.float32)
    with Context(0) as ctx:
        # the formula's float log of a density ratio moves by an ulp when the
        # FP32 partial sums differ (the C++ context is autotuned): 1e-6 relative
        assert np.allclose(mi_ref, ctx.reference_estimator(x, h, REF_MI), rtol=1e-6, atol=1e-9)
        mi_p, hx_p = ctx.mi_all_pairs(x, h)
        assert np.allclose(mi, mi_p, atol=1e-7) and np.allclose(hx, hx_p, atol=1e-7)
