"""The C++ drop-in of the reference's coordinate-file interface
(CoordsFile, coords_file/coords_file.hpp): one driver (tests/cpp/
coords_driver.cpp) is built against the shim and, where the reference sources
are present, against the reference's own coords_file.cpp with its vendored
xdrfile; both must read the same rows and write the same bytes. XTC reading
decodes on the GPU and is checked against the committed fixtures there."""
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT
from oracle import oracle as O

SHIM = ROOT / "entropical_gb300" / "shim"
LIB = ROOT / "entropical_gb300" / "lib"
DRIVER = ROOT / "tests" / "cpp" / "coords_driver.cpp"
REF = O.reference_dir()
GOLD = ROOT / "tests" / "golden" / "xtc_golden.npz"


def _build_shim_driver(td: Path) -> Path:
    from entropical_gb300 import _build
    _build.build()
    (td / "coords_file.hpp").write_text('#include "coords_file_gb300.hpp"\n')
    exe = td / "drv_shim"
    subprocess.run(["g++", "-std=c++14", "-O1", str(DRIVER), "-I", str(td), "-I", str(SHIM),
                    "-I", str(ROOT / "include"), "-L", str(LIB), "-lentropical_shim",
                    "-lentropical_gb300", f"-Wl,-rpath,{LIB}", "-o", str(exe)], check=True)
    return exe


def _build_ref_driver(td: Path) -> Path:
    xdr = REF / "coords_file" / "xdrfile"
    objs = []
    for c in ("xdrfile.c", "xdrfile_xtc.c", "xdrfile_trr.c"):
        o = td / (c + ".o")
        subprocess.run(["gcc", "-O1", "-w", "-c", str(xdr / c), "-o", str(o)], check=True)
        objs.append(str(o))
    exe = td / "drv_ref"
    subprocess.run(["g++", "-std=c++11", "-O1", "-w", str(DRIVER), str(REF / "coords_file" /
                    "coords_file.cpp"), "-I", str(REF / "coords_file"), *objs, "-o", str(exe)],
                   check=True)
    return exe


def _write_rows(path: Path, rows: np.ndarray) -> None:
    rows = np.ascontiguousarray(rows, np.float32)
    with open(path, "wb") as f:
        f.write(struct.pack("ii", *rows.shape))
        f.write(rows.tobytes())


def _read_rows(path: Path) -> list:
    b = path.read_bytes()
    n = struct.unpack_from("i", b, 0)[0]
    off, out = 4, []
    for _ in range(n):
        ln = struct.unpack_from("i", b, off)[0]
        off += 4
        out.append(np.frombuffer(b, np.float32, ln, off).copy())
        off += 4 * ln
    return out


def _run(exe: Path, *args) -> None:
    subprocess.run([str(exe), *map(str, args)], check=True)


@pytest.fixture(scope="module")
def drivers(tmp_path_factory):
    td = tmp_path_factory.mktemp("coords_drv")
    shim = _build_shim_driver(td)
    ref = _build_ref_driver(td) if REF is not None and (REF / "coords_file").exists() else None
    return shim, ref


def _rows_equal(got, want) -> bool:
    return [r.tobytes() for r in got] == [np.asarray(w, np.float32).tobytes() for w in want]


def test_ascii_rows(drivers, tmp_path):
    shim, ref = drivers
    src = tmp_path / "c.txt"
    # an empty line, a trailing space, no line break after the last line
    src.write_text("1 2 3\n\n4.5 -6 7e-3 \n8 9")
    _run(shim, "read", src, tmp_path / "s.bin")
    got = _read_rows(tmp_path / "s.bin")
    # the reference's rules: empty lines are skipped, whitespace after the
    # last value repeats it, the last line without a line break is dropped
    assert _rows_equal(got, [[1, 2, 3], [4.5, -6, 7e-3, 7e-3]])
    if ref is not None:
        _run(ref, "read", src, tmp_path / "r.bin")
        assert [r.tobytes() for r in got] == [r.tobytes() for r in _read_rows(tmp_path / "r.bin")]
    # a line of blanks: one read that finds nothing (T() here; the reference
    # reads an uninitialised variable there)
    src.write_text("   \n1\n")
    _run(shim, "read", src, tmp_path / "s.bin")
    assert _rows_equal(_read_rows(tmp_path / "s.bin"), [[0], [1]])


def test_ascii_write(drivers, tmp_path):
    shim, ref = drivers
    rows = np.array([[1, 2.5, -3], [1e-7, 123456789, 0.1]], np.float32)
    _write_rows(tmp_path / "in.bin", rows)
    _run(shim, "write", tmp_path / "in.bin", tmp_path / "s.txt")
    assert (tmp_path / "s.txt").read_text() == " 1 2.5 -3\n 1e-07 1.23457e+08 0.1\n"
    if ref is not None:
        _run(ref, "write", tmp_path / "in.bin", tmp_path / "r.txt")
        assert (tmp_path / "s.txt").read_bytes() == (tmp_path / "r.txt").read_bytes()


def test_xtc_write_equals_reference(drivers, tmp_path):
    shim, ref = drivers
    g = np.load(GOLD)
    rows = g["water_in"]
    _write_rows(tmp_path / "in.bin", rows)
    _run(shim, "write", tmp_path / "in.bin", tmp_path / "s.xtc")
    assert (tmp_path / "s.xtc").read_bytes() == g["water_bytes"].tobytes()
    if ref is not None:
        _run(ref, "write", tmp_path / "in.bin", tmp_path / "r.xtc")
        assert (tmp_path / "s.xtc").read_bytes() == (tmp_path / "r.xtc").read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["water", "raw3", "chain", "cut"])
def test_xtc_read_through_shim(drivers, tmp_path, case):
    shim, _ = drivers
    g = np.load(GOLD)
    src = tmp_path / f"{case}.xtc"
    src.write_bytes(g[f"{case}_bytes"].tobytes())
    _run(shim, "read", src, tmp_path / "s.bin")
    got = _read_rows(tmp_path / "s.bin")
    want = g[f"{case}_out"]
    assert len(got) == want.shape[0]
    assert all(np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in zip(got, want))
