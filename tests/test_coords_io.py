"""Coordinate files in the reference's ASCII format: the parallel loader
(ent_read_coords) against the reference's own Tools::IO::read_coords
(tools.hxx:153-235, compiled in place; skipped where the reference sources
are absent) and against the values written. Bit-exact: both parse decimal
text to the correctly rounded float."""
import os

import numpy as np
import pytest

from entropical_gb300 import NativeError, coords_file_shape, read_coords
from oracle import oracle as O


def _have_ref() -> bool:
    try:
        O.ref()
        return True
    except Exception:
        return False


HAVE_REF = _have_ref()


def write(path, text: str) -> str:
    with open(path, "w", newline="") as f:
        f.write(text)
    return str(path)


def matrix_text(x: np.ndarray, fmt: str, sep: str = " ", eol: str = "\n") -> str:
    return eol.join(sep.join(fmt % v for v in row) for row in x.T) + eol


@pytest.mark.parametrize("fmt,sep,eol", [("%.9g", " ", "\n"), ("%.6e", "\t", "\n"),
                                         ("%.3f", "   ", "\r\n"), ("%.17g", " ", "\n")])
def test_matches_values_and_reference(tmp_path, fmt, sep, eol):
    rng = np.random.default_rng(len(fmt) + len(sep))
    x = (rng.standard_normal((5, 777)) * 10 ** rng.uniform(-3, 3, (5, 1))).astype(np.float32)
    if fmt == "%.17g":  # doubles between floats: the parser rounds each to float
        x = x.astype(np.float64) * (1 + 1e-9 * rng.standard_normal(x.shape))
    p = write(tmp_path / "c.txt", matrix_text(x, fmt, sep, eol))
    y = read_coords(p)
    expect = np.array([[np.float32(float(fmt % v)) for v in row] for row in x], np.float32)
    assert y.shape == (5, 777)
    assert np.array_equal(y, expect)
    assert coords_file_shape(p) == (777, 5)
    if HAVE_REF:
        assert np.array_equal(y, O.ref_read_coords(p, "C"))
        assert np.array_equal(read_coords(p, primary="R"), O.ref_read_coords(p, "R"))


def test_usecols_blank_lines_and_spacing(tmp_path):
    text = "\n\n  1.5  -2e3\t+3.25 4\n\n5 6 7 8   \n9 10 11 12"  # no final newline
    p = write(tmp_path / "c.txt", text)
    assert coords_file_shape(p) == (3, 4)
    y = read_coords(p, usecols=[3, 0])  # the file's order is kept
    assert np.array_equal(y, np.array([[1.5, 5, 9], [4, 8, 12]], np.float32))
    r = read_coords(p, usecols=[1, 2], primary="R")
    assert np.array_equal(r, np.array([[-2000, 3.25], [6, 7], [10, 11]], np.float32))
    if HAVE_REF:
        assert np.array_equal(y, O.ref_read_coords(p, "C", [3, 0]))
        assert np.array_equal(r, O.ref_read_coords(p, "R", [1, 2]))


def test_errors(tmp_path):
    with pytest.raises(NativeError) as e:
        read_coords(str(tmp_path / "missing.txt"))
    assert e.value.status == 11
    p = write(tmp_path / "ragged.txt", "1 2 3\n4 5\n")
    with pytest.raises(NativeError) as e:
        read_coords(p)
    assert e.value.status == 11 and "row 2" in str(e.value)
    p = write(tmp_path / "nan.txt", "1 2\n3 x\n")
    with pytest.raises(NativeError) as e:
        read_coords(p)
    assert e.value.status == 11
    p = write(tmp_path / "ok.txt", "1 2\n3 4\n")
    with pytest.raises(NativeError) as e:
        read_coords(p, usecols=[2])
    assert e.value.status == 4


def test_large_file_parallel_parse(tmp_path):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((3, 200_000)).astype(np.float32)
    p = str(tmp_path / "big.txt")
    np.savetxt(p, x.T, fmt="%.9g")
    y = read_coords(p)
    assert np.array_equal(y, x)
    assert os.path.getsize(p) > 4_000_000


def test_empty_and_blank_files(tmp_path):
    assert coords_file_shape(write(tmp_path / "e.txt", "")) == (0, 0)
    assert coords_file_shape(write(tmp_path / "b.txt", "\n\n\n")) == (0, 0)
    assert read_coords(str(tmp_path / "e.txt")).shape == (0, 0)


def test_large_file_ragged_layout(tmp_path):
    """Many threads' byte ranges over CRLF lines, runs of blank lines and a
    last line without a line break: the same rows as the values written."""
    rng = np.random.default_rng(11)
    x = rng.standard_normal((4, 60_000)).astype(np.float32)
    rows = [" ".join("%.9g" % v for v in r) for r in x.T]
    parts = []
    for i, r in enumerate(rows):
        parts.append(r)
        parts.append("\r\n" + ("\n" * int(i % 97 == 0)))
    text = "".join(parts).rstrip("\r\n")  # no final line break
    p = write(tmp_path / "big.txt", text)
    assert coords_file_shape(p) == (60_000, 4)
    assert np.array_equal(read_coords(p), x)
    assert np.array_equal(read_coords(p, usecols=[2], primary="R")[:, 0], x[2])


def test_stream_without_size(tmp_path):
    """A file that cannot be mapped (a FIFO) is read as a stream."""
    import threading
    fifo = tmp_path / "c.fifo"
    os.mkfifo(fifo)
    text = "".join(f"{i} {i + 0.5} {-i}\n" for i in range(50_000))

    def writer():
        with open(fifo, "w") as f:
            f.write(text)

    th = threading.Thread(target=writer, daemon=True)
    th.start()
    assert coords_file_shape(str(fifo)) == (50_000, 3)
    th.join(timeout=30)
    assert not th.is_alive()


def test_values_beyond_float_range(tmp_path):
    """Values below the float range read as (signed) zero or the subnormal
    strtof gives, however they are spelled; the reference's `ifs >> float`
    reads the same. Values above it saturate to infinity as strtof does (the
    reference stores FLT_MAX there and reads nothing after it)."""
    z50 = "0." + "0" * 50 + "1"
    p = write(tmp_path / "tiny.txt", f"{z50} -{z50} 1e-50 -1e-50\n.00001e-45 1e-40 8e-46 0.5\n")
    y = read_coords(p, primary="R")
    assert np.array_equal(y.view(np.uint32), np.array(
        [[0.0, -0.0, 0.0, -0.0], [0.0, np.float32(1e-40), np.float32(1.4e-45), 0.5]],
        np.float32).view(np.uint32))
    if HAVE_REF:
        assert np.array_equal(y.view(np.uint32), O.ref_read_coords(p, "R").view(np.uint32))
    p = write(tmp_path / "huge.txt", "1e39 -1e39 " + "9" * 42 + " 0.0001e50\n")
    assert np.array_equal(read_coords(p, primary="R"),
                          np.array([[np.inf, -np.inf, np.inf, np.inf]], np.float32))
