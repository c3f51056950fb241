"""XTC trajectories, host side: the oracle's reader (xtc_oracle.c) and the
library's writer and file index (ent_write_xtc, ent_xtc_file_shape) against
the reference's own codec -- its vendored xdrfile behind
CoordsFile::XtcHandler (coords_file/coords_file.cpp:70-126) -- through the
committed fixtures (tests/golden/xtc_golden.npz, made by
tests/golden/make_xtc_golden.py) and, where the reference sources are
present, the codec compiled in place (oracle/_ref/libentxdr.so).

Bit-exact throughout: the reader's floats, the writer's bytes."""
from pathlib import Path

import numpy as np
import pytest

from entropical_gb300 import NativeError, coords_file_shape, is_xtc, write_xtc, xtc_file_shape
from oracle import oracle as O

GOLD = Path(__file__).resolve().parent / "golden" / "xtc_golden.npz"
CASES = ["water", "raw3", "ten", "chain", "large", "prec10"]


@pytest.fixture(scope="module")
def xg():
    return dict(np.load(GOLD, allow_pickle=False))


def _file(tmp_path, name, data: np.ndarray) -> str:
    p = tmp_path / f"{name}.xtc"
    p.write_bytes(data.tobytes())
    return str(p)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("case", CASES + ["cut"])
def test_oracle_reads_reference_files(xg, tmp_path, case):
    p = _file(tmp_path, case, xg[f"{case}_bytes"])
    want = xg[f"{case}_out"]
    assert O.xtc_shape(p) == (want.shape[0], want.shape[1] // 3)
    assert np.array_equal(_bits(O.read_xtc(p)), _bits(want))
    # a frame range, as the CPU baseline samples it
    if want.shape[0] > 3:
        assert np.array_equal(_bits(O.read_xtc(p, 1, 3)), _bits(want[1:3]))


@pytest.mark.parametrize("case", CASES)
def test_writer_bytes_equal_reference(xg, tmp_path, case):
    p = str(tmp_path / f"{case}.xtc")
    write_xtc(p, xg[f"{case}_in"].T.copy(), float(xg[f"{case}_prec"][0]))
    assert Path(p).read_bytes() == xg[f"{case}_bytes"].tobytes()


@pytest.mark.parametrize("case", CASES + ["cut"])
def test_file_index(xg, tmp_path, case):
    p = _file(tmp_path, case, xg[f"{case}_bytes"])
    want = xg[f"{case}_out"].shape
    assert xtc_file_shape(p) == want
    assert coords_file_shape(p) == want  # the ".xtc" name picks the XTC index


def test_names():
    # CoordsFile::open: longer than four characters and ending in ".xtc"
    assert is_xtc("a.xtc") and is_xtc("/x/traj.xtc")
    assert not is_xtc(".xtc") and not is_xtc("a.xtc.txt") and not is_xtc("a.XTC")


def test_writer_refusals(tmp_path):
    p = str(tmp_path / "bad.xtc")
    x = np.zeros((30, 4), np.float32)
    x[4, 1] = np.nan
    with pytest.raises(NativeError, match="non-finite"):
        write_xtc(p, x)
    with pytest.raises(NativeError, match="too large"):
        write_xtc(p, np.full((30, 2), 3.0e6, np.float32))  # 3e9 units at precision 1000
    with pytest.raises(NativeError, match="multiple of 3"):
        write_xtc(p, np.zeros((31, 2), np.float32))
    far = np.zeros((30, 2), np.float32)
    far[:, 0] = np.arange(30) * 5000.0  # consecutive atoms 5 km apart
    with pytest.raises(NativeError, match="too far apart"):
        write_xtc(p, far)


def test_index_stops_at_first_bad_frame(xg, tmp_path):
    data = bytearray(xg["water_bytes"].tobytes())
    # second frame's magic broken: one frame remains, as XtcHandler::next
    # reports the end at the first failing read_xtc
    first = 92 + ((int.from_bytes(data[88:92], "big") + 3) & ~3)
    data[first:first + 4] = (1996).to_bytes(4, "big")
    p = tmp_path / "one.xtc"
    p.write_bytes(bytes(data))
    assert xtc_file_shape(str(p)) == (1, 117)
    assert O.xtc_shape(str(p)) == (1, 39)
    with pytest.raises(NativeError):
        xtc_file_shape(str(tmp_path / "missing.xtc"))
    q = tmp_path / "junk.xtc"
    q.write_bytes(b"\0" * 200)
    with pytest.raises(NativeError, match="no XTC frame"):
        xtc_file_shape(str(q))


def _trajectory(rng, kind: str, n_atoms: int, n_frames: int, scale: float) -> np.ndarray:
    if kind == "water":
        n_mol = n_atoms // 3
        o = rng.uniform(0, scale, (n_mol, 1, 3))
        base = np.concatenate([o, o + rng.normal(0, 0.06, (n_mol, 2, 3))], 1).reshape(-1, 3)
    elif kind == "chain":
        base = np.cumsum(rng.normal(0, 0.15, (n_atoms, 3)), 0)
    else:
        base = rng.uniform(-scale, scale, (n_atoms, 3))
    noise = rng.choice([0.0, 0.001, 0.03])
    return np.stack([(base + rng.normal(0, noise, base.shape)).reshape(-1)
                     for _ in range(n_frames)]).astype(np.float32)


@pytest.mark.skipif(not O.xdr_available(), reason="reference sources absent (make -C oracle ref)")
@pytest.mark.parametrize("seed", range(6))
def test_against_reference_codec(tmp_path, seed):
    """Random trajectories: the library's writer gives the reference writer's
    bytes, and the oracle reads them as the reference reader does."""
    rng = np.random.default_rng(100 + seed)
    for kind, n_atoms, scale in [("water", 3 * int(rng.integers(4, 60)), 3.0),
                                 ("chain", int(rng.integers(10, 300)), 0.0),
                                 ("uniform", int(rng.integers(1, 40)),
                                  float(rng.choice([0.01, 5.0, 900.0])))]:
        rows = _trajectory(rng, kind, n_atoms, int(rng.integers(1, 9)), scale)
        pr, pm = str(tmp_path / "r.xtc"), str(tmp_path / "m.xtc")
        O.ref_write_xtc(pr, rows)
        write_xtc(pm, rows.T.copy())
        assert Path(pm).read_bytes() == Path(pr).read_bytes(), (kind, n_atoms)
        assert np.array_equal(_bits(O.read_xtc(pm)), _bits(O.ref_read_xtc(pr, n_atoms)))


def test_writer_row_major_input(xg, tmp_path):
    """primary 'R' (one row per frame) writes the same bytes as the
    column-major input."""
    rows = xg["water_in"]
    pc, pr = str(tmp_path / "c.xtc"), str(tmp_path / "r.xtc")
    write_xtc(pc, rows.T.copy())
    write_xtc(pr, rows, primary="R")
    assert Path(pr).read_bytes() == Path(pc).read_bytes() == xg["water_bytes"].tobytes()
    with pytest.raises(ValueError):
        write_xtc(pr, rows, primary="X")
