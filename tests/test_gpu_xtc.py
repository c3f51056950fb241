"""XTC trajectories decoded on the device (ent_read_xtc, ent_load_xtc_device:
a walk over each frame's atom groups, then one thread per 64-atom segment,
straight into the column-major coordinate matrix)
against the reference's own reader (XtcHandler::next over the vendored
xdrfile, coords_file/coords_file.cpp:90-110) through the committed fixtures,
and against the oracle's reader on larger trajectories. Bit-exact."""
from pathlib import Path

import numpy as np
import pytest

from entropical_gb300 import NativeError, write_xtc, xtc_file_shape
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "xtc_golden.npz"
CASES = ["water", "raw3", "ten", "chain", "large", "prec10", "cut"]


@pytest.fixture(scope="module")
def xg():
    return dict(np.load(GOLD, allow_pickle=False))


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _file(tmp_path, name, data) -> str:
    p = tmp_path / f"{name}.xtc"
    p.write_bytes(bytes(data))
    return str(p)


@pytest.mark.parametrize("case", CASES)
def test_device_reader_matches_reference(ctx, xg, tmp_path, case):
    p = _file(tmp_path, case, xg[f"{case}_bytes"].tobytes())
    want = xg[f"{case}_out"]  # rows: frames
    assert np.array_equal(_bits(ctx.read_xtc(p, primary="R")), _bits(want))
    assert np.array_equal(_bits(ctx.read_xtc(p)), _bits(want.T))
    st = ctx.last_stats()
    assert st.kernel_launches == 2 and st.instances == want.shape[0]  # walk + decode


def test_selected_columns_and_device_load(ctx, xg, tmp_path):
    torch = pytest.importorskip("torch")
    p = _file(tmp_path, "water", xg["water_bytes"].tobytes())
    want = xg["water_out"].T  # (columns, frames)
    cols = [100, 3, 3, 116, 0, 57]  # the file's order, duplicates once
    keep = sorted(set(cols))
    assert np.array_equal(_bits(ctx.read_xtc(p, cols)), _bits(want[keep]))
    assert np.array_equal(_bits(ctx.read_xtc(p, cols, primary="R")), _bits(want[keep].T))
    dev = torch.full((117, want.shape[1]), -1.0, dtype=torch.float32, device="cuda")
    # a ".xtc" name sends load_coords_device to the XTC decoder
    n_rows, n_cols = ctx.load_coords_device(p, dev.data_ptr())
    torch.cuda.synchronize()
    assert (n_cols, n_rows) == want.shape
    assert np.array_equal(_bits(dev.cpu().numpy()), _bits(want))
    with pytest.raises(NativeError):
        ctx.read_xtc(p, [117])


def _water(rng, n_mol, n_frames, box=4.0, noise=0.02):
    o = rng.uniform(0, box, (n_mol, 1, 3))
    base = np.concatenate([o, o + rng.normal(0, 0.06, (n_mol, 2, 3))], 1).reshape(-1, 3)
    return np.stack([(base + rng.normal(0, noise, base.shape)).reshape(-1)
                     for _ in range(n_frames)]).astype(np.float32)


@pytest.mark.parametrize("kind", ["water", "chain", "mixed", "few_frames"])
def test_larger_trajectories_match_oracle(ctx, tmp_path, kind):
    """Thousands of frames (many warps, lanes of a warp diverging in their
    run structure) written by the library's writer; the device reader equals
    the oracle's reader frame for frame."""
    rng = np.random.default_rng({"water": 1, "chain": 2, "mixed": 3, "few_frames": 4}[kind])
    if kind == "water":
        rows = _water(rng, 150, 3000)
    elif kind == "chain":
        base = np.cumsum(rng.normal(0, 0.15, (700, 3)), 0)
        rows = np.stack([(base + rng.normal(0, 0.02, base.shape)).reshape(-1)
                         for _ in range(1500)]).astype(np.float32)
    elif kind == "few_frames":
        # many atoms in few frames: hundreds of decoding segments per frame
        rows = _water(rng, 10_000, 5, box=8.0)
    else:  # protein-like chain plus water, frames drifting apart
        w = _water(rng, 60, 2000, noise=0.05)
        base = np.cumsum(rng.normal(0, 0.15, (120, 3)), 0)
        drift = np.cumsum(rng.normal(0, 0.01, (2000, 1, 3)), 0)
        c = (base[None] + drift + rng.normal(0, 0.02, (2000, 120, 3))).reshape(2000, -1)
        rows = np.concatenate([c.astype(np.float32), w], axis=1)
    p = str(tmp_path / f"{kind}.xtc")
    write_xtc(p, rows.T.copy())
    assert xtc_file_shape(p) == rows.shape
    got = ctx.read_xtc(p, primary="R")
    assert np.array_equal(_bits(got), _bits(O.read_xtc(p)))
    # quantised to the precision: within half a unit (plus float rounding)
    assert np.max(np.abs(got - rows)) <= 0.5e-3 + 1e-6 * np.max(np.abs(rows))


def _patched(xg, at: int, value: int) -> bytes:
    data = bytearray(xg["ten_bytes"].tobytes())
    data[at:at + 4] = int(value).to_bytes(4, "big", signed=True)
    return bytes(data)


def test_malformed_frames_are_errors(ctx, xg, tmp_path):
    """Malformed compressed frames end the call with ENT_ERR_IO naming the
    frame; every read stays inside the frame and every write inside the
    output, so the context stays usable."""
    # table index outside the format (smallidx, byte offset 84 of frame 0)
    with pytest.raises(NativeError, match="frame 0: small-integer table index"):
        ctx.read_xtc(_file(tmp_path, "idx", _patched(xg, 84, 80)))
    # an empty coordinate range (maxint below minint by one: size 0)
    data = _patched(xg, 72, int.from_bytes(xg["ten_bytes"][60:64].tobytes(), "big",
                                           signed=True) - 1)
    with pytest.raises(NativeError, match="frame 0: empty or 32-bit coordinate range"):
        ctx.read_xtc(_file(tmp_path, "rng", data))
    # flipped bits inside the compressed data: an error or some values, never
    # a fault; the next call decodes a good file exactly
    rng = np.random.default_rng(7)
    good = xg["water_bytes"].tobytes()
    n_bytes = int.from_bytes(good[88:92], "big")
    for _ in range(20):
        data = bytearray(good)
        for k in rng.integers(92, 92 + n_bytes, 3):
            data[k] ^= 1 << int(rng.integers(0, 8))
        try:
            ctx.read_xtc(_file(tmp_path, "flip", data))
        except NativeError as e:
            assert e.status == 11
    p = _file(tmp_path, "good", good)
    assert np.array_equal(_bits(ctx.read_xtc(p, primary="R")), _bits(xg["water_out"]))
