"""Generate tests/golden/xtc_golden.npz with the reference's own XTC codec.

The reference vendors GROMACS' xdrfile (coords_file/xdrfile) behind
CoordsFile::XtcHandler (coords_file/coords_file.cpp:70-126). Its sources are
compiled in place by ``make -C oracle ref`` into oracle/_ref/libentxdr.so;
this script writes small seeded trajectories with its write_xtc, as
XtcHandler::write calls it (step and time = the row, zero box, precision
1000, plus one file at another precision), and reads them back with its
read_xtc, as XtcHandler::next does. The fixture holds, per case, the input
rows, the file's bytes and the rows read back, so that the oracle, the
library's writer and its device decoder can be checked against the
reference where the reference sources are absent.

Usage:  python tests/golden/make_xtc_golden.py [--reference PATH]
"""
from __future__ import annotations

import argparse
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402


def water_box(rng, n_mol: int, box: float, n_frames: int, noise: float) -> np.ndarray:
    """Three-atom molecules (atoms 0.1 nm apart) in a box, jittered per frame."""
    o = rng.uniform(0, box, (n_mol, 1, 3))
    h = o + rng.normal(0, 0.06, (n_mol, 2, 3))
    base = np.concatenate([o, h], axis=1).reshape(-1, 3)
    return np.stack([(base + rng.normal(0, noise, base.shape)).reshape(-1)
                     for _ in range(n_frames)]).astype(np.float32)


def chain(rng, n_atoms: int, n_frames: int, step: float, noise: float) -> np.ndarray:
    """A random-walk chain (consecutive atoms ~step nm apart), jittered."""
    base = np.cumsum(rng.normal(0, step, (n_atoms, 3)), axis=0) + 3.0
    return np.stack([(base + rng.normal(0, noise, base.shape)).reshape(-1)
                     for _ in range(n_frames)]).astype(np.float32)


def clusters(rng, n_atoms: int, half: float, n_frames: int) -> np.ndarray:
    """Two clusters of atoms (1 nm wide) centred at -half and +half nm."""
    side = np.where(np.arange(n_atoms) < n_atoms // 2, -half, half)[:, None]
    base = side + rng.uniform(-0.5, 0.5, (n_atoms, 3))
    return np.stack([(base + rng.normal(0, 0.01, base.shape)).reshape(-1)
                     for _ in range(n_frames)]).astype(np.float32)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None,
                    help="reference checkout (default: $ENT_REFERENCE or ../reference)")
    args = ap.parse_args()
    if O.build_ref(args.reference) is None:
        raise SystemExit("reference sources not found")
    rng = np.random.default_rng(20261204)
    cases = {
        # water-like runs and run-length / table-index adaptation
        "water": (water_box(rng, 13, 2.5, 25, 0.02), 1000.0),
        # three atoms: raw floats, no compression
        "raw3": (rng.uniform(-4, 4, (6, 9)).astype(np.float32), 1000.0),
        # ten atoms: the smallest compressed frame
        "ten": (rng.uniform(0, 3, (6, 30)).astype(np.float32), 1000.0),
        # a chain: small steps between consecutive atoms, no water swaps
        "chain": (chain(rng, 400, 12, 0.15, 0.01), 1000.0),
        # ranges above 2^24 units (two clusters 40 km apart): one bit field
        # per coordinate
        "large": (clusters(rng, 50, 20000.0, 8), 1000.0),
        # another precision (write_xtc's argument; XtcHandler passes 1000)
        "prec10": (water_box(rng, 20, 4.0, 7, 0.05), 10.0),
    }
    g: dict[str, np.ndarray] = {}
    with tempfile.TemporaryDirectory() as d:
        for name, (rows, prec) in cases.items():
            path = f"{d}/{name}.xtc"
            O.ref_write_xtc(path, rows, prec)
            data = Path(path).read_bytes()
            g[f"{name}_in"] = rows
            g[f"{name}_prec"] = np.array([prec], np.float32)
            g[f"{name}_bytes"] = np.frombuffer(data, np.uint8).copy()
            g[f"{name}_out"] = O.ref_read_xtc(path, rows.shape[1] // 3)
        # a file cut inside its last frame: the reader stops before it
        cut = g["water_bytes"][: len(g["water_bytes"]) - 37]
        Path(f"{d}/cut.xtc").write_bytes(cut.tobytes())
        g["cut_bytes"] = cut
        g["cut_out"] = O.ref_read_xtc(f"{d}/cut.xtc", 39)
    np.savez_compressed(Path(__file__).with_name("xtc_golden.npz"), **g)
    print({k: v.shape for k, v in g.items()})


if __name__ == "__main__":
    main()
