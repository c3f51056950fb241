"""Host mirror of the reference density interface over the C ABI.

``combined_densities`` keeps the reference's name, argument order and meaning
(densities_cuda.hpp:9-24): a column-major float32 coordinate buffer, the
number of rows, the selected column indices, one bandwidth per selected
column and optional lags. It returns float64 densities of the n_rows-max(tau)
selected points, computed by the CUDA library; invalid selections raise
``NativeError`` with the reference's message instead of exiting.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Sequence

import numpy as np

from . import _native
from ._native import (CallStats, HestStats, Instance, NativeError, c_f32_p, c_f64_p, c_size_p,
                      c_u32_p)

COMPAT_NORM = 1
BATCH_SUPPORT_COUNTS = 2
BATCH_DEVICE_INPUT = 4
HEST_THUMB, HEST_AMISE, HEST_AMISE_WARM = 0, 1, 2
BATCH_DEVICE_OUTPUT = 8
REF_MI, REF_TRANSS, REF_AUTOENT, REF_NEGS, REF_KLDIV = 1, 2, 3, 4, 5


def as_colmajor(coords, n_rows: int | None = None) -> tuple[np.ndarray, int, int]:
    """Return (flat float32 column-major buffer, n_rows, n_cols).

    Accepts a flat buffer (then n_rows is required) or a 2-D array of shape
    (n_cols, n_rows) -- one row per coordinate column, the reference layout.
    """
    a = np.asarray(coords)
    if a.ndim == 1:
        if n_rows is None or n_rows <= 0 or a.size % n_rows:
            raise ValueError("flat coords need n_rows dividing their length")
        n_cols = a.size // n_rows
    elif a.ndim == 2:
        n_cols, n_rows_a = a.shape
        if n_rows is not None and n_rows != n_rows_a:
            raise ValueError("n_rows does not match coords.shape[1]")
        n_rows = n_rows_a
    else:
        raise ValueError("coords must be 1-D (flat) or 2-D (n_cols, n_rows)")
    flat = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    return flat, int(n_rows), int(n_cols)


def _usecols(usecols):
    if usecols is None or len(usecols) == 0:
        return None
    return np.ascontiguousarray(np.asarray(usecols, dtype=np.uintp))


def _io_check(st: int) -> None:
    if st != 0:
        lib = _native.load()
        raise NativeError(st, (lib.ent_io_last_error() or b"").decode() or
                          lib.ent_status_string(st).decode())


def is_xtc(path) -> bool:
    """True for names CoordsFile::open gives to its XTC handler: longer than
    four characters and ending in ".xtc" (coords_file.cpp:137-145)."""
    name = os.fsdecode(path)
    return len(name) > 4 and name.endswith(".xtc")


def _xtc_check(st: int) -> None:
    if st != 0:
        lib = _native.load()
        raise NativeError(st, (lib.ent_xtc_last_error() or b"").decode() or
                          lib.ent_status_string(st).decode())


def xtc_file_shape(path) -> tuple[int, int]:
    """(frames, 3 natoms) of an XTC trajectory."""
    lib = _native.load()
    r, c = C.c_size_t(), C.c_size_t()
    _xtc_check(lib.ent_xtc_file_shape(os.fsencode(path), C.byref(r), C.byref(c)))
    return r.value, c.value


def write_xtc(path, coords, precision: float = 1000.0, primary: str = "C") -> None:
    """Write coordinates as XTC frames, one per row, as XtcHandler::write does
    (coords_file.cpp:112-126): step and time = row, zero box, precision 1000
    unless given. primary 'C': coords is (n_cols, n_rows), one row per
    coordinate like the other calls take; 'R': (n_rows, n_cols), one row per
    frame. n_cols = 3 natoms (x, y, z per atom). Encoded by all host threads;
    the bytes equal the reference's writer's."""
    if primary not in ("C", "R"):
        raise ValueError("primary must be 'C' or 'R'")
    a = np.ascontiguousarray(coords, dtype=np.float32)
    if a.ndim != 2:
        raise ValueError("coords must be 2-D")
    n_rows, n_cols = (a.shape[1], a.shape[0]) if primary == "C" else a.shape
    lib = _native.load()
    _xtc_check(lib.ent_write_xtc(os.fsencode(path), a.ctypes.data_as(C.c_void_p), n_rows,
                                 n_cols, primary.encode(), float(precision)))


def coords_file_shape(path) -> tuple[int, int]:
    """(n_rows, n_cols) of a coordinate file: the reference's ASCII format,
    or an XTC trajectory for names ending in ".xtc" (frames, 3 natoms)."""
    if is_xtc(path):
        return xtc_file_shape(path)
    lib = _native.load()
    r, c = C.c_size_t(), C.c_size_t()
    _io_check(lib.ent_coords_file_shape(os.fsencode(path), C.byref(r), C.byref(c)))
    return r.value, c.value


def read_coords(path, usecols=None, primary: str = "C") -> np.ndarray:
    """Tools::IO::read_coords (tools.hxx:153-235), parsed by all host threads.
    primary 'C' returns the column-major matrix as an (n_cols, n_rows) array
    (one row per coordinate, the layout the other calls take); 'R' returns
    (n_rows, n_cols). usecols keep the file's column order."""
    lib = _native.load()
    n_rows, n_all = coords_file_shape(path)
    uc = _usecols(usecols)
    n_cols = n_all if uc is None else len(set(int(c) for c in uc))
    if uc is not None and np.any(uc >= n_all):
        raise NativeError(4, f"given column index is not compatible with available number "
                             f"of columns ({n_all})")
    out = np.empty((n_cols, n_rows) if primary == "C" else (n_rows, n_cols), dtype=np.float32)
    _io_check(lib.ent_read_coords(os.fsencode(path),
                                  None if uc is None else uc.ctypes.data_as(c_size_p),
                                  0 if uc is None else len(uc), primary.encode(),
                                  out.ctypes.data_as(C.c_void_p), n_rows, n_cols))
    return out


def _u32(v: Sequence[int]) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, dtype=np.uint32))


def _f32(v: Sequence[float]) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32))


class Context:
    """One CUDA device, one stream and a grow-only device workspace."""

    def __init__(self, device: int = -1):
        self._lib = _native.load()
        h = C.c_void_p()
        _native.check(self._lib, None, self._lib.ent_create(C.byref(h), int(device)))
        self._h = h

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def lib(self) -> C.CDLL:
        return self._lib

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.ent_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def check(self, status: int) -> None:
        _native.check(self._lib, self._h, status)

    def last_stats(self) -> CallStats:
        s = CallStats()
        self.check(self._lib.ent_last_stats(self._h, C.byref(s)))
        return s

    def tuning(self) -> dict:
        t = _native.Tuning()
        self.check(self._lib.ent_get_tuning(self._h, C.byref(t)))
        return {"targets_per_warp": list(t.targets_per_warp), "cells_per_h": t.cells_per_h,
                "cells_per_h3": t.cells_per_h3, "moment_cells_per_h": t.moment_cells_per_h,
                "pair_variant": t.pair_variant - 1,
                "pair_variant_by_dim": [v - 1 for v in t.pair_variant_by_dim]}

    def set_tuning(self, targets_per_warp=(0, 0, 0), cells_per_h: int = 0,
                   pair_variant: int | None = None, cells_per_h3: int = 0,
                   moment_cells_per_h: int = 0) -> None:
        """Tile shapes and pair body (0 min-based, 1 saturating FMA, 2 the same at
        5 CTAs/SM, 3 as 2 with larger chunks, 4 symmetric with 4 warps of 32
        targets, 5 symmetric with 8 warps of 16) for every dimension, or a list
        of three per-dimension bodies (the first may also be 6: 1-D range sums
        from exact prefix sums, the default for d = 1; the second 7: 2-D strip
        moments, the default for d = 2); cells per bandwidth of the strips of
        the pair bodies for d = 2 (1..4) and d = 3 (1..2), and of the strip
        moments (2..12); 0/None keeps."""
        t = _native.Tuning()
        for i, v in enumerate(targets_per_warp):
            t.targets_per_warp[i] = int(v)
        t.cells_per_h = int(cells_per_h)
        t.cells_per_h3 = int(cells_per_h3)
        t.moment_cells_per_h = int(moment_cells_per_h)
        if isinstance(pair_variant, (list, tuple)):
            for i, v in enumerate(pair_variant):
                t.pair_variant_by_dim[i] = 0 if v is None else int(v) + 1
        else:
            t.pair_variant = 0 if pair_variant is None else int(pair_variant) + 1
        self.check(self._lib.ent_set_tuning(self._h, C.byref(t)))

    def _selection(self, i_cols, h, tau):
        d = len(i_cols)
        cols = _u32(i_cols)
        hv = _f32(h)
        if len(hv) != d:
            raise _native.NativeError(2, self._lib.ent_status_string(2).decode())
        tv = None
        if tau is not None:
            tv = _u32(tau)
            if len(tv) != d:
                raise _native.NativeError(3, self._lib.ent_status_string(3).decode())
        return d, cols, hv, tv

    def combined_densities(self, coords, n_rows: int | None, i_cols: Sequence[int],
                           h: Sequence[float], tau: Sequence[int] | None = None,
                           compat_norm: bool = False) -> np.ndarray:
        flat, n_rows, n_cols = as_colmajor(coords, n_rows)
        d, cols, hv, tv = self._selection(i_cols, h, tau)
        n_sel = n_rows - (int(tv.max()) if tv is not None and d else 0)
        out = np.empty(max(n_sel, 0), dtype=np.float64)
        n_out = C.c_size_t(0)
        st = self._lib.ent_densities(
            self._h, flat.ctypes.data_as(C.c_void_p), n_rows, n_cols,
            cols.ctypes.data_as(c_u32_p), hv.ctypes.data_as(c_f32_p),
            tv.ctypes.data_as(c_u32_p) if tv is not None else None, d,
            COMPAT_NORM if compat_norm else 0, out.ctypes.data_as(C.c_void_p), C.byref(n_out))
        self.check(st)
        return out[: n_out.value]

    def combined_densities_device(self, d_coords: int, n_rows: int, n_cols: int,
                                  i_cols: Sequence[int], h: Sequence[float],
                                  tau: Sequence[int] | None, d_out: int,
                                  compat_norm: bool = False) -> int:
        """Device-pointer form; returns n_sel. Pointers are raw CUDA addresses."""
        d, cols, hv, tv = self._selection(i_cols, h, tau)
        n_out = C.c_size_t(0)
        st = self._lib.ent_densities_device(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, cols.ctypes.data_as(c_u32_p),
            hv.ctypes.data_as(c_f32_p), tv.ctypes.data_as(c_u32_p) if tv is not None else None,
            d, COMPAT_NORM if compat_norm else 0, C.c_void_p(d_out), C.byref(n_out))
        self.check(st)
        return n_out.value

    def combined_densities_part_device(self, d_coords: int, n_rows: int, n_cols: int,
                                       i_cols: Sequence[int], h: Sequence[float],
                                       tau: Sequence[int] | None, part: int, n_parts: int,
                                       d_out: int, compat_norm: bool = False
                                       ) -> tuple[int, float]:
        """One share of one density's targets (of n_parts, in the library's
        sorted order) against every source: their densities into d_out (device,
        by original index; other entries untouched). Returns (n_sel, sum of
        log p over the share's targets)."""
        d, cols, hv, tv = self._selection(i_cols, h, tau)
        n_out = C.c_size_t(0)
        ls = C.c_double(0.0)
        st = self._lib.ent_densities_part_device(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, cols.ctypes.data_as(c_u32_p),
            hv.ctypes.data_as(c_f32_p), tv.ctypes.data_as(c_u32_p) if tv is not None else None,
            d, COMPAT_NORM if compat_norm else 0, int(part), int(n_parts), C.c_void_p(d_out),
            C.byref(n_out), C.byref(ls))
        self.check(st)
        return n_out.value, ls.value

    def support_counts(self, coords, n_rows: int | None, i_cols: Sequence[int],
                       h: Sequence[float], tau: Sequence[int] | None = None) -> np.ndarray:
        """Per point, the number of sources inside the product-kernel support."""
        flat, n_rows, n_cols = as_colmajor(coords, n_rows)
        d, cols, hv, tv = self._selection(i_cols, h, tau)
        n_sel = n_rows - (int(tv.max()) if tv is not None and d else 0)
        out = np.empty(max(n_sel, 0), dtype=np.float64)
        n_out = C.c_size_t(0)
        st = self._lib.ent_support_counts(
            self._h, flat.ctypes.data_as(C.c_void_p), n_rows, n_cols,
            cols.ctypes.data_as(c_u32_p), hv.ctypes.data_as(c_f32_p),
            tv.ctypes.data_as(c_u32_p) if tv is not None else None, d,
            out.ctypes.data_as(C.c_void_p), C.byref(n_out))
        self.check(st)
        return out[: n_out.value]


    # ------------------------------------------------------------ batches
    def mi_all_pairs(self, coords, h: Sequence[float], counts: bool = False
                     ) -> tuple[np.ndarray, np.ndarray]:
        """All-pairs MI (resubstitution) of the rows of coords (n_cols, n_rows)
        in one batch; returns (MI matrix, marginal entropies). With
        counts=True, the in-support pair counts of every density instead."""
        flat, n_rows, n_cols = as_colmajor(coords)
        hv = _f32(h)
        if len(hv) != n_cols:
            raise ValueError("one bandwidth per column")
        mi = np.zeros((n_cols, n_cols), dtype=np.float64)
        hx = np.zeros(n_cols, dtype=np.float64)
        st = self._lib.ent_mi_all_pairs(
            self._h, flat.ctypes.data_as(C.c_void_p), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            BATCH_SUPPORT_COUNTS if counts else 0, mi.ctypes.data_as(c_f64_p),
            hx.ctypes.data_as(c_f64_p))
        self.check(st)
        return mi, hx

    def mi_all_pairs_device(self, d_coords: int, n_rows: int, n_cols: int,
                            h: Sequence[float], counts: bool = False
                            ) -> tuple[np.ndarray, np.ndarray]:
        hv = _f32(h)
        mi = np.zeros((n_cols, n_cols), dtype=np.float64)
        hx = np.zeros(n_cols, dtype=np.float64)
        st = self._lib.ent_mi_all_pairs_device(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            BATCH_SUPPORT_COUNTS if counts else 0, mi.ctypes.data_as(c_f64_p),
            hx.ctypes.data_as(c_f64_p))
        self.check(st)
        return mi, hx

    def mi_entropies_device(self, d_coords: int, n_rows: int, n_cols: int, h: Sequence[float],
                            items: Sequence[int], counts: bool = False) -> np.ndarray:
        """Entropies of the listed densities of the all-pairs MI batch (batch
        order: the n_cols marginals, then the joints i < j in row order),
        computed as one batch from device coordinates."""
        hv = _f32(h)
        it = np.ascontiguousarray(np.asarray(items, dtype=np.uint64))
        out = np.zeros(len(it), dtype=np.float64)
        self.check(self._lib.ent_mi_entropies_device(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            it.ctypes.data_as(C.POINTER(C.c_uint64)), len(it),
            BATCH_SUPPORT_COUNTS if counts else 0, out.ctypes.data_as(c_f64_p)))
        return out

    def te_entropies_device(self, d_coords: int, n_rows: int, n_cols: int, h: Sequence[float],
                            taus: Sequence[int], items: Sequence[int],
                            counts: bool = False) -> np.ndarray:
        """Entropies of the listed densities of the all-ordered-pairs TE batch
        (batch order per lag: n_cols 1-D, n_cols lagged 2-D, the joints i < j,
        the 3-D (i, j), i != j), computed as one batch from device
        coordinates."""
        hv, tv = _f32(h), _u32(taus)
        it = np.ascontiguousarray(np.asarray(items, dtype=np.uint64))
        out = np.zeros(len(it), dtype=np.float64)
        self.check(self._lib.ent_te_entropies_device(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            tv.ctypes.data_as(c_u32_p), len(tv), it.ctypes.data_as(C.POINTER(C.c_uint64)),
            len(it), BATCH_SUPPORT_COUNTS if counts else 0, out.ctypes.data_as(c_f64_p)))
        return out

    def te_all_pairs(self, coords, h: Sequence[float], taus: Sequence[int],
                     counts: bool = False) -> np.ndarray:
        """All-ordered-pairs transfer entropy; returns (n_taus, M, M) with
        [q, i, j] = TE_{j->i}(taus[q])."""
        flat, n_rows, n_cols = as_colmajor(coords)
        hv, tv = _f32(h), _u32(taus)
        out = np.zeros((len(tv), n_cols, n_cols), dtype=np.float64)
        self.check(self._lib.ent_te_all_pairs(
            self._h, flat.ctypes.data_as(C.c_void_p), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            tv.ctypes.data_as(c_u32_p), len(tv), BATCH_SUPPORT_COUNTS if counts else 0,
            out.ctypes.data_as(c_f64_p)))
        return out

    def te_all_pairs_device(self, d_coords: int, n_rows: int, n_cols: int, h, taus,
                            counts: bool = False) -> np.ndarray:
        hv, tv = _f32(h), _u32(taus)
        out = np.zeros((len(tv), n_cols, n_cols), dtype=np.float64)
        self.check(self._lib.ent_te_all_pairs_device(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            tv.ctypes.data_as(c_u32_p), len(tv), BATCH_SUPPORT_COUNTS if counts else 0,
            out.ctypes.data_as(c_f64_p)))
        return out

    def _instances(self, instances, device: bool):
        arr = (Instance * len(instances))()
        keep = []
        for q, item in enumerate(instances):
            if device:
                addr, d, n, h = item
                arr[q].coords = C.c_void_p(addr)
            else:
                x, h = item
                x = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float32)
                keep.append(x)
                d, n = x.shape
                arr[q].coords = x.ctypes.data_as(C.c_void_p)
            arr[q].n = n
            arr[q].d = d
            for j in range(d):
                arr[q].h[j] = float(h[j])
        return arr, keep

    def autotune(self, instances, d: int, force: bool = False, device: bool = False) -> dict:
        """The library's own autotuner (ent_autotune): time the candidate shapes of
        dimension d on a sample batch [(coords (d, n), h)...] (or device tuples
        as in entropy_batch), apply the fastest and keep it in the context's
        cache; returns the context's tuning afterwards."""
        arr, keep = self._instances(instances, device)
        t = _native.Tuning()
        flags = (1 if force else 0) | (BATCH_DEVICE_INPUT if device else 0)
        self.check(self._lib.ent_autotune(self._h, C.cast(arr, C.c_void_p), len(instances),
                                          int(d), flags, C.byref(t)))
        return self.tuning()

    def autotune_cache_size(self) -> int:
        return int(self._lib.ent_autotune_cache_size(self._h))

    def entropy_batch(self, instances, counts: bool = False, device: bool = False) -> np.ndarray:
        """Resubstitution entropies of [(coords (d, n), h (d,))...] in one batch.
        With device=True, coords entries are raw device addresses and the
        tuples are (address, d, n, h)."""
        arr = (Instance * len(instances))()
        keep = []
        for q, item in enumerate(instances):
            if device:
                addr, d, n, h = item
                arr[q].coords = C.c_void_p(addr)
            else:
                x, h = item
                x = np.ascontiguousarray(np.atleast_2d(x), dtype=np.float32)
                keep.append(x)
                d, n = x.shape
                arr[q].coords = x.ctypes.data_as(C.c_void_p)
            arr[q].n = n
            arr[q].d = d
            for j in range(d):
                arr[q].h[j] = float(h[j])
        out = np.zeros(len(instances), dtype=np.float64)
        flags = (BATCH_SUPPORT_COUNTS if counts else 0) | (BATCH_DEVICE_INPUT if device else 0)
        st = self._lib.ent_entropy_batch(self._h, C.cast(arr, C.c_void_p), len(instances),
                                         flags, out.ctypes.data_as(c_f64_p))
        self.check(st)
        return out

    def reference_estimator(self, coords, h: Sequence[float], estimator: int,
                            tau: int = 0) -> np.ndarray:
        """One of the reference's estimators (REF_MI, REF_TRANSS, REF_AUTOENT,
        REF_NEGS, REF_KLDIV) over all columns of coords (n_cols, n_rows) with
        its own formula, as one device batch (ent_reference_estimator).
        Returns an (n_cols, n_cols) matrix or an (n_cols,) vector."""
        flat, n_rows, n_cols = as_colmajor(coords)
        hv = _f32(h)
        if len(hv) != n_cols:
            raise ValueError("one bandwidth per column")
        vec = estimator in (REF_AUTOENT, REF_NEGS)
        out = np.zeros(n_cols if vec else n_cols * n_cols, dtype=np.float64)
        st = self._lib.ent_reference_estimator(
            self._h, flat.ctypes.data_as(C.c_void_p), n_rows, n_cols,
            hv.ctypes.data_as(c_f32_p), int(estimator), int(tau), 0,
            out.ctypes.data_as(c_f64_p))
        self.check(st)
        return out if vec else out.reshape(n_cols, n_cols)

    def log64_selftest(self, x) -> np.ndarray:
        """The FP64 log of the per-point epilogues evaluated on the device."""
        xv = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
        out = np.empty_like(xv)
        self.check(self._lib.ent_log64_selftest(self._h, xv.ctypes.data_as(c_f64_p), xv.size,
                                                 out.ctypes.data_as(c_f64_p)))
        return out

    def ilog_selftest(self, values) -> np.ndarray:
        """The strip-moment epilogue's log of nonnegative integers below 2^128
        evaluated on the device: round(log(T) 2^48) per value (int64)."""
        vals = [int(v) for v in values]
        t = np.zeros(2 * len(vals), dtype=np.uint64)
        for i, v in enumerate(vals):
            t[2 * i] = v & 0xFFFFFFFFFFFFFFFF
            t[2 * i + 1] = v >> 64
        out = np.zeros(len(vals), dtype=np.int64)
        self.check(self._lib.ent_ilog_selftest(self._h, t.ctypes.data_as(C.POINTER(C.c_uint64)),
                                               len(vals),
                                               out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def reference_estimator_device(self, d_coords: int, n_rows: int, n_cols: int,
                                   h: Sequence[float], estimator: int, tau: int = 0
                                   ) -> np.ndarray:
        """reference_estimator on a column-major device matrix (raw address)."""
        hv = _f32(h)
        vec = estimator in (REF_AUTOENT, REF_NEGS)
        out = np.zeros(n_cols if vec else n_cols * n_cols, dtype=np.float64)
        st = self._lib.ent_reference_estimator(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            int(estimator), int(tau), BATCH_DEVICE_INPUT, out.ctypes.data_as(c_f64_p))
        self.check(st)
        return out if vec else out.reshape(n_cols, n_cols)

    def dens_all_device(self, d_coords: int, n_rows: int, n_cols: int, h: Sequence[float],
                        dims: int, d_out: int, taus=None) -> tuple[int, int]:
        """dens_all with device coordinates and device output (raw addresses;
        d_out holds n_densities x n_sel doubles). Returns (n_densities, n_sel)."""
        hv = _f32(h)
        tv = None if taus is None else _u32(taus)
        ni, ns = C.c_size_t(), C.c_size_t()
        st = self._lib.ent_dens_all(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, hv.ctypes.data_as(c_f32_p), int(dims),
            None if tv is None else tv.ctypes.data_as(c_u32_p),
            BATCH_DEVICE_INPUT | BATCH_DEVICE_OUTPUT, C.c_void_p(d_out), C.byref(ni), C.byref(ns))
        self.check(st)
        return ni.value, ns.value

    def dens_all(self, coords, h: Sequence[float], dims: int, taus=None) -> np.ndarray:
        """Sum-normalised densities of every column (dims=1), pair (2) or
        triple (3) in the reference's order (dens.cpp:19-106), one device
        batch (ent_dens_all); returns an (n_densities, n_sel) array."""
        flat, n_rows, n_cols = as_colmajor(coords)
        hv = _f32(h)
        if len(hv) != n_cols:
            raise ValueError("one bandwidth per column")
        tv = None if taus is None else _u32(taus)
        if tv is not None and len(tv) != dims:
            raise ValueError("one lag per density dimension")
        M = n_cols
        n_inst = M if dims == 1 else (M * (M - 1) // 2 if dims == 2 else M * (M - 1) * (M - 2) // 6)
        mx = 0 if (tv is None or dims == 1) else int(tv.max())
        out = np.zeros((max(n_inst, 1), max(n_rows - mx, 0)), dtype=np.float64)
        ni, ns = C.c_size_t(), C.c_size_t()
        st = self._lib.ent_dens_all(
            self._h, flat.ctypes.data_as(C.c_void_p), n_rows, n_cols, hv.ctypes.data_as(c_f32_p),
            int(dims), None if tv is None else tv.ctypes.data_as(c_u32_p), 0,
            out.ctypes.data_as(C.c_void_p), C.byref(ni), C.byref(ns))
        self.check(st)
        return out[: ni.value, : ns.value]
    def load_coords_device(self, path, d_out: int, usecols=None) -> tuple[int, int]:
        """Parse a coordinate file into the column-major device matrix at
        address d_out (n_rows x n_cols floats; see coords_file_shape), with
        pinned, overlapped host-to-device copies. Names ending in ".xtc" are
        XTC trajectories, decoded on the device (load_xtc_device), as
        CoordsFile::open picks its handler. Returns (n_rows, n_cols)."""
        if is_xtc(path):
            return self.load_xtc_device(path, d_out, usecols)
        n_rows, n_all = coords_file_shape(path)
        uc = _usecols(usecols)
        n_cols = n_all if uc is None else len(set(int(c) for c in uc))
        st = self._lib.ent_load_coords_device(
            self._h, os.fsencode(path), None if uc is None else uc.ctypes.data_as(c_size_p),
            0 if uc is None else len(uc), C.c_void_p(d_out), n_rows, n_cols)
        self.check(st)
        return n_rows, n_cols

    def _xtc_shape(self, path, usecols):
        n_rows, n_all = xtc_file_shape(path)
        uc = _usecols(usecols)
        n_cols = n_all if uc is None else len(set(int(c) for c in uc))
        return n_rows, n_cols, uc

    def load_xtc_device(self, path, d_out: int, usecols=None) -> tuple[int, int]:
        """Decode an XTC trajectory on the device into the column-major matrix
        at d_out (frames x columns; column 3a + c is coordinate c of atom a).
        The compressed file is what is copied to the device. Returns
        (n_rows, n_cols)."""
        n_rows, n_cols, uc = self._xtc_shape(path, usecols)
        st = self._lib.ent_load_xtc_device(
            self._h, os.fsencode(path), None if uc is None else uc.ctypes.data_as(c_size_p),
            0 if uc is None else len(uc), C.c_void_p(d_out), n_rows, n_cols)
        self.check(st)
        return n_rows, n_cols

    def read_xtc(self, path, usecols=None, primary: str = "C") -> np.ndarray:
        """XTC trajectory decoded on the device, returned in host memory:
        primary 'C' as an (n_cols, n_frames) array (one row per coordinate,
        the layout the other calls take), 'R' as (n_frames, n_cols) (the rows
        XtcHandler::next returns)."""
        n_rows, n_cols, uc = self._xtc_shape(path, usecols)
        out = np.empty((n_cols, n_rows) if primary == "C" else (n_rows, n_cols), np.float32)
        st = self._lib.ent_read_xtc(
            self._h, os.fsencode(path), None if uc is None else uc.ctypes.data_as(c_size_p),
            0 if uc is None else len(uc), primary.encode(), out.ctypes.data_as(C.c_void_p),
            n_rows, n_cols)
        self.check(st)
        return out

    # ---------------------------------------------------- neighbour search
    def neighbor_windows(self, col, h: float) -> tuple[np.ndarray, np.ndarray]:
        """The reference boxes() source window [lo, hi] of every point."""
        return self._neighbors(col, h, 0)[:2]

    def boxed_neighbors(self, col, box: float) -> tuple[int, np.ndarray, np.ndarray]:
        """BoxedSearch: (number of boxes, box of every point, neighbour-list sizes)."""
        a, b, nb = self._neighbors(col, box, 1)
        return nb, a, b

    def _neighbors(self, col, h, mode):
        x = np.ascontiguousarray(np.asarray(col, dtype=np.float32).ravel())
        a = np.zeros(x.size, np.uint64)
        b = np.zeros(x.size, np.uint64)
        nb = C.c_uint64(0)
        self.check(self._lib.ent_neighbor_counts(self._h, x.ctypes.data_as(C.c_void_p), x.size,
                                                 float(h), mode, a.ctypes.data_as(C.c_void_p),
                                                 b.ctypes.data_as(C.c_void_p), C.byref(nb)))
        return a, b, int(nb.value)

    # ------------------------------------------------- bandwidth estimation
    def epa_convolution(self, sorted_coords, h: float) -> float:
        """1/n^2 sum_ij max(0, 4.5 - 2.25 |x_i - x_j| / h) (reference
        epa_convolution, densities_omp.cpp:235-277)."""
        x = np.ascontiguousarray(np.asarray(sorted_coords, dtype=np.float32).ravel())
        out = C.c_float(0.0)
        self.check(self._lib.ent_epa_convolution(self._h, x.ctypes.data_as(C.c_void_p), x.size,
                                                 float(h), C.byref(out)))
        return float(out.value)

    def hestimate(self, coords, mode: int = HEST_AMISE, cols: Sequence[int] | None = None,
                  h_init: Sequence[float] | None = None, skip_levels: int = 0
                  ) -> tuple[np.ndarray, list[dict]]:
        """Per-column bandwidths (Thumb or AMISE search; warm-started from
        h_init when mode == HEST_AMISE_WARM). coords: (n_cols, n_rows)."""
        flat, n_rows, n_cols = as_colmajor(coords)
        sel = np.arange(n_cols, dtype=np.uint32) if cols is None else _u32(cols)
        hout = np.zeros(len(sel), dtype=np.float32)
        hin = None if h_init is None else _f32(h_init)
        st = (HestStats * len(sel))()
        self.check(self._lib.ent_hestimate(
            self._h, flat.ctypes.data_as(C.c_void_p), n_rows, n_cols, sel.ctypes.data_as(c_u32_p),
            len(sel), int(mode), hin.ctypes.data_as(c_f32_p) if hin is not None else None,
            int(skip_levels), hout.ctypes.data_as(c_f32_p), C.cast(st, C.c_void_p)))
        return hout, [dict(h0=s.h0, conv_evals=s.conv_evals, levels_skipped=s.levels_skipped,
                           warm_converged=s.warm_converged) for s in st]

    def hestimate_device(self, d_coords: int, n_rows: int, n_cols: int, mode: int = HEST_AMISE,
                         h_init: Sequence[float] | None = None, skip_levels: int = 0
                         ) -> tuple[np.ndarray, list[dict]]:
        sel = np.arange(n_cols, dtype=np.uint32)
        hout = np.zeros(n_cols, dtype=np.float32)
        hin = None if h_init is None else _f32(h_init)
        st = (HestStats * n_cols)()
        self.check(self._lib.ent_hestimate_device(
            self._h, C.c_void_p(d_coords), n_rows, n_cols, sel.ctypes.data_as(c_u32_p), n_cols,
            int(mode), hin.ctypes.data_as(c_f32_p) if hin is not None else None,
            int(skip_levels), hout.ctypes.data_as(c_f32_p), C.cast(st, C.c_void_p)))
        return hout, [dict(h0=s.h0, conv_evals=s.conv_evals, levels_skipped=s.levels_skipped,
                           warm_converged=s.warm_converged) for s in st]


_default: Context | None = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context()
    return _default


def combined_densities(coords, n_rows: int | None, i_cols: Sequence[int], h: Sequence[float],
                       tau: Sequence[int] | None = None, compat_norm: bool = False) -> np.ndarray:
    """Densities of the selected (lagged) columns; see ``Context.combined_densities``."""
    return default_context().combined_densities(coords, n_rows, i_cols, h, tau, compat_norm)
