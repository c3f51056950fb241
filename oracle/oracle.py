"""Python access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
this module, and only as the checker. It wraps

* ``lib/libentoracle.so``: the C restatement of the reference algorithms and
  the FP64 brute force (ent_oracle.c, built by ``make -C oracle oracle``);
* ``_ref/libentref.so``: the reference's own OpenMP sources compiled in place
  (``make -C oracle ref``; only where the reference sources exist);

plus FP64 numpy forms of the estimators (entropy, mutual information,
transfer entropy) on oracle densities.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "lib" / "libentoracle.so"
REF_SO = HERE / "_ref" / "libentref.so"

_orc = None
_ref = None


def _p(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
    return ORACLE_SO


def reference_dir() -> Path | None:
    """The reference checkout: $ENT_REFERENCE, else a ``reference`` directory
    beside this repository; None when neither holds the reference sources."""
    env = os.environ.get("ENT_REFERENCE")
    cand = Path(env) if env else HERE.parent.parent / "reference"
    return cand if (cand / "densities_omp.cpp").exists() else None


def build_ref(reference: str | Path | None = None) -> Path | None:
    ref_dir = Path(reference) if reference else reference_dir()
    if ref_dir is None or not (ref_dir / "densities_omp.cpp").exists():
        return None
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "ref", f"REF={ref_dir}"], check=True)
    return REF_SO


def orc() -> C.CDLL:
    global _orc
    if _orc is None:
        if not ORACLE_SO.exists():
            build_oracle()
        lib = C.CDLL(str(ORACLE_SO))
        lib.orc_epa_conv_ref.restype = C.c_float
        lib.orc_epa_conv_fp64.restype = C.c_double
        lib.orc_thumb_ref.restype = C.c_float
        lib.orc_amise_from_conv.restype = C.c_float
        lib.orc_amise_from_conv.argtypes = [C.c_float, C.c_float, C.c_size_t]
        lib.orc_hestimate_amise.restype = C.c_float
        lib.orc_boxedsearch.restype = C.c_uint64
        lib.orc_support_count_fp64.restype = C.c_uint64
        _orc = lib
    return _orc


def ref_available() -> bool:
    return REF_SO.exists()


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        lib = C.CDLL(str(REF_SO))
        lib.ref_epa_convolution.restype = C.c_float
        lib.ref_thumb.restype = C.c_float
        lib.ref_amise_h.restype = C.c_float
        lib.ref_boxedsearch.restype = C.c_uint64
        _ref = lib
    return _ref


# ------------------------------------------------------------- selections
def repack(coords: np.ndarray, cols, tau=None) -> np.ndarray:
    """(n_cols, n_rows) column-major coords -> (d, n_sel) selected, lagged
    columns, as prob_dens_coord_prep builds them (densities_common.hxx:37-48)."""
    coords = np.asarray(coords, dtype=np.float32)
    d = len(cols)
    tau = [0] * d if tau is None else list(tau)
    n_sel = coords.shape[1] - max(tau)
    return np.ascontiguousarray(
        np.stack([coords[c, t:t + n_sel] for c, t in zip(cols, tau)]).astype(np.float32))


# ---------------------------------------------------------------- densities
def density_fp64(sel: np.ndarray, h, norm: float | None = None, targets=None) -> np.ndarray:
    sel = np.ascontiguousarray(sel, dtype=np.float32)
    d, n = sel.shape
    hd = np.ascontiguousarray(np.asarray(h, dtype=np.float32).astype(np.float64))
    norm = float(n if norm is None else norm)
    if targets is None:
        out = np.empty(n)
        st = orc().orc_density_fp64(_p(sel), C.c_size_t(n), C.c_int(d), _p(hd),
                                    C.c_double(norm), _p(out))
    else:
        t = np.ascontiguousarray(np.asarray(targets, dtype=np.uint32))
        out = np.empty(len(t))
        st = orc().orc_density_fp64_at(_p(sel), C.c_size_t(n), C.c_int(d), _p(hd),
                                       C.c_double(norm), _p(t), C.c_size_t(len(t)), _p(out))
    assert st == 0
    return out


def support_count_fp64(sel: np.ndarray, h) -> int:
    """Ordered pairs inside the product-kernel support (FP64 test)."""
    sel = np.ascontiguousarray(sel, dtype=np.float32)
    d, n = sel.shape
    hd = np.ascontiguousarray(np.asarray(h, dtype=np.float32).astype(np.float64))
    return int(orc().orc_support_count_fp64(_p(sel), C.c_size_t(n), C.c_int(d), _p(hd)))


def density_ref_f32(sel: np.ndarray, h, linear_scan: bool = False) -> np.ndarray:
    """Reference OpenMP density restated; linear_scan=True also keeps the
    reference's O(n) window scans per point (for timing)."""
    sel = np.ascontiguousarray(sel, dtype=np.float32)
    d, n = sel.shape
    hf = np.ascontiguousarray(np.asarray(h, dtype=np.float32))
    out = np.empty(n, dtype=np.float32)
    fn = orc().orc_density_ref_f32_linear if linear_scan else orc().orc_density_ref_f32
    assert fn(_p(sel), C.c_size_t(n), C.c_int(d), _p(hf), _p(out)) == 0
    return out


def boxes(col: np.ndarray, h: float) -> tuple[np.ndarray, np.ndarray]:
    col = np.ascontiguousarray(col, dtype=np.float32)
    lo = np.empty(len(col), np.uint64)
    hi = np.empty(len(col), np.uint64)
    orc().orc_boxes(_p(col), C.c_size_t(len(col)), C.c_float(h), _p(lo), _p(hi))
    return lo, hi


def boxedsearch(col: np.ndarray, box: float):
    col = np.ascontiguousarray(col, dtype=np.float32)
    b = np.empty(len(col), np.uint64)
    c = np.empty(len(col), np.uint64)
    nb = orc().orc_boxedsearch(_p(col), C.c_size_t(len(col)), C.c_float(box), _p(b), _p(c))
    return int(nb), b, c


def epa_conv_ref(sorted_col: np.ndarray, h: float) -> float:
    s = np.ascontiguousarray(sorted_col, dtype=np.float32)
    return float(orc().orc_epa_conv_ref(_p(s), C.c_size_t(len(s)), C.c_float(h)))


def epa_conv_fp64(sorted_col: np.ndarray, h: float) -> float:
    s = np.ascontiguousarray(sorted_col, dtype=np.float32)
    return float(orc().orc_epa_conv_fp64(_p(s), C.c_size_t(len(s)), C.c_double(h)))


def thumb_ref(col: np.ndarray) -> float:
    c = np.ascontiguousarray(col, dtype=np.float32)
    return float(orc().orc_thumb_ref(_p(c), C.c_size_t(len(c))))


def amise_from_conv(conv: float, h: float, n: int) -> float:
    return float(orc().orc_amise_from_conv(conv, h, n))


def hestimate_amise(col: np.ndarray, exact: bool = False) -> tuple[float, int]:
    c = np.ascontiguousarray(col, dtype=np.float32)
    nc = C.c_int(0)
    h = orc().orc_hestimate_amise(_p(c), C.c_size_t(len(c)), C.c_int(1 if exact else 0),
                                  C.byref(nc))
    return float(h), nc.value


# -------------------------------------------------------------- estimators
def entropy_fp64(sel: np.ndarray, h, norm=None) -> float:
    """Resubstitution entropy -mean(log p) with FP64 oracle densities."""
    p = density_fp64(sel, h, norm)
    return float(-np.mean(np.log(p)))


def mi_fp64(x: np.ndarray, y: np.ndarray, hx: float, hy: float) -> float:
    """MI = H(X) + H(Y) - H(X, Y), resubstitution, FP64 oracle densities."""
    return (entropy_fp64(x[None], [hx]) + entropy_fp64(y[None], [hy])
            - entropy_fp64(np.stack([x, y]), [hx, hy]))


def te_fp64(x: np.ndarray, y: np.ndarray, tau: int, hx: float, hy: float) -> float:
    """TE_{X->Y}(tau) = mean_t log[p(y+,y,x) p(y) / (p(y,x) p(y+,y))] over
    t < n - tau (resubstitution, FP64 oracle densities)."""
    n = len(y) - tau
    yp, yc, xc = y[tau:tau + n], y[:n], x[:n]
    l3 = np.log(density_fp64(np.stack([yp, yc, xc]), [hy, hy, hx]))
    l1 = np.log(density_fp64(yc[None], [hy]))
    l2a = np.log(density_fp64(np.stack([yc, xc]), [hy, hx]))
    l2b = np.log(density_fp64(np.stack([yp, yc]), [hy, hy]))
    return float(np.mean(l3 + l1 - l2a - l2b))


def _flog32(v):
    """Tools::select_log(false) (tools.cpp:18-37): float log of the value cast
    to float, 0 at 0."""
    v32 = np.asarray(v, dtype=np.float64).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(v32 == 0, np.float32(0), np.log(v32)).astype(np.float64)


def _inv(v):
    v = np.asarray(v, dtype=np.float64)
    with np.errstate(divide="ignore"):
        return np.where(v == 0, v, 1.0 / v)


def reference_estimator_fp64(x: np.ndarray, h, estimator: str, tau: int = 0,
                             bound: bool = False):
    """The reference estimators' formulas (mi.cpp:37-59, transs.cpp:39-115,
    autoent.cpp:39-58, negs.cpp:36-47, kldiv.cpp:36-54) over FP64 oracle
    densities normalised by n_rows (densities_cuda.cu:98-103), with the float
    log of tools.cpp:18-37 and FP64 sums. x: (n_cols, n_rows).

    bound=True also returns, per output, sum_k (|term_k| + |weight_k|) (weight
    = the factor in front of the log): the scale against which float-log
    results are compared (a relative density error e moves a term by at most
    e (|term| + 3 |weight|), a float rounding of the log argument by 6e-8
    |weight|)."""
    x = np.asarray(x, np.float32)
    M, N = x.shape
    h = np.asarray(h, np.float32)
    bnd = None

    def dens(cols, lags=None):
        lags = [0] * len(cols) if lags is None else lags
        n = N - max(lags)
        sel = np.stack([x[c][l:l + n] for c, l in zip(cols, lags)])
        return density_fp64(sel, [h[c] for c in cols], norm=float(N))

    if estimator == "mi":
        p = [dens([i]) for i in range(M)]
        out, bnd = np.zeros((M, M)), np.zeros((M, M))
        for i in range(M):
            for j in range(i + 1, M):
                pij = dens([i, j])
                t = pij * _flog32(pij / p[i] / p[j])
                out[i, j] = out[j, i] = np.sum(t)
                bnd[i, j] = bnd[j, i] = np.sum(np.abs(t) + np.abs(pij))
        return (out, bnd) if bound else out
    if estimator == "transs":
        m = N - tau
        p = [dens([i]) for i in range(M)]
        pt = [dens([i, i], [0, tau]) for i in range(M)]
        out, bnd = np.zeros((M, M)), np.zeros((M, M))
        for i in range(M):
            for j in range(i + 1, M):
                hi, hj = float(h[i]), float(h[j])
                pij = dens([i, j])
                for (a, b, p3, w, pp, ptt) in (
                        (i, j, dens([i, i, j], [0, tau, 0]), (hi, hi, hj), p[i], pt[i]),
                        (j, i, dens([i, j, j], [0, 0, tau]), (hi, hj, hi), p[j], pt[j])):
                    p3, pp, pq, ptt = p3[:m], pp[:m], pij[:m], ptt[:m]
                    arg = p3 * pp * _inv(pq) * _inv(ptt)
                    with np.errstate(invalid="ignore"):
                        te = p3 * w[0] * w[1] * w[2] * _flog32(arg)
                    ok = (p3 > 0) & np.isfinite(te) & (p3 <= 1.0)
                    out[a, b] = np.sum(te[ok])
                    bnd[a, b] = np.sum(np.abs(te[ok]) + np.abs(p3 * w[0] * w[1] * w[2])[ok])
        return (out, bnd) if bound else out
    if estimator == "autoent":
        out, bnd = np.zeros(M), np.zeros(M)
        for i in range(M):
            hh = float(h[i])
            p1 = dens([i], [tau])
            p2 = dens([i, i], [0, tau])
            ok = p2 > 0
            t = (p2 * hh * hh * _flog32(p1 * _inv(p2 * hh)))[ok]
            out[i] = np.sum(t)
            bnd[i] = np.sum(np.abs(t) + (p2 * hh * hh)[ok])
        return (out, bnd) if bound else out
    ps = []
    for i in range(M):
        p = dens([i])
        ps.append(p / p.sum())
    if estimator == "negs":
        out = np.array([-np.sum(_flog32(q) * q) for q in ps])
        bnd = np.array([np.sum(np.abs(_flog32(q) * q) + q) for q in ps])
        return (out, bnd) if bound else out
    if estimator == "kldiv":
        out, bnd = np.zeros((M, M)), np.zeros((M, M))
        for i in range(M):
            for j in range(M):
                if i != j:
                    t = ps[i] * _flog32(ps[i] / ps[j])
                    out[i, j] = np.sum(t)
                    bnd[i, j] = np.sum(np.abs(t) + ps[i])
        return (out, bnd) if bound else out
    raise ValueError(estimator)


# ------------------------------------------------------- reference build
def ref_densities(coords: np.ndarray, cols, h, tau=None) -> np.ndarray:
    """The reference's OpenMP combined_densities on repacked columns (float32,
    already divided by n_sel)."""
    coords = np.ascontiguousarray(coords, dtype=np.float32)
    n_cols, n_rows = coords.shape
    d = len(cols)
    tau = [0] * d if tau is None else list(tau)
    c = np.ascontiguousarray(np.asarray(cols, np.uint32))
    hh = np.ascontiguousarray(np.asarray(h, np.float32))
    t = np.ascontiguousarray(np.asarray(tau, np.uint32))
    out = np.empty(n_rows - max(tau), np.float32)
    assert ref().ref_densities(_p(coords), C.c_size_t(n_rows), _p(c), _p(hh), _p(t),
                               C.c_uint(d), _p(out)) == 0
    return out


def ref_epa_convolution(sorted_col: np.ndarray, h: float) -> float:
    s = np.ascontiguousarray(sorted_col, dtype=np.float32)
    return float(ref().ref_epa_convolution(_p(s), C.c_size_t(len(s)), C.c_float(h)))


def ref_boxes(col: np.ndarray, h: float):
    col = np.ascontiguousarray(col, dtype=np.float32)
    lo = np.empty(len(col), np.uint64)
    hi = np.empty(len(col), np.uint64)
    ref().ref_boxes(_p(col), C.c_size_t(len(col)), C.c_float(h), _p(lo), _p(hi))
    return lo, hi


def ref_boxedsearch(col: np.ndarray, box: float):
    col = np.ascontiguousarray(col, dtype=np.float32)
    b = np.empty(len(col), np.uint64)
    c = np.empty(len(col), np.uint64)
    nb = ref().ref_boxedsearch(_p(col), C.c_size_t(len(col)), C.c_float(box), _p(b), _p(c))
    return int(nb), c


def ref_read_coords(path, primary: str = "C", usecols=None) -> np.ndarray:
    """The reference's Tools::IO::read_coords (tools.hxx:153-235), compiled in
    place: 'C' -> (n_cols, n_rows) array of the column-major buffer, 'R' ->
    (n_rows, n_cols)."""
    uc = np.ascontiguousarray(np.asarray([] if usecols is None else usecols, dtype=np.uintp))
    r, k = C.c_size_t(), C.c_size_t()
    lib = ref()
    p = C.c_char_p(os.fsencode(str(path)))
    lib.ref_read_coords(p, C.c_char(primary.encode()), _p(uc), C.c_size_t(len(uc)), None,
                        C.byref(r), C.byref(k))
    out = np.empty((k.value, r.value) if primary == "C" else (r.value, k.value), np.float32)
    lib.ref_read_coords(p, C.c_char(primary.encode()), _p(uc), C.c_size_t(len(uc)), _p(out),
                        C.byref(r), C.byref(k))
    return out


def ref_thumb(col: np.ndarray) -> float:
    c = np.ascontiguousarray(col, dtype=np.float32)
    return float(ref().ref_thumb(_p(c), C.c_size_t(len(c)), C.c_size_t(0)))


def ref_amise_h(col: np.ndarray) -> float:
    c = np.ascontiguousarray(col, dtype=np.float32)
    return float(ref().ref_amise_h(_p(c), C.c_size_t(len(c)), C.c_size_t(0)))


def ref_run_mode(mode: str, coords: np.ndarray, bandwidths, workdir: Path, tau: int = 0,
                 dims: int = 1, taus: str = "") -> np.ndarray:
    """Run a reference estimator main() (mi, transs, autoent, negs, kldiv, dens)
    on an ASCII file, as the entropical CLI would, and parse its output."""
    workdir = Path(workdir)
    workdir.mkdir(parents=True, exist_ok=True)
    fin, fbw, fout = workdir / "coords.txt", workdir / "bw.txt", workdir / "out.txt"
    np.savetxt(fin, np.asarray(coords, np.float32).T, fmt="%.9g")
    np.savetxt(fbw, np.asarray(bandwidths, np.float32)[None], fmt="%.9g")
    st = ref().ref_run_mode(mode.encode(), str(fin).encode(), str(fbw).encode(),
                            str(fout).encode(), C.c_uint(tau), C.c_uint(dims), taus.encode())
    assert st == 0
    if mode == "dens" and dims > 1:
        rows = [ln.split() for ln in fout.read_text().splitlines() if ln.strip()]
        return np.array([float(r[1]) for r in rows])
    return np.loadtxt(fout, ndmin=2)


# ------------------------------------------------------------- XTC files
XDR_SO = HERE / "_ref" / "libentxdr.so"
_xdr = None


def xtc_shape(path) -> tuple[int, int]:
    """(frames, natoms) by the oracle's XTC reader (xtc_oracle.c)."""
    lib = orc()
    nf, na = C.c_size_t(), C.c_size_t()
    st = lib.orc_xtc_shape(str(path).encode(), C.byref(nf), C.byref(na))
    if st != 0:
        raise ValueError(f"orc_xtc_shape: {st}")
    return nf.value, na.value


def read_xtc(path, f0: int = 0, f1: int | None = None) -> np.ndarray:
    """Frames [f0, f1) as rows of 3 natoms floats, decoded by the oracle's
    restatement of read_xtc (xtc_oracle.c)."""
    lib = orc()
    lib.orc_read_xtc.restype = C.c_long
    n_frames, natoms = xtc_shape(path)
    f1 = n_frames if f1 is None else min(f1, n_frames)
    out = np.zeros((3 * natoms, f1 - f0), np.float32)
    got = lib.orc_read_xtc(str(path).encode(), C.c_size_t(f0), C.c_size_t(f1), _p(out),
                           C.c_size_t(f1 - f0))
    if got != f1 - f0:
        raise ValueError(f"orc_read_xtc: {got}")
    return np.ascontiguousarray(out.T)


def xdr_available() -> bool:
    return XDR_SO.exists()


def xdr() -> C.CDLL:
    """The reference's vendored xdrfile, compiled in place (make -C oracle ref)."""
    global _xdr
    if _xdr is None:
        lib = C.CDLL(str(XDR_SO))
        lib.xdrfile_open.restype = C.c_void_p
        lib.xdrfile_open.argtypes = [C.c_char_p, C.c_char_p]
        lib.xdrfile_close.argtypes = [C.c_void_p]
        lib.write_xtc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_void_p,
                                  C.c_void_p, C.c_float]
        lib.read_xtc.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float),
                                 C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]
        _xdr = lib
    return _xdr


def ref_write_xtc(path, rows: np.ndarray, precision: float = 1000.0) -> None:
    """XtcHandler::write for every row (coords_file.cpp:112-126): step and
    time = the row, zero box."""
    lib = xdr()
    xd = lib.xdrfile_open(str(path).encode(), b"w")
    box = np.zeros((3, 3), np.float32)
    for r, row in enumerate(np.asarray(rows, np.float32)):
        x = np.ascontiguousarray(row.reshape(-1, 3))
        lib.write_xtc(xd, x.shape[0], r, float(r), _p(box), _p(x), precision)
    lib.xdrfile_close(xd)


def ref_read_xtc(path, natoms: int) -> np.ndarray:
    """XtcHandler::next until it reports the end (coords_file.cpp:90-110)."""
    lib = xdr()
    xd = lib.xdrfile_open(str(path).encode(), b"r")
    box = np.zeros((3, 3), np.float32)
    x = np.zeros((natoms, 3), np.float32)
    step, t, p = C.c_int(), C.c_float(), C.c_float()
    out = []
    while lib.read_xtc(xd, natoms, C.byref(step), C.byref(t), _p(box), _p(x), C.byref(p)) == 0:
        out.append(x.reshape(-1).copy())
    lib.xdrfile_close(xd)
    return np.array(out, np.float32).reshape(len(out), 3 * natoms)
