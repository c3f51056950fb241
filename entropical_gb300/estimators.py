"""The reference estimators' own formulas over GPU densities.

These mirror the host loops of the reference's estimator mains -- mi.cpp:37-59,
transs.cpp:39-115, autoent.cpp:39-58, negs.cpp:36-47, kldiv.cpp:36-54,
dens.cpp:19-106 -- calling the density interface as they do (one
combined_densities call per density, normalised by the original n_rows as
the reference CUDA build does, densities_cuda.cu:98-103) and reducing on the
host with the same formulas, including the float log of tools.cpp:18-37, the
Kahan normalisation of tools.hxx:33-43 and the Y->X weight of transs.cpp:96.
They give the reference's numbers; the batched, resubstitution estimators
are Context.mi_all_pairs / te_all_pairs / entropy_batch.

By default (batched=True) each estimator is one device batch through
ent_reference_estimator / ent_dens_all (all densities in one engine batch,
FP64 sums on the device); batched=False keeps the reference's loop structure,
one density call per density and the sums on the host.
"""
from __future__ import annotations

import numpy as np

from .densities import (REF_AUTOENT, REF_KLDIV, REF_MI, REF_NEGS, REF_TRANSS, Context,
                        as_colmajor)


def _flog(x):
    """Tools::select_log(false): float log, 0 at 0 (tools.cpp:29-35)."""
    x32 = np.asarray(x, dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = np.where(x32 == 0, np.float32(0), np.log(x32)).astype(np.float32)
    return out


def _kahan(xs) -> float:
    s = c = 0.0
    for x in np.asarray(xs, dtype=np.float64):
        y = x - c
        t = s + y
        c = (t - s) - y
        s = t
    return s


def sum1_normalized(xs):
    """Tools::sum1_normalized (tools.hxx:33-43)."""
    xs = np.asarray(xs, dtype=np.float64)
    s = _kahan(xs)
    return xs / s if s != 0 else xs


def _inv(x):
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(divide="ignore"):
        return np.where(x == 0, x, 1.0 / x)


class ReferenceEstimators:
    """The reference's estimators (compat formulas) on a Context."""

    def __init__(self, ctx: Context, batched: bool = True):
        self.ctx = ctx
        self.batched = batched

    def _dens(self, x, cols, h, tau=None):
        return self.ctx.combined_densities(x, None, cols, h, tau, compat_norm=True)

    def mi(self, coords, h):
        """Mi::main (mi.cpp:37-59): sum_k p_ij log(p_ij / p_i / p_j), float accumulator."""
        if self.batched:
            return self.ctx.reference_estimator(coords, h, REF_MI).astype(np.float32)
        x, n_rows, n = as_colmajor(coords)
        x = x.reshape(n, n_rows)
        out = np.zeros((n, n), np.float32)
        for i in range(n):
            p_i = self._dens(x, [i], [h[i]])
            for j in range(i + 1, n):
                p_j = self._dens(x, [j], [h[j]])
                p_ij = self._dens(x, [i, j], [h[i], h[j]])
                v = np.float32(np.sum(p_ij * _flog(p_ij / p_i / p_j)))
                out[i, j] = out[j, i] = v
        return out

    def transs(self, coords, h, tau: int):
        """Transs::main (transs.cpp:39-115), including the reference's weights."""
        if self.batched:
            return self.ctx.reference_estimator(coords, h, REF_TRANSS, tau)
        x, n_rows, n = as_colmajor(coords)
        x = x.reshape(n, n_rows)
        p = [self._dens(x, [i], [h[i]]) for i in range(n)]
        p_tau = [self._dens(x, [i, i], [h[i], h[i]], [0, tau]) for i in range(n)]
        out = np.zeros((n, n), np.float64)
        m = n_rows - tau
        for i in range(n):
            for j in range(i + 1, n):
                hi, hj = np.float32(h[i]), np.float32(h[j])
                p_ij = self._dens(x, [i, j], [hi, hj])
                p_itau = self._dens(x, [i, i, j], [hi, hi, hj], [0, tau, 0])
                p_jtau = self._dens(x, [i, j, j], [hi, hj, hj], [0, 0, tau])
                for (a, b, pt, w, pp, ptt) in ((i, j, p_itau, hi * hi * hj, p[i], p_tau[i]),
                                               (j, i, p_jtau, hi * hj * hi, p[j], p_tau[j])):
                    k = slice(0, m)
                    arg = pt[k] * pp[k] * _inv(p_ij[k]) * _inv(ptt[k])
                    te = pt[k] * float(w) * _flog(arg)
                    ok = (pt[k] > 0) & np.isfinite(te) & (pt[k] <= 1.0)
                    out[a, b] += np.sum(te[ok])
        return out

    def autoent(self, coords, h, tau: int):
        """AutoEnt::main (autoent.cpp:39-58)."""
        if self.batched:
            return self.ctx.reference_estimator(coords, h, REF_AUTOENT, tau)
        x, n_rows, n = as_colmajor(coords)
        x = x.reshape(n, n_rows)
        out = np.zeros(n, np.float64)
        for i in range(n):
            hh = np.float32(h[i])
            p_itau = self._dens(x, [i], [hh], [tau])
            p_ii = self._dens(x, [i, i], [hh, hh], [0, tau])
            ok = p_ii > 0
            arg = p_itau * _inv(p_ii * float(hh))
            out[i] = np.sum((p_ii * float(hh) * float(hh) * _flog(arg))[ok])
        return out

    def negs(self, coords, h):
        """Negs::main (negs.cpp:36-47): -sum_k p log p of the sum-normalised density."""
        if self.batched:
            return self.ctx.reference_estimator(coords, h, REF_NEGS).astype(np.float32)
        x, n_rows, n = as_colmajor(coords)
        x = x.reshape(n, n_rows)
        out = np.zeros(n, np.float32)
        for i in range(n):
            pk = sum1_normalized(self._dens(x, [i], [h[i]]))
            out[i] = -np.float32(np.sum(_flog(pk) * pk))
        return out

    def kldiv(self, coords, h):
        """KLDiv::main (kldiv.cpp:36-54)."""
        if self.batched:
            return self.ctx.reference_estimator(coords, h, REF_KLDIV)
        x, n_rows, n = as_colmajor(coords)
        x = x.reshape(n, n_rows)
        ps = [sum1_normalized(self._dens(x, [i], [h[i]])) for i in range(n)]
        out = np.zeros((n, n), np.float64)
        for i in range(n):
            for j in range(i + 1, n):
                out[i, j] = np.sum(ps[i] * _flog(ps[i] / ps[j]))
                out[j, i] = np.sum(ps[j] * _flog(ps[j] / ps[i]))
        return out

    def dens_1d(self, coords, h):
        """Dens::compute_densities_1d (dens.cpp:19-47): sum-normalised density of
        every column, concatenated."""
        if self.batched:
            return self.ctx.dens_all(coords, h, 1).reshape(-1)
        x, n_rows, n = as_colmajor(coords)
        x = x.reshape(n, n_rows)
        return np.concatenate([sum1_normalized(self._dens(x, [i], [h[i]])) for i in range(n)])

    def dens_nd(self, coords, h, dims: int, taus=None):
        """Dens::compute_densities_nd (dens.cpp:49-106): sum-normalised densities of
        all column pairs (dims=2) or triples (dims=3), concatenated in the
        reference's order."""
        if self.batched:
            return self.ctx.dens_all(coords, h, dims, taus).reshape(-1)
        x, n_rows, n = as_colmajor(coords)
        x = x.reshape(n, n_rows)
        taus = [0] * dims if taus is None else list(taus)
        out = []
        for i in range(n):
            for j in range(i + 1, n):
                if dims == 2:
                    out.append(sum1_normalized(self._dens(x, [i, j], [h[i], h[j]], taus)))
                else:
                    for k in range(j + 1, n):
                        out.append(sum1_normalized(
                            self._dens(x, [i, j, k], [h[i], h[j], h[k]], taus)))
        return np.concatenate(out)


def _f32(v) -> np.float32:
    return np.float32(v)


def amise_from_conv(conv: float, h: float, n: int) -> np.float32:
    """AmiseMin::_amise (hestimate.cpp:41-53) with its float/double mix."""
    a = _f32(0.04 * 1 / np.float64(_f32(h)) ** 5 * np.float64(_f32(conv)))
    a = _f32(np.float64(a) ** 0.2)
    return _f32(np.float64(a) * 1.25 * 0.6 ** 0.8 / np.float64(_f32(n)) ** 0.8)


def hestimate_amise_plain(ctx: Context, col, h0: float) -> tuple[float, int]:
    """AmiseMin::operator() (hestimate.cpp:88-104) driven through the plain
    single-instance entry point: one epa_convolution call per AMISE
    evaluation, the bracket recursion (:55-86) on the host. Returns (h, calls)."""
    col = np.ascontiguousarray(np.asarray(col, np.float32).ravel())
    n = col.size
    calls = 0

    def amise(h):
        nonlocal calls
        calls += 1
        return amise_from_conv(ctx.epa_convolution(col, float(h)), h, n)

    h0 = _f32(h0)
    prec = _f32(0.01 * np.float64(h0))
    lo = _f32(0.1 * np.float64(h0))
    hi = _f32(2 * h0)
    it = 20
    while True:
        delta = _f32(hi - lo)
        pivot = _f32(np.float64(lo) + 0.5 * np.float64(delta))
        if it == 0 or delta <= prec:
            return float(pivot), calls
        pl = _f32(np.float64(pivot) - 0.25 * np.float64(delta))
        ph = _f32(np.float64(pivot) + 0.25 * np.float64(delta))
        if amise(pl) < amise(ph):
            hi = pivot
        else:
            lo = pivot
        it -= 1
