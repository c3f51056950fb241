"""Host-side check of the integer identities behind the exact range sums
(1-D) and strip moments (2-D): with coordinates in fixed point (Y = y 2^F,
rounded) and every sum and product taken modulo 2^128, the polynomial
identities return the exact integer sum of the kernel over a range, for data
with large offsets, ties, outliers and tiny spreads. Python integers restate
the device arithmetic (the kernels use unsigned __int128); the reference is
the direct FP64 sum of the same kernel terms on the same float inputs."""
import struct

import numpy as np
import pytest

M128 = 1 << 128


def quant(v: float, F: int) -> int:
    """round(v 2^F) modulo 2^128 from the float32 bits (zero for subnormals)."""
    b = struct.unpack("<I", struct.pack("<f", float(v)))[0]
    e = (b >> 23) & 0xFF
    if e == 0:
        return 0
    m = (b & 0x7FFFFF) | 0x800000
    sh = e - 150 + F
    if sh >= 128:
        q = 0
    elif sh >= 0:
        q = (m << sh) % M128
    elif sh > -25:
        q = (m + (1 << (-sh - 1))) >> (-sh)
    else:
        q = 0
    return (-q) % M128 if b >> 31 else q


def signed(v: int) -> int:
    v %= M128
    return v - M128 if v >> 127 else v


def range_sum_1d(y, k, lo, hi, g2):
    """sum_{j in [lo, hi)} (g2 - (y_j - y_k)^2) by prefix sums of Y and Y^2."""
    k, lo, hi = int(k), int(lo), int(hi)
    Y = [quant(v, 46) for v in y]
    sy = sum(Y[lo:hi]) % M128
    sy2 = sum(v * v for v in Y[lo:hi]) % M128
    c = hi - lo
    q = (sy2 - 2 * Y[k] * sy + c * Y[k] * Y[k]) % M128
    assert signed(q) >= 0 and signed(q) < 1 << 124
    return c * float(g2) - signed(q) * 2.0 ** -92


def strip_sum_2d(x, y, t, idx, g1, g2):
    """sum over idx of (g1 - (x - x_t)^2)(g2 - (y - y_t)^2) by the eight
    moments of X = x 2^23, Y = y 2^23 and G = g^2 2^46."""
    t = int(t)
    TX, TY = quant(x[t], 23), quant(y[t], 23)
    mo = [0] * 9  # index 3a + b: sum X^a Y^b
    for j in map(int, idx):
        X, Y = quant(x[j], 23), quant(y[j], 23)
        for a in range(3):
            for b in range(3):
                mo[3 * a + b] = (mo[3 * a + b] + X ** a * Y ** b) % M128
    c = [(quant(g1, 46) - TX * TX) % M128, 2 * TX % M128, M128 - 1]
    d = [(quant(g2, 46) - TY * TY) % M128, 2 * TY % M128, M128 - 1]
    ex = sum(c[a] * d[b] * mo[3 * a + b] for a in range(3) for b in range(3)) % M128
    assert abs(signed(ex)) < 1 << 124
    return signed(ex) * 2.0 ** -92


def _data(kind, rng, n):
    base = rng.normal(0.0, 3.0, n)
    if kind == "offset":
        base = base + 5e5
    elif kind == "ties":
        base = np.round(base, 1)
    elif kind == "outlier":
        base = np.concatenate([base[:-2], [1e30, -3e25]])
    elif kind == "narrow":
        base = rng.normal(2.0, 1e-6, n)
    return np.sort(base.astype(np.float32))


@pytest.mark.parametrize("kind", ["plain", "offset", "ties", "outlier", "narrow"])
def test_range_sum_1d_is_exact(kind):
    rng = np.random.default_rng(3)
    y = _data(kind, rng, 300)
    g = np.float32(0.75)
    g2 = np.float32(g * g)
    for k in rng.choice(len(y), 20, replace=False):
        d = (y - y[k]).astype(np.float32)
        inside = (np.float64(g2) - d.astype(np.float64) ** 2) > 0
        lo, hi = np.flatnonzero(inside)[[0, -1]]
        got = range_sum_1d(y, k, lo, hi + 1, g2)
        ref = sum(float(g2) - (float(y[j]) - float(y[k])) ** 2 for j in range(lo, hi + 1))
        assert abs(got - ref) <= 1e-12 * max(ref, 1.0)


@pytest.mark.parametrize("kind", ["plain", "offset", "ties", "outlier", "narrow"])
def test_strip_sum_2d_is_exact_to_fixed_point(kind):
    rng = np.random.default_rng(5)
    x = _data(kind, rng, 200)
    y = _data(kind, rng, 200)
    rng.shuffle(y)
    g1, g2 = np.float32(0.7) ** 2, np.float32(0.9) ** 2
    for t in rng.choice(len(x), 10, replace=False):
        dx = np.abs(x.astype(np.float64) - float(x[t]))
        dy = np.abs(y.astype(np.float64) - float(y[t]))
        idx = np.flatnonzero((dx ** 2 < float(g1)) & (dy ** 2 < float(g2)))
        got = strip_sum_2d(x, y, t, idx, g1, g2)
        ref = sum((float(g1) - dx[j] ** 2) * (float(g2) - dy[j] ** 2) for j in idx)
        # fixed point at 2^-23: at most ~2^-21 g^2 per dimension and pair
        assert abs(got - ref) <= 2.0 ** -19 * len(idx) + 1e-12 * ref


def test_quant_is_a_ring_map_on_differences():
    """Differences of quantised coordinates equal the quantised difference
    for values on the float grid, whatever their magnitude (mod 2^128)."""
    for a, b in [(1e30, 1e30 + 2 ** 76), (-3.5, 2.25), (5e5, 5e5 + 0.03125), (1e-9, 0.0)]:
        a32, b32 = np.float32(a), np.float32(b)
        diff = (quant(b32, 23) - quant(a32, 23)) % M128
        exact = int(round((float(b32) - float(a32)) * 2 ** 23)) % M128
        assert abs(signed(diff - exact)) <= 1
