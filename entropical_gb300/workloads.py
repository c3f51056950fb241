"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is referenced by the reference; every workload here is generated
from a seed with the sizes and distributions of the five configurations:

1. ``gmm_1d``          -- 1-D three-component Gaussian mixture, N=20,000, h=0.1
2. ``mi_coords``       -- 64 coordinates x 100,000 frames, tanh(A z_t) of a
                          16-dim AR(1) process, columns standardised
3. ``langevin``        -- 32 coupled double-well Langevin coordinates x 200,000
                          Euler-Maruyama steps (transfer entropy)
4. ``uneven_batch``    -- 512 mixtures, d in {1,2,3}, N log-uniform 2k..500k
5. ``mixture_instance``-- the mixture generator behind 4 (and the training set
                          of the learned bandwidth model)

All arrays are float32 in the reference's column-major layout, i.e. shape
(n_coords, n_frames).
"""
from __future__ import annotations

import numpy as np

try:  # scipy is present on the build and the GPU hosts
    from scipy.signal import lfilter
except Exception:  # pragma: no cover
    lfilter = None


def gmm_1d(n: int = 20_000, seed: int = 42) -> np.ndarray:
    """Config 1: means (-1.0, 0.2, 1.5), sd 0.3, weights (0.3, 0.4, 0.3)."""
    rng = np.random.default_rng(seed)
    comp = rng.choice(3, size=n, p=[0.3, 0.4, 0.3])
    means = np.array([-1.0, 0.2, 1.5])
    return (means[comp] + 0.3 * rng.standard_normal(n)).astype(np.float32)


def _ar1(n: int, dim: int, phi: float, rng: np.random.Generator) -> np.ndarray:
    e = rng.standard_normal((n, dim))
    z0 = rng.standard_normal(dim) / np.sqrt(1.0 - phi * phi)
    if lfilter is not None:
        return lfilter([1.0], [1.0, -phi], e, axis=0, zi=(phi * z0)[None, :])[0]
    z = np.empty((n, dim))
    prev = z0
    for t in range(n):
        prev = phi * prev + e[t]
        z[t] = prev
    return z


def mi_coords(n_frames: int = 100_000, n_coords: int = 64, latent: int = 16,
              phi: float = 0.95, seed: int = 2024) -> np.ndarray:
    """Config 2: x_t = tanh(A z_t), z a unit-innovation AR(1) (phi), A ~ N(0,1),
    each column standardised (mean 0, sd 1)."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n_coords, latent))
    z = _ar1(n_frames, latent, phi, rng)
    x = np.tanh(z @ a.T)  # (n_frames, n_coords)
    x = (x - x.mean(axis=0)) / x.std(axis=0)
    return np.ascontiguousarray(x.T.astype(np.float32))


def scott_bandwidth(x: np.ndarray, d: int) -> np.ndarray:
    """Scott's rule h = sigma * n^(-1/(d+4)) for every row of x (n_coords, n)."""
    x = np.atleast_2d(np.asarray(x, dtype=np.float64))
    n = x.shape[1]
    return (x.std(axis=1) * n ** (-1.0 / (d + 4))).astype(np.float32)


def langevin(n_coords: int = 32, n_steps: int = 200_000, dt: float = 0.01,
             noise: float = 0.5, density: float = 0.1, seed: int = 11) -> tuple[np.ndarray, np.ndarray]:
    """Config 3: dx_i = (x_i - x_i^3 + sum_j C_ij x_j) dt + noise dW_i,
    C sparse (density 0.1, entries U(-0.3, 0.3), zero diagonal). Returns
    (trajectory (n_coords, n_steps) float32, C)."""
    rng = np.random.default_rng(seed)
    c = np.where(rng.random((n_coords, n_coords)) < density,
                 rng.uniform(-0.3, 0.3, (n_coords, n_coords)), 0.0)
    np.fill_diagonal(c, 0.0)
    x = rng.choice([-1.0, 1.0], n_coords) + 0.1 * rng.standard_normal(n_coords)
    out = np.empty((n_steps, n_coords), dtype=np.float32)
    sq = noise * np.sqrt(dt)
    block = 4096
    for t0 in range(0, n_steps, block):
        dw = rng.standard_normal((min(block, n_steps - t0), n_coords)) * sq
        for k in range(dw.shape[0]):
            x = x + (x - x * x * x + c @ x) * dt + dw[k]
            out[t0 + k] = x
    return np.ascontiguousarray(out.T), c


def mixture_instance(rng: np.random.Generator, d: int, n: int) -> np.ndarray:
    """One mixture: 1-6 components, means U(-2,2), sd U(0.1,0.8) per dim,
    Dirichlet(1) weights. Returns (d, n) float32."""
    k = int(rng.integers(1, 7))
    w = rng.dirichlet(np.ones(k))
    mu = rng.uniform(-2.0, 2.0, (k, d))
    sd = rng.uniform(0.1, 0.8, (k, d))
    comp = rng.choice(k, size=n, p=w)
    x = mu[comp] + sd[comp] * rng.standard_normal((n, d))
    return np.ascontiguousarray(x.T.astype(np.float32))


def uneven_batch(n_inst: int = 512, n_min: int = 2_000, n_max: int = 500_000,
                 seed: int = 5) -> list[tuple[np.ndarray, np.ndarray]]:
    """Config 4: n_inst instances, d ~ U{1,2,3}, N log-uniform in [n_min, n_max];
    returns [(coords (d, n) float32, Scott bandwidths (d,) float32)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_inst):
        d = int(rng.integers(1, 4))
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        x = mixture_instance(rng, d, n)
        out.append((x, scott_bandwidth(x, d)))
    return out
