"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (no public dataset is available offline).

All generators use numpy's PCG64 (``default_rng(seed)``), whose streams are
identical on x86-64 and aarch64, so an object file regenerated on the GPU
host is byte-identical to the one the reference indexed here.
"""
from __future__ import annotations

import numpy as np


def clipped_exponential(n: int, dim: int, seed: int, mean: float = 25.0) -> np.ndarray:
    """Coordinates min(255, rint(Exponential(mean))) as float32 (integer valued)."""
    rng = np.random.default_rng(seed)
    return np.minimum(255.0, np.rint(rng.exponential(mean, size=(n, dim)))).astype(np.float32)


def gaussian_mixture(n: int, dim: int, nclusters: int, seed_means: int, seed: int, sigma: float = 0.5,
                     normalize: bool = False) -> np.ndarray:
    """Points drawn around `nclusters` N(0,1) means with per-coordinate sigma."""
    means = np.random.default_rng(seed_means).standard_normal((nclusters, dim)).astype(np.float32)
    rng = np.random.default_rng(seed)
    lab = rng.integers(0, nclusters, size=n)
    x = means[lab] + sigma * rng.standard_normal((n, dim)).astype(np.float32)
    x = x.astype(np.float32)
    if normalize:
        x /= np.linalg.norm(x, axis=1, keepdims=True).astype(np.float32)
    return x


def lowrank_bytes(n: int, dim: int, rank: int, seed_basis: int, seed: int, spread: float = 10.0,
                  chunk: int = 1 << 20) -> np.ndarray:
    """uint8 points of low intrinsic dimension: 128 + A z, z ~ N(0, I_rank), A a fixed
    dim x rank matrix of N(0, spread^2) entries, rounded and clipped to [0, 255];
    generated in chunks."""
    a = np.random.default_rng(seed_basis).standard_normal((rank, dim)).astype(np.float32) * spread
    rng = np.random.default_rng(seed)
    out = np.empty((n, dim), np.uint8)
    for s0 in range(0, n, chunk):
        m = min(chunk, n - s0)
        z = rng.standard_normal((m, rank), dtype=np.float32)
        out[s0:s0 + m] = np.clip(np.rint(128.0 + z @ a), 0, 255).astype(np.uint8)
    return out


def random_bytes(n: int, dim: int, seed: int, p_one: float = 0.5) -> np.ndarray:
    """uint8 vectors whose bits are 1 with probability p_one (for Hamming / Jaccard)."""
    rng = np.random.default_rng(seed)
    bits = (rng.random((n, dim * 8)) < p_one).astype(np.uint8)
    return np.packbits(bits, axis=1, bitorder="little").astype(np.float32)


def poincare_ball(n: int, dim: int, nclusters: int, seed_means: int, seed: int) -> np.ndarray:
    """Gaussian-mixture points mapped into the open unit ball (x / (1 + |x|) x 0.9),
    valid objects of a Poincare index."""
    x = gaussian_mixture(n, dim, nclusters, seed_means, seed).astype(np.float64)
    x *= 0.9 / (1.0 + np.linalg.norm(x, axis=1, keepdims=True))
    return x.astype(np.float32)


def lorentz_hyperboloid(n: int, dim: int, nclusters: int, seed_means: int, seed: int) -> np.ndarray:
    """Points of the hyperboloid x0 = sqrt(1 + |x_rest|^2) (x_rest a scaled Gaussian
    mixture of dim - 1 coordinates), valid objects of a Lorentz index."""
    y = 0.5 * gaussian_mixture(n, dim - 1, nclusters, seed_means, seed).astype(np.float64)
    x0 = np.sqrt(1.0 + (y * y).sum(1, keepdims=True))
    return np.concatenate([x0, y], axis=1).astype(np.float32)
