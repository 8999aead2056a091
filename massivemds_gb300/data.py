"""Seeded synthetic inputs with the shapes of the MassiveMDS workloads.

The reference publishes no benchmark dataset for this path; its own benchmark
draws delta as mirrored squared normals (src/benchmark.cpp:174-189). The
workloads here use Euclidean dissimilarities of latent points instead:

* ``euclidean_delta(n, dim, seed)``: delta_ij = ||Y_i - Y_j||, Y ~ N(0, I_dim),
  symmetric, zero diagonal (the N=1000 FP64 workload).
* ``noisy_delta(n, dim, noise_sd, seed)``: the same plus iid N(0, noise_sd^2)
  noise drawn once per unordered pair, mirrored, clipped at 0 (the N=20 000 workload).
* ``clustered_delta(...)``: points in Gaussian clusters plus noise (the HMC workload).

Large matrices are built in row blocks in float32 or float64 without an N x N
temporary of doubles.
"""
from __future__ import annotations

import numpy as np


def latent_points(n: int, dim: int, seed: int, centres: int = 0, centre_scale: float = 3.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, dim))
    if centres:
        c = centre_scale * rng.standard_normal((centres, dim))
        y += c[np.arange(n) % centres]
    return y


def pairwise_distances(y: np.ndarray, dtype=np.float64, block: int = 2048) -> np.ndarray:
    """||y_i - y_j|| in blocks of rows (exact zero diagonal)."""
    n = y.shape[0]
    out = np.empty((n, n), dtype=dtype)
    sq = np.einsum("ij,ij->i", y, y)
    for r0 in range(0, n, block):
        r1 = min(n, r0 + block)
        g = sq[r0:r1, None] + sq[None, :] - 2.0 * (y[r0:r1] @ y.T)
        np.maximum(g, 0.0, out=g)
        d = np.sqrt(g)
        # recompute near-diagonal / small entries exactly to avoid cancellation
        small = g < 1e-6 * (sq[r0:r1, None] + sq[None, :] + 1.0)
        if small.any():
            ii, jj = np.nonzero(small)
            diff = y[r0 + ii] - y[jj]
            d[ii, jj] = np.sqrt(np.einsum("ij,ij->i", diff, diff))
        idx = np.arange(r0, r1)
        d[idx - r0, idx] = 0.0
        out[r0:r1] = d
    return out


def symmetric_from_upper(d: np.ndarray, noise: np.ndarray | None = None, clip: bool = False,
                         block: int = 1024) -> np.ndarray:
    """A new matrix whose (i, j) and (j, i) entries both come from the upper
    triangle (i < j) of d (+ noise), optionally clipped at 0; zero diagonal."""
    n = d.shape[0]
    out = np.empty_like(d)
    for r0 in range(0, n, block):
        r1 = min(n, r0 + block)
        upper = np.arange(n)[None, :] > np.arange(r0, r1)[:, None]
        blk = np.where(upper, d[r0:r1], d[:, r0:r1].T)
        if noise is not None:
            blk = blk + np.where(upper, noise[r0:r1], noise[:, r0:r1].T).astype(d.dtype)
        if clip:
            np.maximum(blk, 0, out=blk)
        blk[np.arange(r1 - r0), np.arange(r0, r1)] = 0
        out[r0:r1] = blk
    return out


def add_symmetric_noise(delta: np.ndarray, sd: float, seed: int) -> np.ndarray:
    """delta_ij + eps_ij with eps drawn once per unordered pair (i < j) and
    mirrored, clipped at 0, zero diagonal (returns a new array)."""
    n = delta.shape[0]
    rng = np.random.default_rng(seed)
    eps = rng.standard_normal((n, n), dtype=np.float32)  # entries with i < j are used
    eps *= np.float32(sd)
    return symmetric_from_upper(delta, eps, clip=True)


def euclidean_delta(n: int, dim: int = 10, seed: int = 666, dtype=np.float64) -> np.ndarray:
    return symmetric_from_upper(pairwise_distances(latent_points(n, dim, seed), dtype=dtype))


def noisy_delta(n: int, dim: int = 10, noise_sd: float = 0.05, seed: int = 666, dtype=np.float32) -> np.ndarray:
    d = pairwise_distances(latent_points(n, dim, seed), dtype=dtype)
    return add_symmetric_noise(d, noise_sd, seed + 1)


def clustered_delta(n: int, dim: int = 10, clusters: int = 5, noise_sd: float = 0.1, seed: int = 666,
                    dtype=np.float32) -> np.ndarray:
    y = latent_points(n, dim, seed, centres=clusters, centre_scale=3.0)
    d = pairwise_distances(y, dtype=dtype)
    return add_symmetric_noise(d, noise_sd, seed + 1)


def locations(n: int, p: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal((n, p))


def classical_mds(delta: np.ndarray, p: int, iterations: int = 60, seed: int = 0) -> np.ndarray:
    """Classical (Torgerson) MDS start: the top-p eigenvectors of
    B = -1/2 J delta^2 J by subspace iteration, scaled by the square roots of
    their eigenvalues. Used only to start chains near the posterior mode."""
    n = delta.shape[0]
    d2 = np.square(delta, dtype=np.float32)

    def bmul(v):
        v = v - v.mean(0)
        w = d2 @ v.astype(np.float32)
        w = w.astype(np.float64)
        return -0.5 * (w - w.mean(0))

    v = np.linalg.qr(np.random.default_rng(seed).standard_normal((n, p)))[0]
    for _ in range(iterations):
        v = np.linalg.qr(bmul(v))[0]
    lam = np.maximum(np.einsum("ip,ip->p", v, bmul(v)), 0.0)
    return v * np.sqrt(lam)
