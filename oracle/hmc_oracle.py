"""Test infrastructure: a numpy restatement of one HMC trajectory.

Checks mdsx_hmc_run step by step. The potential is the reference's
(R/Untitled.R:427-437): U(x) = -(log-likelihood + log matrix-normal prior),
log-likelihood from the oracle (R/mds.R:24-28 assembly), prior with row
covariance I and column precision Lambda (R/Untitled.R:68-95). Momenta are
regenerated from the same counter-based generator the GPU uses: Philox4x32
with 10 rounds (Salmon, Moraes, Dror, Shaw, SC'11), counter (pair index,
iteration), key = seed, two 53-bit uniforms per normal pair through the
Box-Muller transform.
"""
from __future__ import annotations

import numpy as np

from . import oracle as _o

_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint32) for v in (c0, c1, c2, c3))
    k0, k1 = np.uint32(k0), np.uint32(k1)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = _M0 * c0.astype(np.uint64)
            p1 = _M1 * c2.astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & _MASK).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & _MASK).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0 = np.uint32(k0 + _W0)
            k1 = np.uint32(k1 + _W1)
    return c0, c1, c2, c3


def _u01(a, b):
    v = ((a >> np.uint32(5)).astype(np.uint64) << np.uint64(26)) | (b >> np.uint32(6)).astype(np.uint64)
    return (v.astype(np.float64) + 1.0) * (1.0 / 9007199254740992.0)


def momentum(count: int, seed: int, iteration: int) -> np.ndarray:
    """The count standard normals the GPU draws for one iteration."""
    pairs = np.arange((count + 1) // 2, dtype=np.uint64)
    r = philox4x32_10((pairs & _MASK).astype(np.uint32), (pairs >> np.uint64(32)).astype(np.uint32),
                      np.full(pairs.shape, iteration & 0xFFFFFFFF, np.uint32),
                      np.full(pairs.shape, (iteration >> 32) & 0xFFFFFFFF, np.uint32),
                      seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    rad = np.sqrt(-2.0 * np.log(_u01(r[0], r[1])))
    ang = 6.283185307179586476925 * _u01(r[2], r[3])
    out = np.empty(2 * pairs.size)
    out[0::2] = rad * np.cos(ang)
    out[1::2] = rad * np.sin(ang)
    return out[:count]


def log_prior(x, lam):
    n, p = x.shape
    q = np.einsum("ir,rq,iq->", x, lam, x)
    return -0.5 * q - 0.5 * n * p * np.log(2 * np.pi) + 0.5 * n * np.linalg.slogdet(lam)[1]


def potential(delta, x, tau, lam, truncation=True):
    s = _o.sum_of_increments(delta, x, tau, truncation)
    return -(_o.log_likelihood(s, x.shape[0], tau) + log_prior(x, lam))


def grad_log_post(delta, x, tau, lam, truncation=True):
    return _o.gradient(delta, x, tau, truncation) - x @ lam


def trajectory(delta, x0, tau, eps, steps, seed, iteration, lam=None, truncation=True, likelihood_gradient=None):
    """One leapfrog trajectory from x0 with the GPU's momentum; returns
    (proposal, Hamiltonian difference H(x0, p0) - H(x*, p*)).

    likelihood_gradient(x), when given, replaces the exact log-likelihood
    gradient in every kick (a surrogate); the Hamiltonian stays exact."""
    n, p = x0.shape
    lam = np.eye(p) if lam is None else lam

    def grad(x):
        if likelihood_gradient is None:
            return grad_log_post(delta, x, tau, lam, truncation)
        return likelihood_gradient(x) - x @ lam

    p0 = momentum(n * p, seed, iteration).reshape(n, p)
    x = x0.copy()
    mom = p0 + 0.5 * eps * grad(x)
    for k in range(1, steps + 1):
        x = x + eps * mom
        g = grad(x)
        mom = mom + (eps if k < steps else 0.5 * eps) * g
    h0 = potential(delta, x0, tau, lam, truncation) + 0.5 * np.sum(p0 * p0)
    h1 = potential(delta, x, tau, lam, truncation) + 0.5 * np.sum(mom * mom)
    return x, h0 - h1
