"""Generates normal_rational.h: the FP32 upper-tail normal approximation.

Method (our own fit, not a library's constants): the upper tail of the standard
normal is written Q(z) = phi(z) * R(z) with R the Mills ratio, and R on
z in [0, inf) is approximated by a rational function P(z)/S(z) of degree (2, 3)
with S monic. The coefficients minimise the weighted maximum error
max_z phi(z) * |R(z) - P(z)/S(z)|, i.e. the absolute error of Q, by Loeb's
iteration: each step solves the linear program
    min t  s.t.  |phi(z_k) (R(z_k) S(z_k) - P(z_k))| / |S_prev(z_k)| <= t
on a dense grid and re-weights with the new denominator. The fitted
coefficients come out all positive, so Horner evaluation in FP32 is
well-conditioned for z >= 0 and S has no root on z >= 0.

The reference for R is scipy.special.erfcx: R(z) = sqrt(pi/2) * erfcx(z / sqrt 2).

Run:  python massivemds_gb300/csrc/normal_rational_fit.py   (rewrites the header)
"""
from __future__ import annotations

import os

import numpy as np
from scipy.optimize import linprog
from scipy.special import erfcx

DEG_P, DEG_S = 2, 3


def mills(z):
    return np.sqrt(np.pi / 2.0) * erfcx(z / np.sqrt(2.0))


def fit(m=DEG_P, k=DEG_S, iters=40):
    z = np.concatenate([np.linspace(0.0, 8.0, 8001), np.linspace(8.0, 40.0, 801)])
    w = np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)
    r = mills(z)
    s_prev = np.ones_like(z)
    best = None
    vp = np.vander(z, m + 1, increasing=True)
    vs = np.vander(z, k, increasing=True)
    lead = z ** k
    for _ in range(iters):
        sc = w / np.abs(s_prev)
        a = np.hstack([-vp * sc[:, None], (r[:, None] * vs) * sc[:, None]])
        b = -(r * lead) * sc
        nv = m + 1 + k
        a_ub = np.vstack([np.hstack([a, -np.ones((len(z), 1))]), np.hstack([-a, -np.ones((len(z), 1))])])
        b_ub = np.concatenate([b, -b])
        c = np.zeros(nv + 1)
        c[-1] = 1.0
        res = linprog(c, A_ub=a_ub, b_ub=b_ub, bounds=[(None, None)] * nv + [(0, None)], method="highs")
        if res.status != 0:
            break
        p = res.x[: m + 1]
        s = np.concatenate([res.x[m + 1: nv], [1.0]])
        sv = np.polyval(s[::-1], z)
        err = float(np.max(w * np.abs(r - np.polyval(p[::-1], z) / sv)))
        if best is None or err < best[0]:
            best = (err, p.copy(), s.copy())
        s_prev = sv
    return best


def main():
    err, p, s = fit()
    assert np.all(p > 0) and np.all(s > 0), "fit lost positivity"
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "normal_rational.h")
    with open(out, "w") as f:
        f.write("// Generated by normal_rational_fit.py; do not edit by hand.\n")
        f.write("//\n")
        f.write("// Upper normal tail Q(z) = phi(z) * P(z) / S(z) for z >= 0, with\n")
        f.write("// P(z) = p0 + p1 z + p2 z^2 and S(z) = s0 + s1 z + s2 z^2 + z^3 (monic).\n")
        f.write(f"// Weighted minimax fit (Loeb iteration); max |Q - approx| = {err:.3e} over z >= 0.\n")
        f.write("#pragma once\n\n")
        f.write("namespace mdsx {\n")
        f.write(f"constexpr double kTailMaxAbsError = {err:.6e};\n")
        for i, v in enumerate(p):
            f.write(f"constexpr double kTailP{i} = {float(v)!r};\n")
        for i, v in enumerate(s[:-1]):
            f.write(f"constexpr double kTailS{i} = {float(v)!r};\n")
        f.write("}  // namespace mdsx\n")
    print(f"wrote {out}: max abs error {err:.3e}")


if __name__ == "__main__":
    main()
