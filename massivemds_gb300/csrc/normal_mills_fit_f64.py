"""Generates normal_mills_f64.h: the FP64 upper-tail normal approximation.

Method (our own fit, not a library's constants): the upper tail of the standard
normal is Q(z) = phi(z) * R(z) with R the Mills ratio; on z in [0, Z_CLAMP]
R is approximated by P(z) / S(z) of degree (DEG, DEG) with S(0) = 1. The
coefficients minimise the weighted maximum error

    max_z phi(z) * |R(z) - P(z) / S(z)|,

the absolute error of Q and hence of Phi = 1 - Q, by Loeb's linearisation
(each step a weighted least-squares problem in which the residual
phi (R S - P) is divided by the previous denominator) with Lawson's
re-weighting towards the minimax solution, in 50-digit arithmetic (mpmath).
Beyond Z_CLAMP the kernels evaluate the fit at Z_CLAMP: there Q < 1e-17, so Phi
is 1 to double precision whatever the ratio.

The reference for R is R(z) = sqrt(pi/2) * exp(z^2 / 2) * erfc(z / sqrt 2)
in mpmath. The generated header states the fit's error measured in double
arithmetic (Horner, one division) on a dense grid.

Run:  python massivemds_gb300/csrc/normal_mills_fit_f64.py   (rewrites the header)
"""
from __future__ import annotations

import os

import mpmath as mp
import numpy as np

DEG = 6
Z_CLAMP = 8.5
mp.mp.dps = 50


def mills(z):
    z = mp.mpf(z)
    return mp.sqrt(mp.pi / 2) * mp.exp(z * z / 2) * mp.erfc(z / mp.sqrt(2))


def phi(z):
    z = mp.mpf(z)
    return mp.exp(-z * z / 2) / mp.sqrt(2 * mp.pi)


def horner(c, z):
    acc = mp.mpf(0)
    for a in reversed(c):
        acc = acc * z + a
    return acc


def fit(deg=DEG, points=600, iters=60):
    # Chebyshev nodes on [0, Z_CLAMP] plus both ends
    zs = [mp.mpf(Z_CLAMP) * (1 - mp.cos(mp.pi * (k + mp.mpf(1) / 2) / points)) / 2 for k in range(points)]
    zs = [mp.mpf(0)] + zs + [mp.mpf(Z_CLAMP)]
    rs = [mills(z) for z in zs]
    ws = [phi(z) for z in zs]
    s_prev = [mp.mpf(1)] * len(zs)
    v = [mp.mpf(1)] * len(zs)
    best = None
    nu = (deg + 1) + deg  # p0..p_deg, s1..s_deg (s0 = 1)
    for _ in range(iters):
        # rows: sqrt(v) * w / s_prev * (R * (1 + sum s_j z^j) - sum p_i z^i)
        a = mp.matrix(len(zs), nu)
        b = mp.matrix(len(zs), 1)
        for k, (z, r, w) in enumerate(zip(zs, rs, ws)):
            sc = mp.sqrt(v[k]) * w / s_prev[k]
            zp = mp.mpf(1)
            for i in range(deg + 1):
                a[k, i] = -sc * zp
                zp *= z
            zp = z
            for j in range(deg):
                a[k, deg + 1 + j] = sc * r * zp
                zp *= z
            b[k] = -sc * r
        ata = a.T * a
        atb = a.T * b
        x = mp.lu_solve(ata, atb)
        p = [x[i] for i in range(deg + 1)]
        s = [mp.mpf(1)] + [x[deg + 1 + j] for j in range(deg)]
        sv = [horner(s, z) for z in zs]
        err = [w * abs(r - horner(p, z) / sd) for z, r, w, sd in zip(zs, rs, ws, sv)]
        e_max = max(err)
        if best is None or e_max < best[0]:
            best = (e_max, p, s)
        tot = mp.fsum(vk * ek for vk, ek in zip(v, err))
        v = [vk * ek / tot for vk, ek in zip(v, err)]
        s_prev = sv
    return best


def check_double(p, s, n=200001):
    """Max |Q_fit - Q| over z in [0, 12] with the fit evaluated in double
    arithmetic as the kernels do (Horner on min(z, Z_CLAMP), one division)."""
    pd = np.array([float(c) for c in p])
    sd = np.array([float(c) for c in s])
    z = np.linspace(0.0, 12.0, n)
    zc = np.minimum(z, Z_CLAMP)
    num = np.zeros_like(zc)
    den = np.zeros_like(zc)
    for c in pd[::-1]:
        num = num * zc + c
    for c in sd[::-1]:
        den = den * zc + c
    q_fit = (np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)) * (num / den)
    q_ref = np.array([float(mp.erfc(mp.mpf(t) / mp.sqrt(2)) / 2) for t in z[::20]])
    err = np.abs(q_fit[::20] - q_ref)
    return float(err.max()), float(z[::20][err.argmax()]), bool(np.all(den > 0)), bool(np.all(pd > 0) and np.all(sd > 0))


def main():
    e_max, p, s = fit()
    d_err, z_at, den_pos, all_pos = check_double(p, s)
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "normal_mills_f64.h"), "w") as f:
        f.write("// Generated by normal_mills_fit_f64.py: FP64 upper-tail normal approximation.\n")
        f.write(f"// Q(z) = phi(z) * P(min(z, {Z_CLAMP})) / S(min(z, {Z_CLAMP})), degree ({DEG}, {DEG}), S(0) = 1;\n")
        f.write(f"// our weighted-minimax fit of the Mills ratio (Loeb + Lawson, 50 digits):\n")
        f.write(f"// max |Q_fit - Q| = {float(e_max):.2e} in exact arithmetic on [0, {Z_CLAMP}],\n")
        f.write(f"// {d_err:.2e} (at z = {z_at:.3f}) evaluated in double on [0, 12];\n")
        f.write(f"// S > 0 on the grid: {den_pos}; all coefficients positive: {all_pos}.\n")
        f.write("#pragma once\n\n#include <cmath>\n\nnamespace mdsx {\n\n")
        f.write(f"constexpr double kMillsClamp = {Z_CLAMP!r};\n\n")

        def horner_src(c, var):
            src = mp.nstr(c[-1], 20, min_fixed=-1, max_fixed=-1)
            for a in reversed(c[:-1]):
                src = f"fma({src}, {var}, {mp.nstr(a, 20, min_fixed=-1, max_fixed=-1)})"
            return src

        f.write("// P(z) and S(z) for 0 <= z <= kMillsClamp (Horner, all coefficients positive).\n")
        f.write("__host__ __device__ inline void mills_ratio_f64(double z, double& num, double& den) {\n")
        f.write(f"    num = {horner_src(p, 'z')};\n")
        f.write(f"    den = {horner_src(s, 'z')};\n")
        f.write("}\n\n}  // namespace mdsx\n")
    print(f"exact max err {float(e_max):.3e}; double max err {d_err:.3e} at z={z_at:.3f}; S>0 {den_pos}; positive {all_pos}")


if __name__ == "__main__":
    main()
