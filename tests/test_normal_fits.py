"""CPU tests of the generated normal-tail approximations the kernels evaluate:
the FP32 tail fit (normal_rational.h) and the FP64 Mills-ratio fit
(normal_mills_f64.h), read from the headers and evaluated in double, against
scipy's ndtr / ndtr-based upper tail. Pins the headers to their stated error
bounds and to the properties the kernels rely on (positive coefficients, so
Horner evaluation has no cancellation and the denominators no root for z >= 0)."""
import os
import re

import numpy as np
import pytest

sp = pytest.importorskip("scipy.special")

CSRC = os.path.join(os.path.dirname(__file__), "..", "massivemds_gb300", "csrc")
NUM = r"[-+]?\d+\.\d*(?:e[-+]?\d+)?"


def _read(name):
    with open(os.path.join(CSRC, name)) as f:
        return f.read()


def _horner_outer_first(coeffs, z):
    """Evaluates fma(fma(c0, z, c1), z, c2) ... as nested in the header's source."""
    acc = np.full_like(z, coeffs[0])
    for c in coeffs[1:]:
        acc = acc * z + c
    return acc


def _z_grid():
    rng = np.random.default_rng(5)
    return np.concatenate([np.linspace(0.0, 10.0, 100001), rng.uniform(0.0, 40.0, 50000), [38.6, 50.0, 1e3]])


def test_fp64_mills_fit_header():
    src = _read("normal_mills_f64.h")
    clamp = float(re.search(r"kMillsClamp = (" + NUM + ")", src).group(1))
    num = [float(v) for v in re.findall(NUM, re.search(r"num = (.*);", src).group(1))]
    den = [float(v) for v in re.findall(NUM, re.search(r"den = (.*);", src).group(1))]
    assert len(num) == len(den) == 7 and clamp == 8.5
    assert all(c > 0 for c in num + den)
    z = _z_grid()
    zc = np.minimum(z, clamp)
    pn, pd = _horner_outer_first(num, zc), _horner_outer_first(den, zc)
    assert np.all(pd >= 1.0)
    pdf = np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)
    cdf = 1.0 - pdf * pn / pd
    # the fit's stated error in Q is 9.4e-16 evaluated in double; ndtr adds ~1e-16
    assert np.abs(cdf - sp.ndtr(z)).max() <= 1.5e-15
    # the upper tail itself, relative, where Q matters (Q >= 1e-300)
    q_ref = sp.ndtr(-z)
    m = q_ref > 1e-300
    q_fit = pdf * pn / pd
    small = z[m] <= clamp
    assert np.all(np.abs(q_fit[m][small] - q_ref[m][small]) <= 1.5e-15)


def test_fp32_tail_fit_header():
    src = _read("normal_rational.h")
    val = {k: float(v) for k, v in re.findall(r"(kTail\w+) = (" + NUM + ")", src)}
    p = [val["kTailP0"], val["kTailP1"], val["kTailP2"]]
    s = [val["kTailS0"], val["kTailS1"], val["kTailS2"], 1.0]
    assert all(c > 0 for c in p + s)
    z = _z_grid()
    q = np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi) * np.polyval(p[::-1], z) / np.polyval(s[::-1], z)
    assert np.abs(q - sp.ndtr(-z)).max() <= val["kTailMaxAbsError"] * 1.001
