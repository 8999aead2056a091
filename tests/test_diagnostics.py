"""CPU tests: the momentum generator's known-answer vectors and the ESS estimator."""
import numpy as np

from massivemds_gb300 import diagnostics as dg
from oracle.hmc_oracle import momentum, philox4x32_10


def test_philox_known_answers():
    # Known-answer vectors published with the Philox4x32-10 generator (Random123).
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        got = philox4x32_10(*[np.array([c], dtype=np.uint32) for c in ctr], *key)
        assert tuple(int(v[0]) for v in got) == want


def test_momentum_is_standard_normal_and_reproducible():
    a = momentum(200001, seed=7, iteration=3)
    assert abs(a.mean()) < 0.01 and abs(a.var() - 1.0) < 0.01
    assert np.array_equal(a, momentum(200001, seed=7, iteration=3))
    assert not np.array_equal(a[:100], momentum(100, seed=7, iteration=4))


def test_ess_of_iid_and_ar1():
    rng = np.random.default_rng(0)
    n = 20000
    iid = rng.standard_normal(n)
    assert 0.85 * n < dg.ess(iid) < 1.15 * n
    phi = 0.6
    ar = np.empty(n)
    ar[0] = rng.standard_normal()
    for t in range(1, n):
        ar[t] = phi * ar[t - 1] + rng.standard_normal()
    expected = n * (1 - phi) / (1 + phi)
    assert 0.8 * expected < dg.ess(ar) < 1.2 * expected


def test_min_ess_picks_the_worst_column():
    rng = np.random.default_rng(1)
    n = 5000
    slow = np.cumsum(rng.standard_normal(n)) * 0.01 + rng.standard_normal(n) * 0.001
    cols = np.column_stack([rng.standard_normal(n), slow])
    v, k = dg.min_ess(cols)
    assert k == 1 and v < dg.ess(cols[:, 0])
