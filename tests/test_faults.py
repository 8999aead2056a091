"""Failure paths of the C ABI, made on the host (no GPU fault, trap or hang).

mdsx_inject_fault arms one host-side call to fail -- a device allocation, a
pinned host allocation, or the enqueue of a sweep -- without making it, and
returns the error the CUDA runtime would. These tests check that:
  * engine creation fails with MDSX_ENOMEM at every one of its allocations in
    turn, with a message, and leaves no device memory behind;
  * a failed setPairwiseData staging allocation returns MDSX_ENOMEM and the
    engine stays usable;
  * a failed sweep enqueue returns MDSX_ECUDA from getSumOfIncrements /
    getLogLikelihoodGradient, and the next call evaluates correctly;
  * the batched engine reports MDSX_ENOMEM / MDSX_ECUDA the same way and
    recovers on the next evaluation.
The reference has nothing to compare with here: it asserts or exits
(src/NewMultiDimensionalScaling.hpp:140,148,258,263,283).
"""
import ctypes

import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, MdsxError, flags as F
from massivemds_gb300._lib import load

NONE, DEVICE_ALLOC, HOST_ALLOC, LAUNCH = 0, 1, 2, 3
ENOMEM, ECUDA = 2, 3


def arm(lib, site, after=0):
    fired = ctypes.c_longlong()
    assert lib.mdsx_inject_fault(site, after, ctypes.byref(fired)) == 0
    return fired.value


def test_inject_fault_arguments(mdsx_lib):
    assert mdsx_lib.mdsx_inject_fault(4, 0, None) == 1
    assert mdsx_lib.mdsx_inject_fault(-1, 0, None) == 1
    assert mdsx_lib.mdsx_inject_fault(DEVICE_ALLOC, -1, None) == 1
    assert mdsx_lib.mdsx_inject_fault(NONE, 0, None) == 0


def _problem(n, p, seed=0):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 10))
    return np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1)), rng.standard_normal((n, p))


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [F.LEFT_TRUNCATION, F.FLOAT | F.LEFT_TRUNCATION])
def test_engine_creation_fails_cleanly_at_every_allocation(flags):
    torch = pytest.importorskip("torch")
    lib = load()
    n, p = 1000, 2
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    for site in (DEVICE_ALLOC, HOST_ALLOC):
        for k in range(64):
            arm(lib, site, k)
            h = ctypes.c_void_p()
            rc = lib.mdsx_create(p, n, flags, -1, ctypes.byref(h))
            if rc == 0:  # creation made fewer than k + 1 calls at this site
                lib.mdsx_destroy(h)
                break
            assert rc == ENOMEM, (site, k, rc)
            assert b"out of memory" in lib.mdsx_last_error(None), lib.mdsx_last_error(None)
            failures += 1
        arm(lib, NONE)
    assert failures >= 10  # every allocation of the engine's plan was made to fail once
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - (64 << 20)  # nothing left allocated
    # and a normal engine still works
    delta, x = _problem(n, p)
    with Engine(p, n, flags) as e:
        e.setPairwiseData(delta)
        e.updateLocations(-1, x)
        e.setParameters([1.5])
        tol = 1e-5 if flags & F.FLOAT else 1e-10
        ref = oracle.sum_of_increments(delta.astype(np.float32) if flags & F.FLOAT else delta, x, 1.5)
        assert abs(e.getSumOfIncrements() - ref) / abs(ref) < tol


@pytest.mark.gpu
def test_failed_staging_and_launch_leave_the_engine_usable():
    lib = load()
    n, p, tau = 701, 3, 0.9  # odd N: FP64 rows are padded, so setPairwiseData stages through a device buffer
    delta, x = _problem(n, p, 1)
    s_ref, g_ref = oracle.evaluate(delta, x, tau, True)
    with Engine(p, n, F.LEFT_TRUNCATION) as e:
        arm(lib, DEVICE_ALLOC, 0)
        with pytest.raises(MdsxError) as err:
            e.setPairwiseData(delta)
        assert err.value.status == ENOMEM
        arm(lib, NONE)
        e.setPairwiseData(delta)
        e.updateLocations(-1, x)
        e.setParameters([tau])
        for schedule in (F.SWEEP_ROWS, F.SWEEP_PAIRS):
            e.set_sweep_schedule(schedule)
            e.makeDirty()
            arm(lib, LAUNCH, 0)
            with pytest.raises(MdsxError) as err:
                e.getSumOfIncrements()
            assert err.value.status == ECUDA
            arm(lib, LAUNCH, 0)
            with pytest.raises(MdsxError) as err:
                e.getLogLikelihoodGradient()
            assert err.value.status == ECUDA
            arm(lib, NONE)
            assert abs(e.getSumOfIncrements() - s_ref) / abs(s_ref) < 1e-10
            g = e.getLogLikelihoodGradient().reshape(n, p)
            assert np.abs(g - g_ref).max() / np.abs(g_ref).max() < 1e-9


@pytest.mark.gpu
def test_batch_reports_and_recovers_from_failures():
    from massivemds_gb300.batch import Batch

    lib = load()
    specs = [(300, 2, 1.1), (257, 3, 0.7), (190, 6, 2.0)]
    problems = []
    with Batch() as b:
        for k, (n, p, tau) in enumerate(specs):
            delta, x = _problem(n, p, 10 + k)
            delta = delta.astype(np.float32)
            b.add_instance(p, n)
            b.setPairwiseData(k, delta)
            b.updateLocations(k, -1, x)
            b.setParameters(k, [tau])
            problems.append((delta, x, tau))
        for site, status in ((DEVICE_ALLOC, ENOMEM), (HOST_ALLOC, ENOMEM), (LAUNCH, ECUDA)):
            b.makeDirty()
            if site != LAUNCH:
                b.force_shape(2, 0)  # drop the plan so the next evaluation allocates again
            arm(lib, site, 0)
            with pytest.raises(MdsxError) as err:
                b.evaluate()
            assert err.value.status == status, site
            arm(lib, NONE)
            b.evaluate()
            for k, (delta, x, tau) in enumerate(problems):
                s_ref, g_ref = oracle.evaluate(delta, x, tau, True)
                assert abs(b.getSumOfIncrements(k) - s_ref) / abs(s_ref) < 1e-5
                g = np.asarray(b.getLogLikelihoodGradient(k)).reshape(g_ref.shape)
                assert np.abs(g - g_ref).max() / np.abs(g_ref).max() < 1e-5
