"""Failure paths on the GPU, made without faulting, trapping or hanging it.

The reference reports failures only as C++ exceptions from its OpenCL setup
(src/open_cl_simulation.cpp:630,648,767).  Here every C-ABI call returns a
status, and the device-side waits are bounded:
  - the single-pass scans' look-back polls a neighbour tile's status word;
  - the far-field kernel waits on an mbarrier for its own bulk copies.
A wait that runs out raises an error word, the kernel returns, and the host
reports NBODY_ERR_CUDA.  The tests make each wait run out on something that
never completes (nbody_selftest_wait: a status word nothing publishes, a
barrier no copy completes) with a short limit, and check the status, the
message and what the context can still do.  Device allocation failures are
injected on the host (NBODY_FAIL_ALLOC_AFTER): every one must come back as
NBODY_ERR_NOMEM and leave a context that nbody_destroy releases cleanly.
"""
import os
import time

import numpy as np
import pytest

from nbody_gb300 import ics

pytestmark = pytest.mark.gpu


def _sim(nb, n=3000, seed=61):
    pos, vel, m = ics.plummer(n, seed=seed)
    return nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=4, leaf_capacity=16,
                                        fixed_box=0, eps=0.01), (pos, vel, m)


def test_scan_wait_runs_out_and_fails_the_context(nb):
    from nbody_gb300 import _lib
    L = _lib.load()
    sim, (pos, vel, m) = _sim(nb)
    a0 = sim.forces()
    sim.set_wait_limits(scan_polls=2000)
    rc = L.nbody_selftest_wait(sim._h, 0)
    assert rc == 2 and b"scan did not complete" in L.nbody_last_error(sim._h)
    # a scan that gave up leaves the context failed: its next evaluation reports it too
    with pytest.raises(nb.NbodyError) as e:
        sim.forces()
    assert e.value.code == 2
    sim.close()
    # a new context is unaffected and gives the same forces
    sim2, _ = _sim(nb)
    np.testing.assert_array_equal(sim2.forces(), a0)


def test_scan_wait_default_limit_is_bounded(nb):
    from nbody_gb300 import _lib
    L = _lib.load()
    sim, _ = _sim(nb, 500)
    t0 = time.perf_counter()
    rc = L.nbody_selftest_wait(sim._h, 0)
    el = time.perf_counter() - t0
    assert rc == 2
    assert el < 20.0, el


def test_copy_wait_runs_out_and_context_stays_usable(nb):
    from nbody_gb300 import _lib
    L = _lib.load()
    sim, _ = _sim(nb)
    a0 = sim.forces()
    sim.set_wait_limits(copy_cycles=20000)
    rc = L.nbody_selftest_wait(sim._h, 1)
    assert rc == 2 and b"far-field copy" in L.nbody_last_error(sim._h)
    # the far-field wait fails one evaluation only: with the default limit back the context works
    sim.set_wait_limits()
    np.testing.assert_array_equal(sim.forces(), a0)
    # and with the default limit the self-test wait still runs out, after about a second
    t0 = time.perf_counter()
    assert L.nbody_selftest_wait(sim._h, 1) == 2
    assert time.perf_counter() - t0 < 20.0


def test_allocation_failures_are_reported(nb):
    """Each of the first allocations of a context's life fails in turn (create, upload, one force
    evaluation, a recorded 2-step run and its reverse sweep): the failing call returns
    NBODY_ERR_NOMEM (3) and nbody_destroy releases the context."""
    pos, vel, m = ics.plummer(2000, seed=62)
    seen_fail = 0
    ok_at = None
    for k in range(0, 400):
        os.environ["NBODY_FAIL_ALLOC_AFTER"] = str(k)
        try:
            try:
                sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=4,
                                                    leaf_capacity=16, fixed_box=0, eps=0.01,
                                                    integrator=nb.INTEG_LEAPFROG)
            except nb.NbodyError as e:
                assert e.code == 3, e
                seen_fail += 1
                continue
            try:
                sim.forces()
                sim.forward_checkpointed(2, 1)
                sim.backward(np.ones_like(pos), None)
            except nb.NbodyError as e:
                assert e.code == 3, e
                assert "NBODY_FAIL_ALLOC_AFTER" in str(e)
                seen_fail += 1
                sim.close()
                continue
            sim.close()
            ok_at = k
            break
        finally:
            del os.environ["NBODY_FAIL_ALLOC_AFTER"]
    assert ok_at is not None and seen_fail == ok_at and seen_fail > 20, (seen_fail, ok_at)
    # without injection everything works
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=4, leaf_capacity=16,
                                        fixed_box=0, eps=0.01)
    assert np.all(np.isfinite(sim.forces()))
