"""Adaptive global time step (nbody_set_timestep_control).

The reference integrates with one fixed dt and lists a variable time step among its goals (its TODO
file); these tests pin the library's rule, dt = clamp(eta * sqrt(length / max|a|), dt_min, dt_max)
from the accelerations at the start of each leapfrog step, against the oracle's FP64 direct-sum
restatement, and check the clamps, the mode switch and the refusals.
"""
import numpy as np
import pytest

from nbody_gb300 import ics

pytestmark = pytest.mark.gpu


def _sim(nb, pos, vel, m, **kw):
    args = dict(precision=nb.PREC_FP64, order=8, leaf_capacity=8, fixed_box=0, eps=0.01, dt=1e-3,
                integrator=nb.INTEG_LEAPFROG)
    args.update(kw)
    return nb.CudaSimulation.from_arrays(pos, vel, m, m, **args)


def test_adaptive_leapfrog_matches_fp64_direct(nb, oracle):
    pos, vel, m = ics.plummer(512, seed=62)
    eta, dt_min, dt_max, steps = 0.01, 1e-6, 2e-3, 10
    sim = _sim(nb, pos, vel, m)
    sim.set_timestep_control("adaptive", eta=eta, length=0.0, dt_min=dt_min, dt_max=dt_max)
    dts = []
    for _ in range(steps):
        sim.step()
        dts.append(sim.last_timestep())
    p1, v1, _, _, _ = sim.state("input")
    p2, v2, _, dts2 = oracle.leapfrog_adaptive(pos, vel, m, m, 0.01, 1.0, eta, 0.0, dt_min, dt_max, steps)
    dts = np.array(dts)
    assert np.all((dts >= dt_min) & (dts <= dt_max))
    assert np.any(dts < dt_max), dts             # the rule, not the clamp, sets the steps here
    np.testing.assert_allclose(dts, dts2, rtol=1e-5, atol=0)
    assert np.abs(p1 - p2).max() < 1e-7
    assert np.abs(v1 - v2).max() < 1e-5
    t = 0.0
    for d in dts:
        t += d
    assert sim.time == pytest.approx(t, rel=1e-14, abs=0)
    sim.close()


def test_adaptive_clamps_modes_and_refusals(nb):
    pos, vel, m = ics.plummer(1024, seed=63)
    sim = _sim(nb, pos, vel, m, precision=nb.PREC_MIXED, order=4, leaf_capacity=16)
    # a ceiling below the rule's value: every step takes dt_max exactly
    sim.set_timestep_control("adaptive", eta=10.0, length=1.0, dt_min=1e-7, dt_max=1e-5)
    t0 = sim.time
    sim.step(3)
    assert sim.last_timestep() == 1e-5
    assert sim.time == pytest.approx(t0 + 3e-5, rel=1e-12, abs=0)
    # the recorded run of the adjoint differentiates fixed steps only
    with pytest.raises(nb.NbodyError):
        sim.forward_checkpointed(2, 0)
    # back to fixed: the constructor's dt again
    sim.set_timestep_control("fixed")
    sim.step()
    assert sim.last_timestep() == 1e-3
    # invalid controls are refused
    for kw in (dict(eta=0.0), dict(dt_min=1e-3, dt_max=1e-4), dict(dt_min=0.0)):
        args = dict(eta=0.05, length=0.0, dt_min=1e-6, dt_max=1e-2)
        args.update(kw)
        with pytest.raises(nb.NbodyError):
            sim.set_timestep_control("adaptive", **args)
    sim.close()
    # explicit Euler: the rule on the previous evaluation's accelerations, within the clamps
    sim = _sim(nb, pos, vel, m, precision=nb.PREC_FP32, order=3, leaf_capacity=16, integrator=nb.INTEG_EULER)
    sim.set_timestep_control("adaptive", eta=0.05, length=0.0, dt_min=1e-6, dt_max=1e-2)
    t = 0.0
    for _ in range(4):
        sim.step()
        d = sim.last_timestep()
        assert 1e-6 <= d <= 1e-2
        t += d
    assert sim.time == pytest.approx(t, rel=1e-12, abs=0)
    p, _, _, _, _ = sim.state("input")
    assert np.all(np.isfinite(p))
    sim.close()


def test_block_steps_match_fp64_direct(nb, oracle):
    """Individual power-of-two steps (NBODY_DT_BLOCK, K = 3: dt_max 8e-3, substeps of 1e-3) against the
    oracle's FP64 direct-sum restatement: the same level for every particle (the FP64 order-8 forces
    are within ~1e-8 of the direct sum, far from a level threshold), positions within 1e-7 and
    velocities within 1e-5, as for the adaptive global step; several levels in use."""
    pos, vel, m = ics.plummer(1024, seed=64)
    eta, dt_min, dt_max, steps = 0.02, 1e-3, 8e-3, 2
    sim = _sim(nb, pos, vel, m)
    sim.set_timestep_control("block", eta=eta, length=0.0, dt_min=dt_min, dt_max=dt_max)
    sim.step(steps)
    assert sim.last_timestep() == dt_max
    assert sim.time == pytest.approx(steps * dt_max, rel=1e-14, abs=0)
    lv = sim.levels()
    p1, v1, _, _, _ = sim.state("input")
    ost = {}
    p2, v2, _, lv2 = oracle.leapfrog_block(pos, vel, m, m, 0.01, 1.0, eta, 0.0, dt_max, 3, steps, stats=ost)
    np.testing.assert_array_equal(lv, lv2)
    assert len(np.unique(lv)) >= 2, np.bincount(lv)
    st = sim.stats()                      # some substeps skipped the near field of some leaves
    assert 0 < st["block_active_leaves"] < st["block_leaves"], st
    assert st["block_evaluations"] == ost["evaluations"], (st, ost)
    assert np.abs(p1 - p2).max() < 1e-7
    assert np.abs(v1 - v2).max() < 1e-5
    # the recorded run of the adjoint refuses block steps; back to the fixed step
    with pytest.raises(nb.NbodyError):
        sim.forward_checkpointed(2, 0)
    sim.set_timestep_control("fixed")
    sim.step()
    assert sim.last_timestep() == 1e-3
    sim.close()


def test_block_substeps_without_an_ending_step_only_drift(nb):
    """K = 3 with every particle on level 0 (a large eta): one force evaluation per base step, at its
    end; the other seven substeps only drift.  The result is the fixed leapfrog step of dt_max with
    its drift taken in eight parts: equal to a few ulps."""
    pos, vel, m = ics.plummer(2048, seed=66)
    a = _sim(nb, pos, vel, m, order=6, leaf_capacity=16, dt=8e-3)
    a.step(2)
    b = _sim(nb, pos, vel, m, order=6, leaf_capacity=16, dt=8e-3)
    b.set_timestep_control("block", eta=1e6, length=0.0, dt_min=1e-3, dt_max=8e-3)
    b.step(2)
    assert np.all(b.levels() == 0)
    st = b.stats()
    assert st["block_evaluations"] == 1, st
    assert st["block_active_leaves"] == st["block_leaves"] == st["leaves"], st
    pa, va = a.state("input")[:2]
    pb, vb = b.state("input")[:2]
    np.testing.assert_allclose(pb, pa, rtol=0, atol=1e-13)
    np.testing.assert_allclose(vb, va, rtol=0, atol=1e-12)
    a.close()
    b.close()


def test_block_steps_with_one_level_are_the_fixed_leapfrog(nb):
    """K = 0 (dt_min = dt_max): the block scheme is the fixed-step kick-drift-kick leapfrog, computed by
    separate kick and drift kernels instead of the fused ones: equal to 1e-14."""
    pos, vel, m = ics.plummer(2048, seed=65)
    a = _sim(nb, pos, vel, m, precision=nb.PREC_MIXED, order=5, leaf_capacity=16, dt=2e-3)
    a.step(3)
    b = _sim(nb, pos, vel, m, precision=nb.PREC_MIXED, order=5, leaf_capacity=16, dt=2e-3)
    b.set_timestep_control("block", eta=0.02, length=0.0, dt_min=2e-3, dt_max=2e-3)
    b.step(3)
    pa, va = a.state("input")[:2]
    pb, vb = b.state("input")[:2]
    np.testing.assert_allclose(pb, pa, rtol=0, atol=1e-14)
    np.testing.assert_allclose(vb, va, rtol=0, atol=1e-13)
    with pytest.raises(nb.NbodyError):
        b.set_timestep_control("block", eta=0.02, length=0.0, dt_min=3e-4, dt_max=2e-3)   # not 2^K
