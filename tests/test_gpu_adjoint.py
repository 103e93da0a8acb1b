"""Adjoint of the CUDA step (through the C ABI) against the oracle.  Needs a GPU.

Checks
  force VJP, FP64 form        = frozen-tree derivative of the FP64 oracle FMM
                                (central differences along random directions),
                                1e-7 relative
  force VJP vs FP64 direct-sum VJP (oracle)   within the FMM truncation error:
                                order 8 FP64 3e-6, order 5 mixed 3e-4 relative rms
  trajectory adjoint          vs the FP64 direct-sum leapfrog adjoint (oracle),
                                order 8 FP64, 1e-6 relative
  checkpoint spacing          every = 1, 2, 3, N and recorded evaluations (0) give bitwise
                                identical gradients
  state after the reverse sweep is the recorded run's final state, bitwise
"""
import numpy as np
import pytest

from nbody_gb300 import ics

pytestmark = pytest.mark.gpu

EPS = 0.01


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _rel_rms_rows(a, b):
    a = np.asarray(a).reshape(len(b), -1)
    b = np.asarray(b).reshape(len(b), -1)
    e = np.linalg.norm(a - b, axis=1) / np.sqrt(np.mean(np.sum(b * b, axis=1)))
    return float(np.sqrt(np.mean(e ** 2)))


def _sim(nb, pos, vel, m, q, prec, order, cap=16, **kw):
    p = {"fp32": nb.PREC_FP32, "mixed": nb.PREC_MIXED, "fp64": nb.PREC_FP64}[prec]
    return nb.CudaSimulation.from_arrays(pos, vel, m, q, precision=p, order=order, leaf_capacity=cap, fixed_box=0,
                                         eps=EPS, **kw)


@pytest.mark.parametrize("order", [1, 4, 6])
def test_force_vjp_is_the_frozen_tree_derivative(nb, oracle, order):
    pos, vel, m = ics.plummer(2500, seed=41)
    rng = np.random.default_rng(order)
    q = m * rng.uniform(0.5, 1.5, len(m))
    mu = rng.normal(size=pos.shape)
    sim = _sim(nb, pos, vel, m, q, "fp64", order)
    gx, gq, gm = sim.force_vjp(mu)
    t = oracle.Tree(pos, q, m, cap=16).traverse(0.5)

    def S(**kw):
        t.set_particles(pos=kw.get("pos", pos), q=kw.get("q", q), m=kw.get("m", m))
        a, _ = t.fmm(order, EPS)
        return float(np.sum(mu * a))

    for k in range(3):
        d = rng.normal(size=pos.shape)
        h = 1e-6
        fd = (S(pos=pos + h * d) - S(pos=pos - h * d)) / (2 * h)
        assert abs(np.sum(gx * d) - fd) < 1e-7 * np.abs(gx * d).sum()
    dq = rng.normal(size=q.shape) * q
    fdq = (S(q=q + 1e-4 * dq) - S(q=q - 1e-4 * dq)) / 2e-4
    assert abs(np.sum(gq * dq) - fdq) < 1e-8 * np.abs(gq * dq).sum()
    dm = rng.normal(size=m.shape) * m
    fdm = (S(m=m + 1e-6 * dm) - S(m=m - 1e-6 * dm)) / 2e-6
    assert abs(np.sum(gm * dm) - fdm) < 1e-7 * np.abs(gm * dm).sum()


@pytest.mark.parametrize("prec,order,tol", [("fp64", 8, 3e-6), ("mixed", 5, 3e-4), ("fp32", 4, 3e-3)])
def test_force_vjp_matches_direct_sum_vjp(nb, oracle, prec, order, tol):
    pos, vel, m = ics.clustered(6000, seed=42)
    rng = np.random.default_rng(7)
    mu = rng.normal(size=pos.shape)
    sim = _sim(nb, pos, vel, m, m, prec, order)
    gx, gq, gm = sim.force_vjp(mu)
    if prec == "fp32":
        pos = pos.astype(np.float32).astype(np.float64)
    rx, rq, rm = oracle.direct_vjp(pos, m, m, mu, eps=EPS)
    assert _rel_rms_rows(gx, rx) < tol
    assert _rel_rms_rows(gq, rq) < tol
    assert _rel_rms_rows(gm, rm) < tol


def test_force_vjp_unsoftened_and_duplicates(nb, oracle):
    """eps = 0 with coincident particles: pairs at zero distance contribute nothing (as in the forces)."""
    rng = np.random.default_rng(5)
    pos = np.concatenate([rng.uniform(0, 1, (600, 3)), np.repeat(rng.uniform(0, 1, (4, 3)), 3, axis=0)])
    m = np.full(len(pos), 1.0 / len(pos))
    mu = rng.normal(size=pos.shape)
    sim = nb.CudaSimulation.from_arrays(pos, None, m, m, precision=nb.PREC_FP64, order=8, leaf_capacity=8,
                                        fixed_box=0, eps=0.0)
    gx, gq, gm = sim.force_vjp(mu)
    assert np.all(np.isfinite(gx)) and np.all(np.isfinite(gq)) and np.all(np.isfinite(gm))
    rx, rq, rm = oracle.direct_vjp(pos, m, m, mu, eps=0.0)
    ok = np.isfinite(rx).all(axis=1)
    assert _rel_rms_rows(gx[ok], rx[ok]) < 1e-4


def _run(nb, pos, vel, m, prec, order, steps, every, gxT, gvT, dt=1e-3):
    sim = _sim(nb, pos, vel, m, m, prec, order, cap=8, dt=dt, integrator=nb.INTEG_LEAPFROG)
    sim.forward_checkpointed(steps, every)
    fin = sim.state("leaf", with_acc=True)
    g = sim.backward(gxT, gvT)
    after = sim.state("leaf", with_acc=True)
    for a, b in zip(fin, after):
        np.testing.assert_array_equal(a, b)
    return g, sim


def test_trajectory_adjoint_matches_direct_sum_adjoint(nb, oracle):
    pos, vel, m = ics.plummer(1200, seed=43)
    rng = np.random.default_rng(8)
    gxT, gvT = rng.normal(size=pos.shape), rng.normal(size=pos.shape)
    steps, dt = 6, 1e-3
    (gx0, gv0, gq, gm), sim = _run(nb, pos, vel, m, "fp64", 8, steps, 1, gxT, gvT, dt)
    assert abs(sim.time - steps * dt) < 1e-12
    rx, rv, rq, rm = oracle.leapfrog_adjoint(pos, vel, m, m, EPS, 1.0, dt, steps, gxT, gvT)
    assert _rel(gx0, rx) < 1e-6
    assert _rel(gv0, rv) < 1e-6
    assert _rel(gq, rq) < 1e-5
    assert _rel(gm, rm) < 1e-5


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_checkpoint_spacing_gives_identical_gradients(nb, prec):
    pos, vel, m = ics.clustered(3000, seed=44)
    rng = np.random.default_rng(9)
    gxT, gvT = rng.normal(size=pos.shape), rng.normal(size=pos.shape)
    ref, _ = _run(nb, pos, vel, m, prec, 5, 7, 1, gxT, gvT)
    for every in (0, 2, 3, 7):
        g, _ = _run(nb, pos, vel, m, prec, 5, 7, every, gxT, gvT)
        for a, b in zip(g, ref):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("every", [2, 7])
def test_second_backward_equals_the_first(nb, every):
    """The last checkpoint interval is recorded by the forward run and not recomputed by the first
    reverse sweep; a second reverse sweep over the same run (whose records the first one replaced
    with the earlier intervals' when there are several) gives the same gradients bitwise."""
    pos, vel, m = ics.clustered(3000, seed=46)
    rng = np.random.default_rng(10)
    gxT, gvT = rng.normal(size=pos.shape), rng.normal(size=pos.shape)
    g1, sim = _run(nb, pos, vel, m, "mixed", 5, 7, every, gxT, gvT)
    g2 = sim.backward(gxT, gvT)
    for a, b in zip(g1, g2):
        np.testing.assert_array_equal(a, b)
    sim.close()


def test_backward_needs_a_recorded_run(nb):
    pos, vel, m = ics.plummer(500, seed=45)
    sim = _sim(nb, pos, vel, m, m, "mixed", 3, integrator=nb.INTEG_LEAPFROG)
    with pytest.raises(nb.NbodyError):
        sim.backward(np.zeros_like(pos), None)
    sim.forward_checkpointed(2, 1)
    sim.step(1)                       # drops the recording
    with pytest.raises(nb.NbodyError):
        sim.backward(np.zeros_like(pos), None)
    eu = _sim(nb, pos, vel, m, m, "mixed", 3, integrator=nb.INTEG_EULER)
    with pytest.raises(nb.NbodyError):
        eu.forward_checkpointed(2, 1)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_replay_reproduces_the_recorded_run(nb, prec):
    """nbody_forward_replay from the recorded run's own initial state repeats that run bitwise (same
    trees, lists and arithmetic); from a perturbed state it moves the final state; and the recording
    survives it: the reverse sweep after a replay equals the one before."""
    p = {"mixed": nb.PREC_MIXED, "fp64": nb.PREC_FP64}[prec]
    pos, vel, m = ics.plummer(5000, seed=63)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=p, order=5, leaf_capacity=32, fixed_box=0,
                                        eps=0.01, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
    sim.forward_checkpointed(6, 0)
    x6, v6 = sim.state("input")[:2]
    seed = np.random.default_rng(63).normal(size=pos.shape)
    g_before = sim.backward(seed, None)
    xr, vr = sim.replay(pos, vel, m, m)
    np.testing.assert_array_equal(xr, x6)
    np.testing.assert_array_equal(vr, v6)
    p2 = pos.copy()
    p2[17, 1] += 1e-4
    x2, _ = sim.replay(p2, vel, m, m, 6)
    assert np.abs(x2 - x6).max() > 0 and np.abs(x2 - x6).max() < 1e-3
    for a, b in zip(g_before, sim.backward(seed, None)):
        np.testing.assert_array_equal(a, b)
