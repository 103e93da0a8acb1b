"""The workload configurations beside the headline one, as GPU parity cases.

C0 plummer4k    reference mode (order 1, FP32, explicit Euler, capacity 16, theta 0.5, eps 0.01,
                dt 1e-3) for 100 steps against the oracle's 100-step run of the restated
                reference FMM (trajectories within FP32 rounding); at the last step the tree, the
                interaction sets and the forces match the oracle (forces within 1e-5 of the
                largest)
C1 cube256k     precision study: rms relative force error vs the FP64 direct sum on 8,192 seeded
                targets for theta in {0.3, 0.5, 0.7} and the three precision forms (order 5,
                capacity 32, eps 1e-3): monotone in theta (FP64, mixed), mixed within 5 % of
                FP64, theta 0.5 below 1e-4 (FP64, mixed) and 2e-4 (FP32)
C3 plummer64k   trajectory adjoint (FP64 form, order 5, 20 steps, checkpoint every 5, loss = mean
                squared distance to a perturbed-velocity run) against FP64 central finite
                differences of the GPU forward on 8 components; and, at N = 4,096, against the
                FP64 direct-sum leapfrog adjoint (1e-5: the order-8 truncation error)
C4 clusters4m   N = 4,194,304 in 64 sub-clusters, 50 steps forward + adjoint (mixed, order 5):
                finite gradients, momentum conserved, device high-water mark below 24 GB
"""
import numpy as np
import pytest

from nbody_gb300 import ics

pytestmark = pytest.mark.gpu


def _set(a):
    return set(map(tuple, np.asarray(a).tolist()))


def _rms_rel(a, b):
    e = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
    return float(np.sqrt(np.mean(e ** 2)))


def test_c0_reference_mode_100_steps(nb, oracle):
    """100 steps of the GPU in reference mode against 100 steps of the oracle's restated reference FMM
    (oracle.ref_mode_run: order 0, FP32, explicit Euler, tree rebuilt every step), from the same FP32
    initial state.  The two sum each particle's field in different orders, so the trajectories part
    by FP32 rounding only: positions within 2e-5 (box side 40, coordinates near 20 where one FP32 ulp
    is 1.9e-6), velocities within 1e-4 of the largest.  At step 100 the tree and interaction sets are
    bit-exact and the forces match the reference kernels on the GPU's own final positions."""
    pos, vel, m = ics.workload("plummer4k", seed=51)
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    pos, vel, m = f32(pos + 20.0), f32(vel), f32(m)   # inside the reference's [0, bounds) root box
    b = 40.0
    sim = nb.CudaSimulation([b, b, b, 0.0], None, 1e-3, precision=nb.PREC_FP32, order=1, leaf_capacity=16,
                            theta=0.5, eps=0.01)
    sim.set_state(pos, vel, m, m)
    for _ in range(100):
        sim.step()
    p1, v1, m1, q1, _ = sim.state("input")
    assert np.all(np.isfinite(p1)) and np.all((p1 >= 0) & (p1 < b))
    xo, vo = oracle.ref_mode_run(pos, vel, m, m, [0.0, 0.0, 0.0, b], 16, 0.5, 0.01, 1e-3, 100)
    dx = np.abs(p1 - xo).max()
    dv = np.abs(v1 - vo).max() / np.abs(vo).max()
    assert dx <= 2e-5 and dv <= 1e-4, (dx, dv)
    acc = sim.forces()
    keys, perm, nodes = sim.tree()
    t = oracle.Tree(p1, q1, m1, box=np.array([0.0, 0.0, 0.0, b]), cap=16).traverse(0.5)
    np.testing.assert_array_equal(nodes, t.nodes)
    np.testing.assert_array_equal(perm, t.perm.astype(np.int64))
    assert _set(sim.interactions("p2p")) == _set(t.pairs("p2p"))
    assert _set(sim.interactions("m2l")) == _set(t.pairs("m2l"))
    fl, fn = t.ref_forces_f32(0.01)
    F = acc * m1[:, None]
    Fref = (fl + fn).astype(np.float64)
    assert np.abs(F - Fref).max() <= 1e-5 * np.abs(Fref).max()


def test_c1_precision_study(nb):
    pos, vel, m = ics.workload("cube256k", seed=52)
    tg = np.random.default_rng(52).choice(len(m), 8192, replace=False)
    err = {}
    ref = {}
    for prec in ("fp32", "mixed", "fp64"):
        p = {"fp32": nb.PREC_FP32, "mixed": nb.PREC_MIXED, "fp64": nb.PREC_FP64}[prec]
        for theta in (0.3, 0.5, 0.7):
            sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=p, order=5, leaf_capacity=32, fixed_box=0,
                                                theta=theta, eps=1e-3)
            acc = sim.forces()
            # the FP32 form holds FP32-rounded positions: its direct sum is taken at those
            key = prec == "fp32"
            if key not in ref:
                ref[key], _ = sim.direct(tg)
            err[prec, theta] = _rms_rel(acc[tg], ref[key])
            sim.close()
    for prec in ("mixed", "fp64"):
        assert err[prec, 0.3] < err[prec, 0.5] < err[prec, 0.7], err
    for theta in (0.3, 0.5, 0.7):
        assert abs(err["mixed", theta] - err["fp64", theta]) <= 0.05 * err["fp64", theta] + 2e-7, err
    assert err["fp64", 0.5] < 1e-4 and err["mixed", 0.5] < 1e-4 and err["fp32", 0.5] < 2e-4, err


def test_c2_collision_1000_steps_energy_momentum(nb):
    """Config 2 as specified: the N = 1,048,576 two-Plummer collision, mixed form, order 5, leapfrog
    dt 5e-4 for 1,000 steps (t = 0.5).  FP64 diagnostics before and after: relative energy drift below
    2e-6, momentum drift below 2e-9 and angular-momentum drift below 1e-6 (total mass 1; the FMM forces
    are not exactly antisymmetric, so momenta are conserved only to the force error).  One GB300 run
    measured 1.6e-7, 1.9e-10 and 6.4e-8."""
    pos, vel, m = ics.workload("collision1m", seed=0)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=5, leaf_capacity=64,
                                        fixed_box=0, eps=0.005, dt=5e-4, integrator=nb.INTEG_LEAPFROG)
    d0 = sim.diagnostics()
    sim.step(1000)
    d1 = sim.diagnostics()
    de = (d1["energy"] - d0["energy"]) / abs(d0["energy"])
    dp = np.abs(d1["momentum"] - d0["momentum"]).max()
    dl = np.abs(d1["angular_momentum"] - d0["angular_momentum"]).max()
    assert abs(de) < 2e-6 and dp < 2e-9 and dl < 1e-6, (de, dp, dl)


def _loss_run(nb, pos, vel, m, x_target, steps):
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_FP64, order=5, leaf_capacity=16,
                                        fixed_box=0, eps=0.01, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
    sim.step(steps)
    x = sim.state("input")[0]
    sim.close()
    return float(np.mean(np.sum((x - x_target) ** 2, axis=1)))


def test_c3_trajectory_adjoint_vs_finite_differences(nb):
    pos, vel, m = ics.workload("plummer64k", seed=53)
    n, steps = len(m), 20
    rng = np.random.default_rng(53)
    vel_t = vel + 1e-3 * rng.normal(size=vel.shape)
    tgt = nb.CudaSimulation.from_arrays(pos, vel_t, m, m, precision=nb.PREC_FP64, order=5, leaf_capacity=16,
                                        fixed_box=0, eps=0.01, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
    tgt.step(steps)
    x_target = tgt.state("input")[0]
    tgt.close()
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_FP64, order=5, leaf_capacity=16,
                                        fixed_box=0, eps=0.01, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
    sim.forward_checkpointed(steps, 5)
    xN = sim.state("input")[0]
    gx0, gv0, gq, gm = sim.backward(2.0 * (xN - x_target) / n, None)
    sim.close()
    # components with the largest gradients (well above the finite-difference noise)
    scale_v, scale_x = np.abs(gv0).max(), np.abs(gx0).max()
    iv = np.argsort(-np.abs(gv0).ravel())[:4]
    ix = np.argsort(-np.abs(gx0).ravel())[:4]
    h = 1e-4
    for which, idx, g, scale in (("v", iv, gv0, scale_v), ("x", ix, gx0, scale_x)):
        for flat in idx:
            i, d = divmod(int(flat), 3)
            p_hi, p_lo, v_hi, v_lo = pos.copy(), pos.copy(), vel.copy(), vel.copy()
            if which == "v":
                v_hi[i, d] += h
                v_lo[i, d] -= h
            else:
                p_hi[i, d] += h
                p_lo[i, d] -= h
            fd = (_loss_run(nb, p_hi, v_hi, m, x_target, steps) - _loss_run(nb, p_lo, v_lo, m, x_target, steps)) / (2 * h)
            assert abs(fd - g[i, d]) <= 1e-3 * abs(g[i, d]) + 1e-6 * scale, (which, i, d, fd, g[i, d])


def test_c3_trajectory_adjoint_vs_direct_sum_adjoint_4k(nb, oracle):
    pos, vel, m = ics.plummer(4096, seed=54)
    rng = np.random.default_rng(54)
    gxT, gvT = rng.normal(size=pos.shape), rng.normal(size=pos.shape)
    steps, dt = 10, 1e-3
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_FP64, order=8, leaf_capacity=16,
                                        fixed_box=0, eps=0.01, dt=dt, integrator=nb.INTEG_LEAPFROG)
    sim.forward_checkpointed(steps, 0)
    gx0, gv0, gq, gm = sim.backward(gxT, gvT)
    rx, rv, rq, rm = oracle.leapfrog_adjoint(pos, vel, m, m, 0.01, 1.0, dt, steps, gxT, gvT)
    for a, b in ((gx0, rx), (gv0, rv), (gq, rq), (gm, rm)):
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)


def test_c4_clusters4m_forward_adjoint(nb):
    pos, vel, m = ics.workload("clusters4m", seed=55)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=5, leaf_capacity=64,
                                        fixed_box=0, eps=1e-3, dt=2.5e-4, integrator=nb.INTEG_LEAPFROG)
    p0 = sim.diagnostics()["momentum"]
    sim.forward_checkpointed(50, 10)
    p1 = sim.diagnostics()["momentum"]
    rng = np.random.default_rng(55)
    gx0, gv0, gq, gm = sim.backward(rng.normal(size=pos.shape), None)
    for g in (gx0, gv0, gq, gm):
        assert np.all(np.isfinite(g))
    assert np.abs(gv0).max() > 0
    assert np.abs(p1 - p0).max() < 1e-4
    cur, peak = sim.device_memory()
    assert 0 < cur <= peak < 24 * 2 ** 30, (cur, peak)
