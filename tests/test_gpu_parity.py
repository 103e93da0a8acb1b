"""Parity of the CUDA step (through the C ABI) with the oracle and the
reference fixtures.  Needs a GPU: run with ``-m gpu``.

Tolerances
  tree, Morton order, interaction sets      bit-exact
  order-1 FP32 forces vs reference kernels  1e-5 of the largest force
  FP64 form vs FP64 oracle FMM, same order  1e-10 relative (per particle)
  mixed form vs FP64 oracle FMM             3e-6 relative rms
  FP32 form vs FP64 oracle FMM              1e-4 relative rms
"""
import numpy as np
import pytest

from nbody_gb300 import ics

pytestmark = pytest.mark.gpu


def _set(a):
    return set(map(tuple, np.asarray(a).tolist()))


def _rel_rms(a, b):
    e = np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)
    return float(np.sqrt(np.mean(e ** 2)))


CASES = {
    "plummer": lambda: ics.plummer(4096, seed=21) + (16,),
    "cube": lambda: ics.uniform_cube(6000, seed=22) + (32,),
    "clusters": lambda: ics.clustered(6400, seed=23) + (16,),
}


def _edge(case):
    rng = np.random.default_rng(3)
    if case == "duplicates":
        pos = np.repeat(rng.uniform(0, 1, (12, 3)), 40, axis=0)
        cap = 8
    elif case == "tiny":
        pos = rng.uniform(0, 1, (5, 3))
        cap = 8
    elif case == "single":
        pos = np.array([[0.25, 0.5, 0.75]])
        cap = 1
    elif case == "planes":
        # particles exactly on split planes of a [0,1) box
        g = np.arange(0, 1, 1 / 8.0)
        pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        cap = 4
    n = len(pos)
    return pos, np.zeros((n, 3)), np.full(n, 1.0 / n), cap


@pytest.mark.parametrize("case", ["plummer", "cube", "clusters", "duplicates", "tiny", "single", "planes"])
def test_tree_bitexact_vs_oracle(nb, oracle, case):
    pos, vel, m, cap = CASES[case]() if case in CASES else _edge(case)
    fixed = case == "planes"
    kw = dict(precision=nb.PREC_MIXED, order=3, leaf_capacity=cap, fixed_box=int(fixed))
    if fixed:
        kw.update(box_min=(0.0, 0.0, 0.0), box_size=1.0)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, **kw)
    sim.forces()
    keys, perm, nodes = sim.tree()
    box = np.array([0, 0, 0, 1.0]) if fixed else oracle.bounding_box(pos)
    t = oracle.Tree(pos, m, m, box=box, cap=cap)
    np.testing.assert_array_equal(keys, t.keys)
    np.testing.assert_array_equal(perm, t.perm.astype(np.int64))
    np.testing.assert_array_equal(nodes, t.nodes)


@pytest.mark.parametrize("case", ["plummer", "clusters"])
def test_interaction_sets_bitexact_vs_oracle(nb, oracle, case):
    pos, vel, m, cap = CASES[case]()
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=4, leaf_capacity=cap,
                                        fixed_box=0)
    sim.forces()
    p2p = sim.interactions("p2p")
    m2l = sim.interactions("m2l")
    t = oracle.Tree(pos, m, m, cap=cap).traverse(0.5)
    assert _set(p2p) == _set(t.pairs("p2p"))
    assert _set(m2l) == _set(t.pairs("m2l"))


@pytest.mark.parametrize("name", ["ref_fmm_plummer1k.npz", "ref_fmm_cube2k.npz"])
def test_reference_mode_matches_reference_kernels(nb, golden, name):
    """Order 1, FP32, capacity 8, [0, bounds) box, explicit Euler: the reference's FMM."""
    g = golden(name)
    b = float(g["box"][3])
    sim = nb.CudaSimulation([b, b, b, 0.0], None, float(g["dt"]), precision=nb.PREC_FP32, order=1,
                            leaf_capacity=int(g["cap"]), theta=float(g["theta"]), eps=float(g["eps"]))
    sim.set_state(g["pos"], g["vel"], g["mass"], g["charge"])
    acc = sim.forces()
    keys, perm, nodes = sim.tree()
    np.testing.assert_array_equal(nodes, g["nodes"])
    np.testing.assert_array_equal(perm, g["perm"])
    assert _set(sim.interactions("p2p")) == _set(g["p2p"])
    assert _set(sim.interactions("m2l")) == _set(g["m2l"])
    F = acc * g["mass"][:, None]
    Fref = (g["f_leaf"] + g["f_node"]).astype(np.float64)
    assert np.abs(F - Fref).max() <= 1e-5 * np.abs(Fref).max()
    # one explicit-Euler step (src/open_cl_simulation.cpp:600-607)
    sim.step()
    pos1, vel1, _, _, _ = sim.state("input")
    np.testing.assert_allclose(pos1, g["pos1"], rtol=0, atol=1e-6 * b)
    dv = np.abs(vel1 - g["vel1"]).max()
    assert dv <= 1e-5 * np.abs(Fref / g["mass"][:, None]).max() * float(g["dt"]) + 1e-7


@pytest.mark.parametrize("order", [1, 3, 5, 7])
def test_fp64_form_matches_fp64_oracle_fmm(nb, oracle, order):
    pos, vel, m = ics.plummer(3000, seed=31)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_FP64, order=order, leaf_capacity=16,
                                        fixed_box=0, eps=0.01)
    acc, pot = sim.forces(potential=True)
    t = oracle.Tree(pos, m, m, cap=16).traverse(0.5)
    a_ref, p_ref = t.fmm(order, 0.01)
    e = np.linalg.norm(acc - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
    assert e.max() < 1e-10
    assert np.abs(pot - p_ref).max() < 1e-10 * np.abs(p_ref).max()


@pytest.mark.parametrize("prec,tol", [("mixed", 3e-6), ("fp32", 1e-4)])
@pytest.mark.parametrize("order", [2, 5])
def test_single_precision_forms_match_fp64_oracle_fmm(nb, oracle, prec, tol, order):
    pos, vel, m = ics.plummer(4096, seed=32)
    p = nb.PREC_MIXED if prec == "mixed" else nb.PREC_FP32
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=p, order=order, leaf_capacity=16, fixed_box=0,
                                        eps=0.01)
    acc = sim.forces()
    if prec == "fp32":
        pos = pos.astype(np.float32).astype(np.float64)
    t = oracle.Tree(pos, m, m, cap=16).traverse(0.5)
    a_ref, _ = t.fmm(order, 0.01)
    assert _rel_rms(acc, a_ref) < tol


def test_mixed_order7_accuracy_vs_fp64_direct(nb, oracle):
    pos, vel, m = ics.plummer(32768, seed=33)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=7, leaf_capacity=32,
                                        fixed_box=0, eps=0.01)
    acc = sim.forces()
    tg = np.random.default_rng(0).choice(len(pos), 2048, replace=False)
    ad, _ = oracle.direct(pos, m, m, eps=0.01, targets=tg)
    assert _rel_rms(acc[tg], ad) < 1e-4


@pytest.mark.parametrize("prec", ["fp32", "mixed", "fp64"])
def test_bitwise_deterministic(nb, prec):
    pos, vel, m = ics.clustered(8192, seed=34)
    p = {"fp32": nb.PREC_FP32, "mixed": nb.PREC_MIXED, "fp64": nb.PREC_FP64}[prec]
    a = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=p, order=4, leaf_capacity=16, fixed_box=0).forces()
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=p, order=4, leaf_capacity=16, fixed_box=0)
    b = sim.forces()
    c = sim.forces()
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(b, c)


def test_leapfrog_trajectory_matches_fp64_direct(nb, oracle):
    pos, vel, m = ics.plummer(512, seed=35)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_FP64, order=8, leaf_capacity=8,
                                        fixed_box=0, eps=0.01, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
    sim.step(10)
    p1, v1, _, _, _ = sim.state("input")
    p2, v2, _ = oracle.leapfrog(pos, vel, m, m, 0.01, 1.0, 1e-3, 10)
    assert np.abs(p1 - p2).max() < 1e-8
    assert np.abs(v1 - v2).max() < 1e-6
    assert abs(sim.time - 0.01) < 1e-12


def test_particles_are_returned_in_leaf_order(nb, oracle):
    pos, vel, m = ics.plummer(1000, seed=36)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=2, leaf_capacity=8,
                                        fixed_box=0)
    sim.forces()
    ps = sim.particles()
    t = oracle.Tree(pos, m, m, cap=8)
    got = np.array([p.position for p in ps])
    np.testing.assert_array_equal(got, pos[t.perm])


def test_diagnostics_conserve_momentum_and_energy(nb):
    pos, vel, m = ics.plummer(4096, seed=37)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=6, leaf_capacity=16,
                                        fixed_box=0, eps=0.01, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
    d0 = sim.diagnostics()
    # Plummer: E = -3 pi / 64 for G = M = a = 1 (softening and truncation shift it slightly)
    assert abs(d0["energy"] + 3 * np.pi / 64) < 0.02
    sim.step(20)
    d1 = sim.diagnostics()
    assert abs(d1["energy"] - d0["energy"]) < 1e-5 * abs(d0["energy"])
    assert np.abs(d1["momentum"] - d0["momentum"]).max() < 1e-6


def test_small_and_degenerate_inputs(nb):
    # one particle: no force
    s = nb.CudaSimulation.from_arrays(np.array([[0.3, 0.2, 0.1]]), None, np.array([1.0]), precision=nb.PREC_FP64,
                                      fixed_box=0)
    assert np.all(s.forces() == 0)
    # two particles: the softened pair force
    p = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    s = nb.CudaSimulation.from_arrays(p, None, np.array([1.0, 2.0]), precision=nb.PREC_FP64, fixed_box=0, eps=0.1,
                                      order=4)
    a = s.forces()
    f = 1.0 / (1.0 + 0.01) ** 1.5
    np.testing.assert_allclose(a, [[2 * f, 0, 0], [-f, 0, 0]], rtol=1e-13)
    # coincident particles: depth cap, finite (zero) softened forces
    p = np.zeros((40, 3))
    p[20:] = 1.0
    s = nb.CudaSimulation.from_arrays(p, None, np.ones(40), precision=nb.PREC_MIXED, fixed_box=0, leaf_capacity=4)
    a = s.forces()
    assert np.all(np.isfinite(a))
    assert a[0, 0] > 0 and a[-1, 0] < 0


def test_errors_are_reported(nb):
    with pytest.raises(nb.NbodyError):
        nb.CudaSimulation.from_arrays(np.zeros((0, 3)), None, np.zeros(0))
    with pytest.raises(nb.NbodyError):
        s = nb.CudaSimulation.from_arrays(np.array([[np.nan, 0, 0], [0, 0, 0]]), None, np.ones(2), fixed_box=0,
                                          precision=nb.PREC_MIXED)
        s.forces()
    # an infinite coordinate stays out of the root box (which must still fit the finite ones) and is
    # reported, in both state precisions
    for bad, prec in ((np.inf, nb.PREC_MIXED), (-np.inf, nb.PREC_FP32)):
        with pytest.raises(nb.NbodyError):
            s = nb.CudaSimulation.from_arrays(np.array([[0.1, bad, 0.2], [0, 0, 0], [0.5, 0.5, 0.5]]), None,
                                              np.ones(3), fixed_box=0, precision=prec)
            s.forces()


def test_trajectory_file_rows(nb, tmp_path):
    """Rows every 2 steps, the reference's particles.csv format, in input and in leaf order."""
    pos, vel, m = ics.plummer(1500, seed=38)
    for order in ("input", "leaf"):
        sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=4, leaf_capacity=16,
                                            fixed_box=0, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
        f = tmp_path / f"traj_{order}.csv"
        sim.trajectory_open(f, every=2, order=order, digits=17)
        want = []
        for _ in range(3):
            t = sim.step(2)
            want.append((t, sim.state(order)[0]))
        sim.step(1)                       # an odd step writes no row
        sim.trajectory_close()
        rows = [np.array(line.split(","), dtype=np.float64) for line in f.read_text().splitlines()]
        assert len(rows) == 3
        for row, (t, p) in zip(rows, want):
            assert row[0] == t
            np.testing.assert_array_equal(row[1:].reshape(-1, 3), p)
        sim.close()


def test_list_capacity_retry_small_theta(nb, oracle):
    """theta = 0.2 makes the near-field lists ~15x the first capacity guess: the lists are rebuilt
    with doubled capacities until they fit, and come out identical to the oracle's."""
    pos, vel, m = ics.plummer(4096, seed=39)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=nb.PREC_MIXED, order=3, leaf_capacity=8,
                                        fixed_box=0, theta=0.2, eps=0.01)
    acc = sim.forces()
    t = oracle.Tree(pos, m, m, cap=8).traverse(0.2)
    assert _set(sim.interactions("p2p")) == _set(t.pairs("p2p"))
    assert _set(sim.interactions("m2l")) == _set(t.pairs("m2l"))
    a_ref, _ = t.fmm(3, 0.01)
    assert _rel_rms(acc, a_ref) < 3e-6
    assert sim.stats()["p2p_leaf_pairs"] == len(t.pairs("p2p"))


def test_direct_sum_matches_oracle(nb, oracle):
    """The device FP64 direct sum (the accuracy reference of every force-error figure) against the
    oracle's FP64 direct sum: 1e-12 relative per target (acceleration) and of the largest potential."""
    rng = np.random.default_rng(44)
    pos, vel, m = ics.plummer(20000, seed=44)
    q = m * rng.uniform(0.5, 1.5, len(m))
    tg = rng.choice(len(m), 2048, replace=False)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, q, precision=nb.PREC_FP64, fixed_box=0, eps=0.01, G=0.7)
    acc, pot = sim.direct(tg)
    a_ref, p_ref = oracle.direct(pos, q, m, eps=0.01, G=0.7, targets=tg)
    err = np.linalg.norm(acc - a_ref, axis=1) / np.linalg.norm(a_ref, axis=1)
    assert err.max() < 1e-12, err.max()
    assert np.abs(pot - p_ref).max() < 1e-12 * np.abs(p_ref).max()


def _escaped(n, seed):
    """Particles of a unit cube, a few of them pushed out through different faces."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 1, (n, 3))
    pos[:5] = [[-0.3, 0.5, 0.5], [0.5, 1.7, 0.5], [0.5, 0.5, -2.2], [1.0, 0.2, 0.2], [0.1, 0.9, 0.999999]]
    m = rng.uniform(1, 10, n)
    q = rng.uniform(0.1, 1, n)
    # values the FP32 state holds exactly, so the oracle bins the same coordinates
    f32 = lambda a: a.astype(np.float32).astype(np.float64)
    return f32(pos), f32(m), f32(q)


def test_escape_policy_grow_matches_oracle(nb, oracle):
    """Reference mode on [0, 1): particles outside the box take the grown root box of oracle.grown_box;
    tree and interaction sets bit-exact, forces within 1e-5 of the largest (the reference-kernel
    tolerance), and the evaluation is counted."""
    pos, m, q = _escaped(6000, 45)
    sim = nb.CudaSimulation([1.0, 1.0, 1.0, 0.0], None, 1e-3)
    sim.set_state(pos, None, m, q)
    acc = sim.forces()
    assert sim.stats()["grown_boxes"] == 1
    box = oracle.grown_box(pos, [0.0, 0.0, 0.0, 1.0])
    assert box[3] == 4.0 and tuple(box[:3]) == (-1.0, 0.0, -3.0), box
    keys, perm, nodes = sim.tree()
    t = oracle.Tree(pos, q, m, box=box, cap=8).traverse(0.5)
    np.testing.assert_array_equal(perm, t.perm.astype(np.int64))
    np.testing.assert_array_equal(nodes, t.nodes)
    assert _set(sim.interactions("p2p")) == _set(t.pairs("p2p"))
    assert _set(sim.interactions("m2l")) == _set(t.pairs("m2l"))
    fl, fn = t.ref_forces_f32(0.01)
    F, Fref = acc * m[:, None], (fl + fn).astype(np.float64)
    assert np.abs(F - Fref).max() <= 1e-5 * np.abs(Fref).max()
    # inside the box again: the fixed box, nothing counted
    sim.set_state(np.clip(pos, 0.0, 0.99), None, m, q)
    sim.forces()
    assert sim.stats()["grown_boxes"] == 0


def test_escape_policy_error(nb):
    pos, m, q = _escaped(3000, 46)
    sim = nb.CudaSimulation([1.0, 1.0, 1.0, 0.0], None, 1e-3)
    sim.set_escape_policy("error")
    sim.set_state(pos, None, m, q)
    with pytest.raises(nb.NbodyError) as e:
        sim.forces()
    assert e.value.code == 7
    # explicit Euler: a failed step leaves the state as it was
    before = sim.state("input")[0]
    with pytest.raises(nb.NbodyError):
        sim.step()
    np.testing.assert_array_equal(sim.state("input")[0], before)
    sim.set_escape_policy("grow")
    assert np.all(np.isfinite(sim.forces()))
