"""The CPU oracle, pinned against the reference's own code.

Fixtures in tests/golden/ come from the reference's kernels and naive path
(tests/golden/make_golden.py).  Where oracle/_ref exists (the reference is
mounted), the live tests also run the reference code on fresh inputs.
"""
import numpy as np
import pytest

from nbody_gb300 import ics


def _pairs_set(a):
    return set(map(tuple, np.asarray(a).tolist()))


def test_naive_port_bitexact_vs_reference_fixture(oracle, golden):
    g = golden("ref_naive_256.npz")
    p, v, t = oracle.naive_steps(g["pos4"], g["vel4"], g["mass"], g["charge"], float(g["G"]), float(g["dt"]),
                                 int(g["steps"]))
    np.testing.assert_array_equal(p, g["pos_out"])
    np.testing.assert_array_equal(v, g["vel_out"])
    assert np.float32(t) == g["t_out"]


def test_naive_port_reproduces_delta_bug(oracle):
    # src/naive_simulation.cpp:10-14 uses the x difference for all three components:
    # the velocity change of every particle has equal components
    rng = np.random.default_rng(0)
    n = 32
    p4 = np.zeros((n, 4), np.float32)
    p4[:, :3] = rng.uniform(0, 1, (n, 3))
    v4 = np.zeros((n, 4), np.float32)
    m = np.ones(n, np.float32)
    _, v, _ = oracle.naive_steps(p4, v4, m, m, 1.0, 1e-3, 1)
    np.testing.assert_allclose(v[:, 0], v[:, 1], rtol=0, atol=0)
    np.testing.assert_allclose(v[:, 0], v[:, 2], rtol=0, atol=0)
    _, vf, _ = oracle.naive_steps(p4, v4, m, m, 1.0, 1e-3, 1, fix_delta=True)
    assert not np.allclose(vf[:, 0], vf[:, 1])


@pytest.mark.parametrize("name", ["ref_fmm_plummer1k.npz", "ref_fmm_cube2k.npz"])
def test_oracle_tree_and_interactions_match_reference_kernels(oracle, golden, name):
    g = golden(name)
    t = oracle.Tree(g["pos"], g["charge"], g["mass"], box=g["box"], cap=int(g["cap"])).traverse(float(g["theta"]))
    np.testing.assert_array_equal(t.nodes, g["nodes"])
    np.testing.assert_array_equal(t.perm.astype(np.int64), g["perm"])
    assert _pairs_set(t.pairs("m2l")) == _pairs_set(g["m2l"])
    assert _pairs_set(t.pairs("p2p")) == _pairs_set(g["p2p"])


@pytest.mark.parametrize("name", ["ref_fmm_plummer1k.npz", "ref_fmm_cube2k.npz"])
def test_oracle_order0_forces_match_reference_kernels(oracle, golden, name):
    g = golden(name)
    t = oracle.Tree(g["pos"], g["charge"], g["mass"], box=g["box"], cap=int(g["cap"])).traverse(float(g["theta"]))
    fl, fn = t.ref_forces_f32(float(g["eps"]))
    scale = np.abs(g["f_leaf"] + g["f_node"]).max()
    assert np.abs(fl - g["f_leaf"]).max() <= 1e-5 * scale
    assert np.abs(fn - g["f_node"]).max() <= 1e-5 * scale
    # the FP64 order-1 Cartesian FMM is the same algorithm: a = (q/m) E
    acc, _ = t.fmm(1, float(g["eps"]))
    ref_acc = (g["f_leaf"] + g["f_node"]).astype(np.float64) / g["mass"][:, None]
    err = np.linalg.norm(acc - ref_acc, axis=1) / np.linalg.norm(ref_acc, axis=1)
    assert err.max() < 2e-5


def test_oracle_matches_live_reference_kernels(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("oracle/_ref not built here (the reference is not mounted)")
    p, v, m = ics.plummer(600, seed=99)
    p = (p + 32.0).astype(np.float32).astype(np.float64)
    box = np.array([0.0, 0.0, 0.0, 64.0])
    t = oracle.Tree(p, m, m, box=box, cap=8).traverse(0.5)
    s = t.perm
    r = oracle.ref_fmm_run(p[s], v[s], m[s], m[s], t.nodes, box, 1e-3)
    assert oracle.both_orientations(r["node_pairs"]) == _pairs_set(t.pairs("m2l"))
    assert oracle.both_orientations(r["leaf_pairs"]) == _pairs_set(t.pairs("p2p"))
    fl, fn = t.ref_forces_f32(0.01)
    inv = np.argsort(s)
    scale = np.abs(r["f_leaf"] + r["f_node"]).max()
    assert np.abs(fl - r["f_leaf"][inv]).max() <= 1e-5 * scale
    assert np.abs(fn - r["f_node"][inv]).max() <= 1e-5 * scale


def test_naive_port_matches_live_reference(oracle):
    if oracle.ref_lib() is None:
        pytest.skip("oracle/_ref not built here (the reference is not mounted)")
    rng = np.random.default_rng(5)
    n = 100
    p4 = np.zeros((n, 4), np.float32)
    p4[:, :3] = rng.uniform(0, 1, (n, 3))
    v4 = np.zeros((n, 4), np.float32)
    v4[:, :3] = rng.normal(0, 0.1, (n, 3))
    m = rng.uniform(1, 10, n).astype(np.float32)
    q = rng.uniform(0.1, 1, n).astype(np.float32)
    a = oracle.naive_steps(p4, v4, m, q, 0.5, 1e-3, 2)
    b = oracle.ref_naive_steps(p4, v4, m, q, 0.5, 1e-3, 2)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_fmm_error_falls_with_order(oracle):
    pos, vel, m = ics.plummer(3000, seed=4)
    t = oracle.Tree(pos, m, m, cap=16).traverse(0.5)
    tg = np.arange(0, 3000, 7)
    ad, pd = oracle.direct(pos, m, m, eps=0.01, targets=tg)
    errs = []
    for p in (1, 3, 5, 7):
        a, pt = t.fmm(p, 0.01)
        e = np.linalg.norm(a[tg] - ad, axis=1) / np.linalg.norm(ad, axis=1)
        errs.append(np.sqrt(np.mean(e ** 2)))
    assert errs[0] > errs[1] > errs[2] > errs[3]
    assert errs[3] < 1e-4


def _check_tree(t, cap, n):
    nodes = t.nodes
    lev, beg, cnt, par, cb, nch = (nodes[:, 0], nodes[:, 4], nodes[:, 5], nodes[:, 6], nodes[:, 7], nodes[:, 8])
    leaves = nch == 0
    # leaves partition the particles
    cover = np.zeros(n, np.int32)
    for b, c in zip(beg[leaves], cnt[leaves]):
        cover[b:b + c] += 1
    assert np.all(cover == 1)
    # capacity rule: internal iff count > cap and level < 21
    assert np.all((cnt[~leaves] > cap) & (lev[~leaves] < 21))
    assert np.all((cnt[leaves] <= cap) | (lev[leaves] == 21))
    # children are contiguous, one level down, and tile the parent's range
    for k in np.nonzero(~leaves)[0]:
        ch = np.arange(cb[k], cb[k] + nch[k])
        assert np.all(par[ch] == k) and np.all(lev[ch] == lev[k] + 1)
        assert beg[ch[0]] == beg[k] and beg[ch[-1]] + cnt[ch[-1]] == beg[k] + cnt[k]
        assert np.all(beg[ch[1:]] == beg[ch[:-1]] + cnt[ch[:-1]])
    # breadth-first: levels non-decreasing
    assert np.all(np.diff(lev) >= 0)
    # keys sorted
    assert np.all(np.diff(t.keys.astype(np.float64)) >= 0)


@pytest.mark.parametrize("case", ["plummer", "cube", "clusters", "duplicates", "tiny", "single"])
def test_oracle_tree_invariants(oracle, case):
    if case == "plummer":
        pos, _, m = ics.plummer(5000, seed=1)
        cap = 16
    elif case == "cube":
        pos, _, m = ics.uniform_cube(5000, seed=2)
        cap = 32
    elif case == "clusters":
        pos, _, m = ics.clustered(6400, seed=3)
        cap = 16
    elif case == "duplicates":
        pos = np.repeat(np.random.default_rng(0).uniform(0, 1, (10, 3)), 30, axis=0)
        m = np.ones(len(pos))
        cap = 8
    elif case == "tiny":
        pos = np.random.default_rng(1).uniform(0, 1, (5, 3))
        m = np.ones(5)
        cap = 8
    else:
        pos = np.array([[0.5, 0.5, 0.5]])
        m = np.ones(1)
        cap = 1
    t = oracle.Tree(pos, m, m, cap=cap)
    _check_tree(t, cap, len(pos))
    t.traverse(0.5)
    a, _ = t.fmm(3, 0.01)
    assert np.all(np.isfinite(a))


def test_direct_sum_conserves_momentum(oracle):
    pos, _, m = ics.plummer(800, seed=8)
    a, _ = oracle.direct(pos, m, m, eps=0.01)
    f = (m[:, None] * a).sum(axis=0)
    assert np.abs(f).max() < 1e-12 * np.abs(m[:, None] * a).sum()


def test_derivative_recursion_matches_oracle(oracle):
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "nbody_gb300",
                                    "csrc"))
    import gen_ops as G
    L = oracle.lib()
    rng = np.random.default_rng(0)
    for p in (1, 4, 7, 8):
        r = rng.normal(size=3) * 2
        eps2 = 1e-3
        Dref = np.zeros(G.T(p))
        L.orc_derivs(p, r, eps2, Dref)
        x, y, z = r
        s = x * x + y * y + z * z + eps2
        D = np.zeros(G.T(p))
        D[0] = s ** -0.5
        for n in G.terms(p)[1:]:
            i = 0 if n[0] > 0 else (1 if n[1] > 0 else 2)
            acc = (2 * n[i] - 1) * r[i] * D[G.idx(G.sub(n, i))]
            for d in range(3):
                if d != i and n[d] >= 1:
                    acc += 2 * n[d] * r[d] * D[G.idx(G.sub(n, d))]
            if n[i] >= 2:
                acc += (n[i] - 1) ** 2 * D[G.idx(G.sub(n, i, 2))]
            for d in range(3):
                if d != i and n[d] >= 2:
                    acc += n[d] * (n[d] - 1) * D[G.idx(G.sub(n, d, 2))]
            D[G.idx(n)] = -acc / s
        np.testing.assert_allclose(D, Dref, rtol=1e-12, atol=1e-14 * np.abs(Dref).max())


def test_generated_operators_are_current():
    """csrc/fmm_ops.inc is the output of csrc/gen_ops.py, byte for byte (the build regenerates it only
    when the generator is newer, so a stale committed copy would go unnoticed)."""
    import os
    import subprocess
    import sys
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "nbody_gb300", "csrc")
    out = subprocess.run([sys.executable, os.path.join(csrc, "gen_ops.py")], capture_output=True, check=True).stdout
    with open(os.path.join(csrc, "fmm_ops.inc"), "rb") as f:
        assert f.read() == out


def test_initial_conditions_are_seeded_and_sane():
    a = ics.plummer(2000, seed=3)
    b = ics.plummer(2000, seed=3)
    np.testing.assert_array_equal(a[0], b[0])
    pos, vel, m = a
    r = np.linalg.norm(pos, axis=1)
    assert r.max() <= 20.0 + 1e-9 and abs(m.sum() - 1) < 1e-12
    # Plummer half-mass radius ~ 1.305 a
    assert 1.1 < np.median(r) < 1.5
    # virial ratio 2K/|W| ~ 1 for the Plummer DF (W = -3 pi / 32 for a = M = G = 1)
    K = 0.5 * (m * (vel ** 2).sum(axis=1)).sum()
    assert 0.85 < 2 * K / (3 * np.pi / 32) < 1.15
    p, v, mm = ics.collision(4000, seed=1)
    assert abs(mm.sum() - 1) < 1e-12 and p.shape == (4000, 3)
    c = ics.clustered(6400, seed=2)
    assert abs(c[2].sum() - 1) < 1e-12


def test_direct_sum_vjp_matches_finite_differences(oracle):
    """The FP64 adjoint oracle against central differences of the FP64 direct sum."""
    rng = np.random.default_rng(11)
    n = 150
    pos = rng.normal(size=(n, 3))
    q = rng.uniform(0.5, 1.5, n)
    m = rng.uniform(0.5, 1.5, n)
    mu = rng.normal(size=(n, 3))
    gx, gq, gm = oracle.direct_vjp(pos, q, m, mu, eps=0.05, G=0.7)

    def S(p=pos, qq=q, mm=m):
        a, _ = oracle.direct(p, qq, mm, eps=0.05, G=0.7)
        return float(np.sum(mu * a))

    for k in (0, 17, 149):
        for d in range(3):
            e = np.zeros_like(pos)
            e[k, d] = 1e-6
            fd = (S(p=pos + e) - S(p=pos - e)) / 2e-6
            assert abs(fd - gx[k, d]) < 1e-6 * max(1.0, abs(gx[k, d]))
        e = np.zeros(n)
        e[k] = 1e-6
        assert abs((S(qq=q + e) - S(qq=q - e)) / 2e-6 - gq[k]) < 1e-6 * max(1.0, abs(gq[k]))
        assert abs((S(mm=m + e) - S(mm=m - e)) / 2e-6 - gm[k]) < 1e-6 * max(1.0, abs(gm[k]))


def test_leapfrog_adjoint_matches_finite_differences(oracle):
    """The trajectory adjoint oracle against central differences of the FP64 direct-sum leapfrog."""
    rng = np.random.default_rng(12)
    n, steps, dt, eps = 40, 4, 0.01, 0.05
    pos, vel = rng.normal(size=(n, 3)), 0.3 * rng.normal(size=(n, 3))
    q = m = rng.uniform(0.5, 1.5, n) / n
    wx, wv = rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    gx0, gv0, gq, gm = oracle.leapfrog_adjoint(pos, vel, q, m, eps, 1.0, dt, steps, wx, wv)

    def L(p=pos, v=vel, qq=q, mm=m):
        p1, v1, _ = oracle.leapfrog(p, v, qq, mm, eps, 1.0, dt, steps)
        return float(np.sum(wx * p1) + np.sum(wv * v1))

    h = 1e-6
    for k in (0, 39):
        for d in range(3):
            e = np.zeros_like(pos)
            e[k, d] = h
            assert abs((L(p=pos + e) - L(p=pos - e)) / (2 * h) - gx0[k, d]) < 1e-6
            assert abs((L(v=vel + e) - L(v=vel - e)) / (2 * h) - gv0[k, d]) < 1e-6
        e = np.zeros(n)
        e[k] = h
        fq = (L(qq=q + e, mm=m) - L(qq=q - e, mm=m)) / (2 * h)
        fm = (L(qq=q, mm=m + e) - L(qq=q, mm=m - e)) / (2 * h)
        assert abs(fq - gq[k]) < 1e-5 * max(1.0, abs(gq[k]))
        assert abs(fm - gm[k]) < 1e-5 * max(1.0, abs(gm[k]))


def test_frozen_tree_fmm_derivative_approaches_direct_vjp(oracle):
    """Finite differences of the oracle FMM with its tree frozen converge to the direct-sum VJP with order."""
    pos, vel, m = ics.plummer(1500, seed=13)
    rng = np.random.default_rng(13)
    mu, d = rng.normal(size=pos.shape), rng.normal(size=pos.shape)
    gx, _, _ = oracle.direct_vjp(pos, m, m, mu, eps=0.01)
    exact = float(np.sum(gx * d))
    t = oracle.Tree(pos, m, m, cap=16).traverse(0.5)
    errs = []
    for p in (1, 4, 8):
        def S(x):
            t.set_particles(pos=x)
            a, _ = t.fmm(p, 0.01)
            return float(np.sum(mu * a))
        fd = (S(pos + 1e-6 * d) - S(pos - 1e-6 * d)) / 2e-6
        errs.append(abs(fd - exact) / abs(exact))
    t.set_particles(pos=pos)
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 1e-5 and errs[0] < 2e-2


def test_adaptive_leapfrog_with_a_pinned_step_is_the_fixed_leapfrog(oracle):
    """dt_min = dt_max pins the adaptive rule to one step: the adaptive restatement then walks the
    same trajectory as the C leapfrog."""
    rng = np.random.default_rng(61)
    pos, vel = rng.normal(size=(200, 3)), 0.1 * rng.normal(size=(200, 3))
    m = np.full(200, 1.0 / 200)
    p1, v1, _, dts = oracle.leapfrog_adaptive(pos, vel, m, m, 0.05, 1.0, 0.1, 0.0, 1e-3, 1e-3, 5)
    p2, v2, _ = oracle.leapfrog(pos, vel, m, m, 0.05, 1.0, 1e-3, 5)
    assert np.all(dts == 1e-3)
    np.testing.assert_allclose(p1, p2, rtol=0, atol=1e-12)
    np.testing.assert_allclose(v1, v2, rtol=0, atol=1e-12)


def test_adaptive_dt_rule(oracle):
    acc = np.array([[3.0, 4.0, 0.0], [0.0, 0.0, 1.0]])          # max |a| = 5
    assert oracle.adaptive_dt(acc, 0.1, 0.05, 1e-6, 1.0) == pytest.approx(0.1 * np.sqrt(0.05 / 5.0), rel=1e-15)
    assert oracle.adaptive_dt(acc, 0.1, 0.05, 1e-6, 1e-3) == 1e-3       # clamped above
    assert oracle.adaptive_dt(acc, 1e-9, 0.05, 1e-6, 1.0) == 1e-6       # clamped below
    assert oracle.adaptive_dt(np.zeros((4, 3)), 0.1, 0.05, 1e-6, 0.5) == 0.5   # no acceleration: dt_max


def test_grown_box_rule(oracle):
    """oracle.grown_box: the fixed box is one cell of the grown box, which covers every point and is
    the smallest such box (half its side would not cover them)."""
    import numpy as np
    fixed = [0.0, 0.0, 0.0, 1.0]
    rng = np.random.default_rng(5)
    inside = rng.uniform(0, 1, (100, 3))
    assert list(oracle.grown_box(inside, fixed)) == fixed
    pts = np.array([[-0.3, 0.5, 0.5], [0.5, 1.7, 0.5], [0.5, 0.5, -2.2], [1.0, 0.2, 0.2]])
    assert list(oracle.grown_box(pts, fixed)) == [-1.0, 0.0, -3.0, 4.0]
    for trial in range(200):
        # dyadic corners, so the origin arithmetic is exact and the cell test below can be exact too
        f = np.array([*(rng.integers(-128, 128, 3) / 64.0), 2.0 ** rng.integers(-3, 4)])
        p = f[:3] + f[3] * rng.normal(0.5, rng.uniform(0.1, 8), (50, 3))
        o0, o1, o2, s = oracle.grown_box(p, f)
        o = np.array([o0, o1, o2])
        assert np.all(o <= p.min(axis=0)) and np.all(o + s > p.max(axis=0))
        k = s / f[3]
        assert k >= 1 and k == 2.0 ** round(np.log2(k))
        a = (f[:3] - o) / f[3]
        assert np.all(a == np.round(a)) and np.all(a >= 0) and np.all(a < k)
        if k > 1:
            assert not (np.all(a < k / 2) and np.all(o + s / 2 > p.max(axis=0)))


def test_block_leapfrog_reduces_to_the_fixed_step(oracle):
    """oracle.leapfrog_block with K = 0 is the kick-drift-kick leapfrog of oracle.leapfrog; with K > 0
    its levels follow block_level and every level is used on a Plummer core."""
    import numpy as np
    from nbody_gb300 import ics
    pos, vel, m = ics.plummer(512, seed=9)
    x0, v0, a0 = oracle.leapfrog(pos, vel, m, m, 0.01, 1.0, 2e-3, 3)
    x1, v1, a1, lv = oracle.leapfrog_block(pos, vel, m, m, 0.01, 1.0, 0.05, 0.0, 2e-3, 0, 3)
    np.testing.assert_allclose(x1, x0, rtol=0, atol=1e-14)
    np.testing.assert_allclose(v1, v0, rtol=0, atol=1e-13)
    assert np.all(lv == 0)
    st = {}
    x2, v2, a2, lv2 = oracle.leapfrog_block(pos, vel, m, m, 0.01, 1.0, 0.02, 0.0, 8e-3, 3, 2, stats=st)
    assert np.all((lv2 >= 0) & (lv2 <= 3)) and len(np.unique(lv2)) >= 2
    # forces are needed at a substep only where some step ends: 2^(deepest level) of the 8 at most
    assert 1 <= st["evaluations"] <= 8
    if lv2.max() < 3:
        assert st["evaluations"] < 8
    st1 = {}
    oracle.leapfrog_block(pos, vel, m, m, 0.01, 1.0, 1e6, 0.0, 8e-3, 3, 1, stats=st1)
    assert st1["evaluations"] == 1                 # every particle on level 0: only the last substep
    # a finer global step moves toward the block result more than the coarse one does
    xf, _, _ = oracle.leapfrog(pos, vel, m, m, 0.01, 1.0, 1e-3, 16)
    xc, _, _ = oracle.leapfrog(pos, vel, m, m, 0.01, 1.0, 8e-3, 2)
    assert np.abs(x2 - xf).max() < np.abs(xc - xf).max()
