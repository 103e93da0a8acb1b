"""The C++ drop-in (include/nbody/cuda_simulation.h) used the way the
reference's src/main.cpp uses OpenClSimulation, compiled with g++ against
libnbody_gb300.so, gives exactly the Python binding's results."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_drop_in_matches_python_binding(nb, tmp_path):
    cxx = shutil.which("g++")
    assert cxx, "g++ is needed to build the C++ drop-in test"
    from nbody_gb300 import _lib
    exe = tmp_path / "drop_in"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([cxx, "-std=c++14", "-O2", "-Wall", "-Wextra", "-pedantic", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "drop_in_main.cpp"), "-L", libdir, "-lnbody_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    rng = np.random.default_rng(77)
    n, steps = 6000, 3
    data = np.zeros((n, 8), np.float32)
    data[:, :3] = rng.uniform(0, 1, (n, 3))
    data[:, 3:6] = rng.normal(0, 0.05, (n, 3))
    data[:, 6] = rng.uniform(1, 10, n)
    data[:, 7] = rng.uniform(0.1, 1, n)
    f = tmp_path / "particles.f32"
    data.tofile(f)
    out = subprocess.run([str(exe), str(n), str(steps), str(f), "1e-5"], check=True, capture_output=True,
                         text=True).stdout
    fields = out.split()
    t_cpp, count, checksum = float(fields[1]), int(fields[3]), float(fields[5])
    # the same run through the Python binding (reference defaults, box [0, 1), dt 1e-5)
    sim = nb.CudaSimulation([1.0, 1.0, 1.0, 0.0], [nb.Particle(r[:3], r[3:6], r[6], r[7]) for r in data], 1e-5)
    for _ in range(steps):
        t = sim.step()
    pos = np.array([p.position for p in sim.particles()], dtype=np.float32).astype(np.float64)
    ref = float(np.sum(pos[:, 0] + 2.0 * pos[:, 1] + 3.0 * pos[:, 2]))
    assert count == n
    assert abs(t_cpp - np.float32(t)) == 0
    assert abs(checksum - ref) <= 1e-12 * abs(ref)


def _build_drop_in(tmp_path):
    cxx = shutil.which("g++")
    assert cxx, "g++ is needed to build the C++ drop-in test"
    from nbody_gb300 import _lib
    exe = tmp_path / "drop_in"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([cxx, "-std=c++14", "-O2", "-Wall", "-Wextra", "-pedantic", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "drop_in_main.cpp"), "-L", libdir, "-lnbody_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


def test_cpp_drop_in_reference_parameters(nb, oracle, tmp_path):
    """The reference's own main.cpp workload (N uniform in [0, 1), |v| <= 0.1, masses 1..10, charges
    0.1..1, dt 1e-3, reference defaults: order 1, FP32, explicit Euler, capacity 8) for 10 steps at
    N = 100,000.  The charges repel and particles leave [0, 1) within these steps; the escape policy
    grows the root box.  On the final state the library's tree, interaction sets and forces match the
    oracle's restated reference FMM on the same grown box (forces within 1e-5 of the largest)."""
    exe = _build_drop_in(tmp_path)
    n, steps = 100000, 10
    fin = tmp_path / "final.f32"
    out = subprocess.run([str(exe), str(n), str(steps), "-", "1e-3", str(fin)], check=True, capture_output=True,
                         text=True).stdout.split()
    assert int(out[3]) == n and abs(float(out[1]) - 1e-2) < 1e-6
    assert int(out[7]) > 0, "no particle left the box: the escape path was not exercised"
    d = np.fromfile(fin, np.float32).reshape(n, 8).astype(np.float64)
    pos, vel, m, q = d[:, :3], d[:, 3:6], d[:, 6], d[:, 7]
    assert np.all(np.isfinite(pos))
    assert (pos < 0).any() or (pos >= 1).any()
    sim = nb.CudaSimulation([1.0, 1.0, 1.0, 0.0], None, 1e-3)
    sim.set_state(pos, vel, m, q)
    acc = sim.forces()
    assert sim.stats()["grown_boxes"] == 1
    box = oracle.grown_box(pos, [0.0, 0.0, 0.0, 1.0])
    keys, perm, nodes = sim.tree()
    t = oracle.Tree(pos, q, m, box=box, cap=8).traverse(0.5)
    np.testing.assert_array_equal(perm, t.perm.astype(np.int64))
    np.testing.assert_array_equal(nodes, t.nodes)
    fl, fn = t.ref_forces_f32(0.01)
    F, Fref = acc * m[:, None], (fl + fn).astype(np.float64)
    assert np.abs(F - Fref).max() <= 1e-5 * np.abs(Fref).max()


def test_cpp_adjoint_matches_python_binding(nb, tmp_path):
    """Recorded run + reverse sweep through the C++ class equals the Python binding's, bitwise."""
    cxx = shutil.which("g++")
    assert cxx, "g++ is needed to build the C++ adjoint test"
    from nbody_gb300 import _lib, ics
    exe = tmp_path / "adjoint"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([cxx, "-std=c++14", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-pedantic", "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "adjoint_main.cpp"), "-L", libdir, "-lnbody_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    pos, vel, m = ics.plummer(3000, seed=78)
    data = np.zeros((len(m), 8), np.float32)
    data[:, :3], data[:, 3:6], data[:, 6], data[:, 7] = pos, vel, m, m
    f = tmp_path / "particles.f32"
    data.tofile(f)
    out = subprocess.run([str(exe), str(len(m)), "4", "2", str(f)], check=True, capture_output=True,
                         text=True).stdout.split()
    got = [float(out[i]) for i in (1, 3, 5, 7)]
    d = data.astype(np.float64)
    sim = nb.CudaSimulation.from_arrays(d[:, :3], d[:, 3:6], d[:, 6], d[:, 7], precision=nb.PREC_FP64, order=6,
                                        leaf_capacity=16, fixed_box=0, eps=0.01, dt=np.float32(1e-3),
                                        integrator=nb.INTEG_LEAPFROG)
    sim.forward_checkpointed(4, 2)
    xT = sim.state("input")[0].astype(np.float32).astype(np.float64)
    gx0, gv0, gq, gm = sim.backward(xT, None)
    # the C++ checksums are sequential sums (particle-major, then x, y, z; no fused multiply-adds):
    # sum the same way
    w = np.array([1.0, 2.0, 3.0])
    seq = lambda a: float(np.cumsum(a.ravel())[-1])
    want = [seq(gx0 * w), seq(gv0 * w), seq(gq), seq(gm)]
    for g, e in zip(got, want):
        assert abs(g - e) <= 1e-14 * max(abs(e), 1e-300)
