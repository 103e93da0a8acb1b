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
    out = subprocess.run([str(exe), str(n), str(steps), str(f)], check=True, capture_output=True, text=True).stdout
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
