"""The NBODY_DEBUG_BOUNDS build of the library (libnbody_gb300_debug.so).

Bounds checking without compute-sanitizer: the debug build checks every index its kernels read from device data (the sorted-order
permutation, node ids of the pending, far-field and near-field lists, the
particle ranges of near-field partners, radix-scatter destinations); an index
out of range is replaced by an in-bounds one and reported as NBODY_ERR_CUDA at
the end of the evaluation, so a bug shows as an error, never as a fault.

The test builds it (once per session), then runs, in a child process bound to
it through NBODY_LIB_PATH, small cases of every precision form: force
evaluations (data cube, fixed box with escapes, a small opening angle that
overflows the first list capacity), leapfrog and Euler steps, a force VJP, a
checkpointed run with its reverse sweep and a frozen-structure replay.  No
check may fire, and the forces must equal the release build's (1e-12
relative for FP64, 1e-6 for the FP32 bulk forms: the checks change no
arithmetic).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import nbody_gb300 as nb
from nbody_gb300 import _lib, ics
assert _lib.load().nbody_debug_bounds() == 1, "not the debug build"
out = {}
pos, vel, m = ics.plummer(3000, seed=71)
cpos, cvel, cm = ics.clustered(4000, seed=72)
for name, prec in (("fp32", nb.PREC_FP32), ("mixed", nb.PREC_MIXED), ("fp64", nb.PREC_FP64)):
    s = nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=prec, order=5, leaf_capacity=16, fixed_box=0,
                                      eps=0.01, dt=1e-3, integrator=nb.INTEG_LEAPFROG)
    out[name + "_plummer"] = s.forces()
    s.step(3)
    s.force_vjp(np.ones_like(pos))
    s.forward_checkpointed(4, 2)
    s.backward(np.ones_like(pos), None)
    s.forward_checkpointed(3, 0)
    s.replay(pos, vel, m, m)
    s.close()
    s = nb.CudaSimulation.from_arrays(cpos, cvel, cm, cm, precision=prec, order=4, leaf_capacity=8, fixed_box=0,
                                      eps=0.01, theta=0.2)
    out[name + "_clusters_theta02"] = s.forces()
    s.close()
    rng = np.random.default_rng(73)
    p = rng.uniform(0, 1, (3000, 3))
    p[:3] = [[-0.5, 0.5, 0.5], [0.5, 1.5, 0.5], [0.5, 0.5, 2.5]]
    s = nb.CudaSimulation([1.0, 1.0, 1.0, 0.0], None, 1e-3, precision=prec)
    s.set_state(p, None, np.ones(3000), np.ones(3000))
    out[name + "_escape"] = s.forces()
    s.step(2)
    s.close()
np.savez(sys.argv[2], **out)
'''


@pytest.fixture(scope="module")
def debug_lib():
    from nbody_gb300 import build
    return build.build(debug=True)


def test_debug_build_runs_every_path_without_a_failed_check(nb, debug_lib, tmp_path):
    out = tmp_path / "debug.npz"
    env = dict(os.environ, NBODY_LIB_PATH=debug_lib)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, str(out)], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    got = dict(np.load(out))
    from nbody_gb300 import _lib, ics
    assert _lib.load().nbody_debug_bounds() == 0
    # the same forces from the release build in this process
    pos, vel, m = ics.plummer(3000, seed=71)
    cpos, cvel, cm = ics.clustered(4000, seed=72)
    rng = np.random.default_rng(73)
    p = rng.uniform(0, 1, (3000, 3))
    p[:3] = [[-0.5, 0.5, 0.5], [0.5, 1.5, 0.5], [0.5, 0.5, 2.5]]
    for name, prec in (("fp32", nb.PREC_FP32), ("mixed", nb.PREC_MIXED), ("fp64", nb.PREC_FP64)):
        tol = 1e-12 if name == "fp64" else 1e-6
        want = {
            "plummer": nb.CudaSimulation.from_arrays(pos, vel, m, m, precision=prec, order=5, leaf_capacity=16,
                                                     fixed_box=0, eps=0.01).forces(),
            "clusters_theta02": nb.CudaSimulation.from_arrays(cpos, cvel, cm, cm, precision=prec, order=4,
                                                              leaf_capacity=8, fixed_box=0, eps=0.01,
                                                              theta=0.2).forces(),
        }
        s = nb.CudaSimulation([1.0, 1.0, 1.0, 0.0], None, 1e-3, precision=prec)
        s.set_state(p, None, np.ones(3000), np.ones(3000))
        want["escape"] = s.forces()
        for case, w in want.items():
            g = got[f"{name}_{case}"]
            err = np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-300)
            assert err.max() <= tol, (name, case, err.max())
