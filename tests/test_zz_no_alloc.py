"""The allocation-free direct sum (nbody_direct_forces_static).

It is meant for callers that must not allocate device memory themselves (a
host framework that owns the memory budget, or a latency-critical path), so
the test hands it caller-owned device buffers (allocated here by torch, not by
the library) and checks it against the allocating entry point
nbody_direct_forces on the same state, on two calls in a row: the second call
reuses the library's shared scratch array as the first left it.  Tolerance is
the FP64 one of the other tests (1e-12 relative).  This file runs last so a
failure here cannot hide the others.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr())


def test_static_direct_sum_matches_allocating_entry_point(nb):
    import torch
    from nbody_gb300 import _lib, ics
    L = _lib.load()
    rng = np.random.default_rng(41)
    pos, vel, m = ics.plummer(20000, seed=41)
    q = m * rng.uniform(0.5, 1.5, len(m))
    n = len(m)
    sim = nb.CudaSimulation.from_arrays(pos, vel, m, q, precision=nb.PREC_FP64, eps=0.01, G=0.7, fixed_box=0)
    dev = torch.device("cuda", 0)
    d_pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
    d_m = torch.tensor(m, dtype=torch.float64, device=dev)
    d_q = torch.tensor(q, dtype=torch.float64, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for call, nt in enumerate((3000, 5000)):
        tg = rng.choice(n, nt, replace=False).astype(np.int64)
        ref_acc, ref_pot = sim.direct(tg)
        d_t = torch.tensor(tg, dtype=torch.int64, device=dev)
        d_acc = torch.full((nt, 3), float("nan"), dtype=torch.float64, device=dev)
        d_pot = torch.full((nt,), float("nan"), dtype=torch.float64, device=dev)
        rc = L.nbody_direct_forces_static(0, n, _p(d_pos), _p(d_m), _p(d_q), 0.01, 0.7, nt, _p(d_t), _p(d_acc),
                                          _p(d_pot), stream)
        assert rc == 0, L.nbody_last_error(None)
        torch.cuda.synchronize(dev)
        acc = d_acc.cpu().numpy()
        pot = d_pot.cpu().numpy()
        err = np.linalg.norm(acc - ref_acc, axis=1) / np.linalg.norm(ref_acc, axis=1)
        assert err.max() < 1e-12, (call, err.max())
        assert np.abs(pot - ref_pot).max() < 1e-12 * np.abs(ref_pot).max(), call


def test_static_direct_sum_rejects_oversize_requests(nb):
    import torch
    from nbody_gb300 import _lib
    L = _lib.load()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    idx = torch.zeros(4, dtype=torch.int64, device=dev)
    rc = L.nbody_direct_forces_static(0, 4, _p(buf), _p(buf), None, 0.01, 1.0, 131073, _p(idx), _p(buf), None,
                                      None)
    assert rc == 1
    assert b"131072" in L.nbody_last_error(None)


def test_static_direct_sum_limits_and_bad_targets_against_the_oracle(nb, oracle):
    """The documented limits, on two calls in a row against the CPU oracle's FP64 direct sum (1e-12):
    exactly 131,072 targets (indices repeated) are accepted; target indices outside [0, n) give NaN rows
    and leave the other rows exact.  The calling thread's current device is the same afterwards."""
    import torch
    from nbody_gb300 import _lib, ics
    L = _lib.load()
    rng = np.random.default_rng(42)
    pos, vel, m = ics.plummer(3000, seed=42)
    n = len(m)
    dev = torch.device("cuda", 0)
    d_pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
    d_m = torch.tensor(m, dtype=torch.float64, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    before = torch.cuda.current_device()
    for call, nt in enumerate((131072, 257)):
        tg = rng.integers(0, n, nt).astype(np.int64)
        bad = np.zeros(nt, bool)
        if call == 1:
            bad[[3, 100, 256]] = True
            tg[bad] = [-1, n, 10 ** 12]
        d_t = torch.tensor(tg, dtype=torch.int64, device=dev)
        d_acc = torch.zeros((nt, 3), dtype=torch.float64, device=dev)
        d_pot = torch.zeros((nt,), dtype=torch.float64, device=dev)
        rc = L.nbody_direct_forces_static(0, n, _p(d_pos), _p(d_m), None, 0.01, 1.0, nt, _p(d_t), _p(d_acc),
                                          _p(d_pot), stream)
        assert rc == 0, L.nbody_last_error(None)
        torch.cuda.synchronize(dev)
        acc, pot = d_acc.cpu().numpy(), d_pot.cpu().numpy()
        assert np.all(np.isnan(acc[bad])) and np.all(np.isnan(pot[bad]))
        good = np.unique(tg[~bad])
        a_ref, p_ref = oracle.direct(pos, m, m, eps=0.01, G=1.0, targets=good)
        row = {t: k for k, t in enumerate(good)}
        idx = np.array([row[t] for t in tg[~bad]])
        err = np.linalg.norm(acc[~bad] - a_ref[idx], axis=1) / np.linalg.norm(a_ref[idx], axis=1)
        assert err.max() < 1e-12, (call, err.max())
        assert np.abs(pot[~bad] - p_ref[idx]).max() < 1e-12 * np.abs(p_ref).max()
    assert torch.cuda.current_device() == before
