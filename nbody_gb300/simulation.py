"""Host-side mirror of the reference's Simulation interface over the C ABI.

The reference exposes ``nbody::Simulation<Scalar, Vector>`` with a
``Particle{position, velocity, mass, charge}`` record, ``step()`` returning
the new time and ``particles()`` returning the particles in octree leaf order
(include/nbody/simulation.h:16-35, src/open_cl_simulation.cpp:53-106).
``CudaSimulation`` keeps those names, argument meanings and the constructor
of ``OpenClSimulation(bounds, particles, time_step, log)``
(include/nbody/open_cl_simulation.h:194-198), and adds array-level calls
(forces, diagnostics, tree and interaction inspection) for callers that do
not go through per-particle records.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import INTEG_EULER, INTEG_LEAPFROG, PREC_FP32, PREC_FP64, PREC_MIXED, NbodyError, check, ptr

__all__ = ["Particle", "CudaSimulation", "params", "PREC_FP32", "PREC_MIXED", "PREC_FP64", "INTEG_LEAPFROG",
           "INTEG_EULER", "NbodyError"]


@dataclass
class Particle:
    """Same fields as Simulation::Particle (include/nbody/simulation.h:16-32)."""
    position: Sequence[float]
    velocity: Sequence[float]
    mass: float
    charge: float


def params(**kw) -> _lib.Params:
    """nbody_params with the reference defaults, overridden by keyword."""
    L = _lib.load()
    p = _lib.Params()
    L.nbody_default_params(C.byref(p))
    for k, v in kw.items():
        if k == "box_min":
            p.box_min[0], p.box_min[1], p.box_min[2] = v
        elif hasattr(p, k):
            setattr(p, k, v)
        else:
            raise TypeError(f"unknown parameter {k}")
    return p


class CudaSimulation:
    """Drop-in for OpenClSimulation on one GB300.

    CudaSimulation(bounds, particles, time_step, log=None, **params)
      bounds     extent of the root box [0, bounds) as in the reference
                 (its fourth component, if given, is ignored)
      particles  iterable of Particle (or use from_arrays)
      time_step  dt
      params     any nbody_params field (precision, order, leaf_capacity,
                 theta, eps, G, integrator, fixed_box, box_min, box_size, ...)
    Errors raise NbodyError (the reference raises std::runtime_error /
    cl::Error, src/open_cl_simulation.cpp:630,648,767).
    """

    def __init__(self, bounds=None, particles: Iterable[Particle] | None = None, time_step: float = 1e-3,
                 log=None, **kw):
        L = _lib.load()
        if bounds is not None and "box_size" not in kw:
            kw["box_size"] = float(max(bounds[0], bounds[1], bounds[2]))
            kw.setdefault("box_min", (0.0, 0.0, 0.0))
            kw.setdefault("fixed_box", 1)
        kw.setdefault("dt", time_step)
        self._p = params(**kw)
        self._log = log
        h = C.c_void_p()
        rc = L.nbody_create(C.byref(self._p), C.byref(h))
        if rc != 0:
            raise NbodyError(rc, L.nbody_last_error(None).decode())
        self._h = h
        self.n = 0
        if particles is not None:
            ps = list(particles)
            pos = np.array([p.position[:3] for p in ps], dtype=np.float64)
            vel = np.array([p.velocity[:3] for p in ps], dtype=np.float64)
            mass = np.array([p.mass for p in ps], dtype=np.float64)
            charge = np.array([p.charge for p in ps], dtype=np.float64)
            self.set_state(pos, vel, mass, charge)

    @classmethod
    def from_arrays(cls, pos, vel=None, mass=None, charge=None, **kw):
        sim = cls(None, None, kw.pop("dt", 1e-3), **kw)
        sim.set_state(pos, vel, mass, charge)
        return sim

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            _lib.load().nbody_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state --------------------------------------------------------------
    def set_state(self, pos, vel=None, mass=None, charge=None, acc=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        vel = np.zeros((n, 3)) if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(n, 3)
        mass = np.ones(n) if mass is None else np.ascontiguousarray(mass, dtype=np.float64).reshape(n)
        charge = None if charge is None else np.ascontiguousarray(charge, dtype=np.float64).reshape(n)
        acc = None if acc is None else np.ascontiguousarray(acc, dtype=np.float64).reshape(n, 3)
        check(self._h, _lib.load().nbody_set_state(self._h, n, ptr(pos), ptr(vel), ptr(mass), ptr(charge), ptr(acc)))
        self.n = n

    def state(self, order: str = "input", with_acc: bool = False):
        """(pos, vel, mass, charge, ids[, acc]); order 'input' or 'leaf' (Morton)."""
        n = self.n
        pos, vel = np.empty((n, 3)), np.empty((n, 3))
        mass, charge = np.empty(n), np.empty(n)
        ids = np.empty(n, np.int64)
        acc = np.empty((n, 3)) if with_acc else None
        check(self._h, _lib.load().nbody_get_state(self._h, 1 if order == "input" else 0, ptr(pos), ptr(vel),
                                                   ptr(mass), ptr(charge), ptr(ids), ptr(acc)))
        return (pos, vel, mass, charge, ids, acc) if with_acc else (pos, vel, mass, charge, ids)

    # -- the reference interface ---------------------------------------------
    def step(self, nsteps: int = 1) -> float:
        """Advances nsteps time steps; returns the new time (Simulation::step)."""
        t = C.c_double()
        if self._log is not None:
            self._log.write(f"Starting a new step (t={self.time}).\n")
        check(self._h, _lib.load().nbody_step(self._h, nsteps, C.byref(t)))
        return t.value

    def particles(self):
        """Particles in octree leaf order, as the reference returns them."""
        pos, vel, mass, charge, _ = self.state("leaf")
        return [Particle(tuple(pos[i]), tuple(vel[i]), float(mass[i]), float(charge[i])) for i in range(self.n)]

    @property
    def time(self) -> float:
        t = C.c_double()
        check(self._h, _lib.load().nbody_get_time(self._h, C.byref(t)))
        return t.value

    # -- additions ------------------------------------------------------------
    def forces(self, potential: bool = False):
        """Accelerations (n,3) [and potential per unit charge (n,)], input order."""
        acc = np.empty((self.n, 3))
        pot = np.empty(self.n) if potential else None
        check(self._h, _lib.load().nbody_compute_forces(self._h, ptr(acc), ptr(pot)))
        return (acc, pot) if potential else acc

    def diagnostics(self):
        out = np.empty(9)
        check(self._h, _lib.load().nbody_diagnostics(self._h, ptr(out)))
        return {"kinetic": out[0], "potential": out[1], "energy": out[0] + out[1], "momentum": out[2:5].copy(),
                "angular_momentum": out[5:8].copy(), "mass": out[8]}

    def tree(self):
        """(keys, perm, nodes) of the last tree; nodes rows as in the C ABI."""
        L = _lib.load()
        n, nn, nl, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int()
        check(self._h, L.nbody_tree_info(self._h, C.byref(n), C.byref(nn), C.byref(nl), C.byref(d)))
        keys = np.empty(n.value, np.uint64)
        perm = np.empty(n.value, np.int64)
        nodes = np.empty((nn.value, 9), np.int32)
        check(self._h, L.nbody_get_tree(self._h, ptr(keys), ptr(perm), ptr(nodes)))
        return keys, perm, nodes

    def interactions(self, which: str):
        """(target, source) node pairs: which = 'm2l' or 'p2p'."""
        L = _lib.load()
        w = 0 if which == "m2l" else 1
        k = C.c_int64()
        check(self._h, L.nbody_get_interactions(self._h, w, C.byref(k), None))
        out = np.empty((max(k.value, 1), 2), np.int32)
        check(self._h, L.nbody_get_interactions(self._h, w, C.byref(k), ptr(out)))
        return out[: k.value]

    def direct(self, targets):
        """FP64 softened direct-sum accelerations and potentials of the targets (input indices), on the GPU."""
        tg = np.ascontiguousarray(targets, dtype=np.int64)
        acc = np.empty((len(tg), 3))
        pot = np.empty(len(tg))
        check(self._h, _lib.load().nbody_direct_forces(self._h, len(tg), ptr(tg), ptr(acc), ptr(pot)))
        return acc, pot

    # -- adjoint ----------------------------------------------------------------
    def force_vjp(self, mu):
        """For S = sum_i mu_i . a_i at the current positions: (dS/dx (n,3), dS/dq (n,), dS/dm (n,)),
        input order, tree and interaction lists held fixed."""
        mu = np.ascontiguousarray(mu, dtype=np.float64).reshape(self.n, 3)
        gx = np.empty((self.n, 3))
        gq = np.empty(self.n)
        gm = np.empty(self.n)
        check(self._h, _lib.load().nbody_force_vjp(self._h, ptr(mu), ptr(gx), ptr(gq), ptr(gm)))
        return gx, gq, gm

    def forward_checkpointed(self, nsteps: int, every: int = 1) -> float:
        """nsteps leapfrog steps recorded for backward(): snapshots every `every` steps (the last interval's
        evaluations are kept whole as they happen, the reverse sweep recomputes the earlier intervals),
        or with every = 0 every time point's whole evaluation (no re-evaluation in the reverse sweep)."""
        t = C.c_double()
        check(self._h, _lib.load().nbody_forward_checkpointed(self._h, int(nsteps), int(every), C.byref(t)))
        return t.value

    def backward(self, gx_final=None, gv_final=None):
        """Reverse sweep of the recorded run: given dL/dx_N and dL/dv_N (n,3; None = 0), returns
        (dL/dx_0, dL/dv_0, dL/dq, dL/dm) in input order."""
        gxT = None if gx_final is None else np.ascontiguousarray(gx_final, dtype=np.float64).reshape(self.n, 3)
        gvT = None if gv_final is None else np.ascontiguousarray(gv_final, dtype=np.float64).reshape(self.n, 3)
        gx0 = np.empty((self.n, 3))
        gv0 = np.empty((self.n, 3))
        gq = np.empty(self.n)
        gm = np.empty(self.n)
        check(self._h, _lib.load().nbody_backward(self._h, ptr(gxT), ptr(gvT), ptr(gx0), ptr(gv0), ptr(gq),
                                                  ptr(gm)))
        return gx0, gv0, gq, gm

    def replay(self, pos, vel=None, mass=None, charge=None, steps=None):
        """Frozen-structure replay of the run recorded with forward_checkpointed(steps, 0): from this
        initial state (input order), `steps` leapfrog steps whose evaluations reuse the recorded trees,
        lists and near-field plans.  Returns the final (pos, vel) in input order; the context keeps
        the recorded run."""
        n = self.n
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(n, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(n, 3)
        mass = np.ones(n) if mass is None else np.ascontiguousarray(mass, dtype=np.float64).reshape(n)
        charge = None if charge is None else np.ascontiguousarray(charge, dtype=np.float64).reshape(n)
        po, vo = np.empty((n, 3)), np.empty((n, 3))
        check(self._h, _lib.load().nbody_forward_replay(self._h, ptr(pos), ptr(vel), ptr(mass), ptr(charge),
                                                        -1 if steps is None else int(steps), ptr(po), ptr(vo)))
        return po, vo

    def trajectory_open(self, path, every: int = 1, order: str = "leaf", digits: int = 6):
        """Append a CSV row (time, x, y, z of every particle) every `every` steps, as the reference's
        main loop writes particles.csv; order 'leaf' (the reference's) or 'input'."""
        check(self._h, _lib.load().nbody_trajectory_open(self._h, str(path).encode(), int(every),
                                                         1 if order == "input" else 0, int(digits)))

    def trajectory_close(self):
        check(self._h, _lib.load().nbody_trajectory_close(self._h))

    def set_timestep_control(self, mode: str = "adaptive", eta: float = 0.02, length: float = 0.0,
                             dt_min: float = 1e-8, dt_max: float = 1e-2):
        """Adaptive global step: dt = clamp(eta * sqrt(length / max|a|), dt_min, dt_max) from the last
        evaluation's accelerations (length <= 0: the softening eps); mode "block": individual steps
        dt_max / 2^k per particle from the same criterion on its own |a|, dt_max / dt_min = 2^K substeps
        per step(); mode "fixed" restores params.dt."""
        m = {"fixed": _lib.DT_FIXED, "adaptive": _lib.DT_ADAPTIVE, "block": _lib.DT_BLOCK}[mode]
        check(self._h, _lib.load().nbody_set_timestep_control(self._h, m, float(eta), float(length), float(dt_min),
                                                              float(dt_max)))

    def levels(self):
        """Block steps: each particle's level k (input order) of its last step, dt = dt_max / 2^k."""
        out = np.empty(self.n, np.int32)
        check(self._h, _lib.load().nbody_get_levels(self._h, ptr(out)))
        return out

    def last_timestep(self) -> float:
        """dt of the last step taken."""
        dt = C.c_double()
        check(self._h, _lib.load().nbody_last_timestep(self._h, C.byref(dt)))
        return dt.value

    def device_memory(self):
        """(bytes held on the device now, high-water mark since creation)."""
        cur, peak = C.c_int64(), C.c_int64()
        check(self._h, _lib.load().nbody_device_memory(self._h, C.byref(cur), C.byref(peak)))
        return cur.value, peak.value

    def stats(self):
        """Work counts of the last evaluation (pairs, nodes, leaves, depth, launches), evaluations that
        took a grown root box, and of the last block step: leaves over its evaluated substeps, those
        whose near field ran, and its force evaluations."""
        out = np.zeros(11, np.int64)
        check(self._h, _lib.load().nbody_get_stats(self._h, ptr(out), 11))
        keys = ("m2l_pairs", "p2p_particle_pairs", "p2p_leaf_pairs", "nodes", "leaves", "depth", "launches",
                "grown_boxes", "block_leaves", "block_active_leaves", "block_evaluations")
        return dict(zip(keys, (int(v) for v in out)))

    def set_escape_policy(self, policy: str = "grow"):
        """What an evaluation does when a particle lies outside a fixed root box: "grow" takes the
        smallest power-of-two multiple of the box that has it as a cell and covers every particle;
        "error" fails with NbodyError (code 7)."""
        p = {"grow": _lib.ESCAPE_GROW, "error": _lib.ESCAPE_ERROR}[policy]
        check(self._h, _lib.load().nbody_set_escape_policy(self._h, p))

    def set_wait_limits(self, scan_polls: int = 0, copy_cycles: int = 0):
        """Bounds of the device-side waits (<= 0: the defaults of about a second)."""
        check(self._h, _lib.load().nbody_set_wait_limits(self._h, int(scan_polls), int(copy_cycles)))

    def set_timing(self, on: bool = True):
        check(self._h, _lib.load().nbody_set_timing(self._h, int(on)))

    PHASES = ("kick_drift_keys", "sort_gather", "tree", "upward", "lists", "far_field", "near_field")
    VJP_PHASES = ("adj_seed_l2pT", "adj_l2lT", "adj_m2lT", "adj_m2mT", "adj_near_rest_finish")

    def phase_times(self):
        """Device ms of the last force evaluation's phases (PHASES)."""
        out = np.zeros(12, np.float32)
        check(self._h, _lib.load().nbody_phase_times(self._h, ptr(out), 12))
        return out[:7]

    def vjp_phase_times(self):
        """Device ms of the last force_vjp's phases (VJP_PHASES)."""
        out = np.zeros(12, np.float32)
        check(self._h, _lib.load().nbody_phase_times(self._h, ptr(out), 12))
        return out[7:]

    @property
    def stream(self) -> int:
        return _lib.load().nbody_stream(self._h) or 0
