"""ctypes binding for the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module, and only as the checker or the timed CPU baseline.
The product (``nbody_gb300``) never imports it.

``liboracle.so`` is the C restatement in ``nbody_oracle.c``.  ``libnbody_ref.so``
(``oracle/_ref``) is the reference's own code compiled from its sources; it only
exists where the reference is mounted and is used to pin the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


def reference_dir() -> str:
    """Where the reference tree is mounted: $NBODY_REFERENCE_DIR, else the Makefile's default."""
    env = os.environ.get("NBODY_REFERENCE_DIR")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip()


def build(ref: bool | None = None) -> None:
    """Compile liboracle.so (and, if the reference is mounted, libnbody_ref.so)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    rdir = reference_dir()
    if ref is None:
        ref = bool(rdir) and os.path.isdir(os.path.join(rdir, "src"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={rdir}"], check=True)


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.path.join(HERE, "_build", "liboracle.so")
    if not os.path.exists(path):
        build(ref=False)
    L = C.CDLL(path)
    L.orc_create.restype = C.c_void_p
    L.orc_create.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _f64p, C.c_int, C.c_int]
    L.orc_destroy.argtypes = [C.c_void_p]
    L.orc_nnodes.restype = C.c_int64
    L.orc_nnodes.argtypes = [C.c_void_p]
    L.orc_depth.restype = C.c_int
    L.orc_depth.argtypes = [C.c_void_p]
    L.orc_get_order.argtypes = [C.c_void_p, _u32p, _u64p]
    L.orc_get_nodes.argtypes = [C.c_void_p, _i32p]
    L.orc_traverse.argtypes = [C.c_void_p, C.c_double]
    L.orc_list_size.restype = C.c_int64
    L.orc_list_size.argtypes = [C.c_void_p, C.c_int]
    L.orc_get_list.argtypes = [C.c_void_p, C.c_int, _i32p]
    L.orc_fmm.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, _f64p, _f64p, C.c_void_p, C.c_void_p]
    L.orc_ref_forces_f32.argtypes = [C.c_void_p, C.c_float, _f32p, _f32p]
    L.orc_set_particles.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.orc_set_particles.restype = None
    L.orc_direct.argtypes = [C.c_int64, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_int64, C.c_void_p,
                             _f64p, C.c_void_p, C.c_int]
    L.orc_leapfrog.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_double,
                               C.c_int, _f64p, C.c_int, C.c_int]
    L.orc_naive_steps.restype = C.c_float
    L.orc_naive_steps.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_float, C.c_int, C.c_int]
    L.orc_naive_kick_mt.restype = C.c_int64
    L.orc_naive_kick_mt.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_float, C.c_int, C.c_int,
                                    C.c_int, C.c_int]
    L.orc_naive_rows.restype = C.c_int64
    L.orc_naive_rows.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int]
    L.orc_direct_vjp.argtypes = [C.c_int64, _f64p, _f64p, _f64p, C.c_double, C.c_double, _f64p, _f64p, _f64p, _f64p,
                                 C.c_int]
    L.orc_leapfrog_adjoint.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _f64p, C.c_double, C.c_double, C.c_double,
                                       C.c_int, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p, C.c_int]
    L.orc_morton_keys.argtypes = [C.c_int64, _f64p, _f64p, _u64p]
    L.orc_derivs.argtypes = [C.c_int, _f64p, C.c_double, _f64p]
    L.orc_nterms.restype = C.c_int
    L.orc_nterms.argtypes = [C.c_int]
    _LIB = L
    return L


def ref_lib():
    """The reference's own code compiled here, or None where it was not built."""
    global _REF
    if _REF is not None:
        return _REF
    path = os.path.join(HERE, "_ref", "libnbody_ref.so")
    if not os.path.exists(path):
        return None
    try:
        R = C.CDLL(path)
    except OSError:
        return None
    R.ref_naive_steps.restype = C.c_float
    R.ref_naive_steps.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_float, C.c_int]
    R.ref_fmm_run.restype = C.c_int
    R.ref_fmm_run.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, _i32p, _f64p, C.c_float, C.c_int,
                              C.POINTER(C.c_int), _i32p, C.POINTER(C.c_int), _i32p, _f32p, _f32p, _f32p, _f32p]
    _REF = R
    return R


NODE_FIELDS = ("level", "ix", "iy", "iz", "begin", "count", "parent", "child_begin", "nchild")


def theta2_f32(theta: float) -> float:
    """theta^2 as the reference forms it in single precision (src/interaction.cl:78)."""
    t = np.float32(theta)
    return float(np.float32(t * t))


class Tree:
    """Sorted particles + breadth-first octree + interaction lists (oracle)."""

    def __init__(self, pos, q=None, m=None, box=None, cap=16, maxlevel=21):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        self.n = n
        q = np.ones(n) if q is None else np.ascontiguousarray(q, dtype=np.float64)
        m = q.copy() if m is None else np.ascontiguousarray(m, dtype=np.float64)
        if box is None:
            box = bounding_box(pos)
        self.box = np.ascontiguousarray(box, dtype=np.float64)
        L = lib()
        self._h = L.orc_create(n, pos.reshape(-1), q, m, self.box, cap, maxlevel)
        self.nnodes = L.orc_nnodes(self._h)
        self.depth = L.orc_depth(self._h)
        self.perm = np.zeros(max(n, 1), np.uint32)
        self.keys = np.zeros(max(n, 1), np.uint64)
        L.orc_get_order(self._h, self.perm, self.keys)
        self.perm, self.keys = self.perm[:n], self.keys[:n]
        nodes = np.zeros((self.nnodes, 9), np.int32)
        L.orc_get_nodes(self._h, nodes)
        self.nodes = nodes
        self._lists = None

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def field(self, name):
        return self.nodes[:, NODE_FIELDS.index(name)]

    def traverse(self, theta=0.5):
        lib().orc_traverse(self._h, theta2_f32(theta))
        self._lists = {}
        return self

    def pairs(self, which):
        """which in {'m2l','p2p','pend'}: int32 (k, 2) rows (target, source)."""
        w = {"m2l": 0, "p2p": 1, "pend": 2}[which]
        L = lib()
        k = L.orc_list_size(self._h, w)
        out = np.zeros((max(k, 1), 2), np.int32)
        L.orc_get_list(self._h, w, out)
        return out[:k]

    def fmm(self, order, eps, G=1.0):
        acc = np.zeros(3 * max(self.n, 1))
        pot = np.zeros(max(self.n, 1))
        rc = lib().orc_fmm(self._h, order, eps, G, acc, pot, None, None)
        if rc != 0:
            raise RuntimeError("orc_fmm failed (traverse first; order in 1..10)")
        return acc[: 3 * self.n].reshape(-1, 3), pot[: self.n]

    def set_particles(self, pos=None, q=None, m=None):
        """New positions / charges / masses (input order) with the tree and lists kept (frozen tree)."""
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)[: k * self.n].copy()
                for a, k in ((pos, 3), (q, 1), (m, 1))]
        ptrs = [None if a is None else a.ctypes.data_as(C.c_void_p) for a in keep]
        lib().orc_set_particles(self._h, *ptrs)
        return self

    def ref_forces_f32(self, eps=0.01):
        fl = np.zeros(3 * max(self.n, 1), np.float32)
        fn = np.zeros(3 * max(self.n, 1), np.float32)
        lib().orc_ref_forces_f32(self._h, eps, fl, fn)
        return fl[: 3 * self.n].reshape(-1, 3), fn[: 3 * self.n].reshape(-1, 3)


def bounding_box(pos):
    """Power-of-two cube enclosing pos, origin on a multiple of side/2.

    Same rule as the device (data-bounding root box): side = smallest power of
    two >= (max extent) * (1 + 2^-20), origin = floor(min / (side/2)) * (side/2),
    and doubled until the box covers every particle.
    """
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    if pos.shape[0] == 0:
        return np.array([0.0, 0.0, 0.0, 1.0])
    lo, hi = pos.min(axis=0), pos.max(axis=0)
    ext = float((hi - lo).max()) * (1.0 + 2.0 ** -20)
    side = 1.0
    while side < ext:
        side *= 2.0
    while side * 0.5 >= ext and ext > 0:
        side *= 0.5
    while True:
        half = side / 2.0
        origin = np.floor(lo / half) * half
        if np.all(origin + side > hi):
            return np.array([origin[0], origin[1], origin[2], side])
        side *= 2.0


def grown_box(pos, fixed):
    """Root box of a step whose particles leave the fixed box (fx, fy, fz, side), policy "grow".

    Restates the library's rule for particles outside the reference's [0, bounds) root box (the
    reference leaves that case to its external octree, src/open_cl_simulation.cpp:43-47,120-123):
    per axis the origin moves down by a whole number a of box sides until it is at or below the
    lowest coordinate, then the side doubles until every coordinate is below origin + side, so the
    fixed box stays one cell of the grown box.  Returns the fixed box itself if nothing left it.
    """
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    f = np.asarray(fixed[:3], dtype=np.float64)
    fs = float(fixed[3])
    lo, hi = pos.min(axis=0), pos.max(axis=0)
    if np.all(lo >= f) and np.all(hi < f + fs):
        return np.array([f[0], f[1], f[2], fs])
    o = np.zeros(3)
    a = np.zeros(3)
    for d in range(3):
        a[d] = np.ceil((f[d] - lo[d]) / fs) if lo[d] < f[d] else 0.0
        it = 0
        while it < 4 and f[d] - a[d] * fs > lo[d]:
            a[d] += 1.0
            it += 1
        o[d] = f[d] - a[d] * fs
    s = fs
    while not all(a[d] * fs < s and o[d] + s > hi[d] for d in range(3)):
        s *= 2.0
    return np.array([o[0], o[1], o[2], s])


def ref_mode_run(pos, vel, q, m, box, cap, theta, eps, dt, steps, escape="grow"):
    """The reference's FMM step repeated: order 0 (monopole about the geometric centre, constant
    local field), FP32 arithmetic, explicit Euler v += F/m dt, x += v_old dt
    (src/open_cl_simulation.cpp:572-616, src/field.cl, src/force.cl), the octree rebuilt every
    step over the fixed root box (grown by grown_box when a particle has left it).  Inputs and
    outputs are in input order; returns (pos, vel) as float32."""
    x = np.asarray(pos, dtype=np.float32).reshape(-1, 3).copy()
    v = np.asarray(vel, dtype=np.float32).reshape(-1, 3).copy()
    q64 = np.asarray(q, dtype=np.float64)
    m64 = np.asarray(m, dtype=np.float64)
    m32 = m64.astype(np.float32)[:, None]
    dt32 = np.float32(dt)
    for _ in range(steps):
        b = grown_box(x.astype(np.float64), box) if escape == "grow" else np.asarray(box, np.float64)
        t = Tree(x.astype(np.float64), q64, m64, box=b, cap=cap).traverse(theta)
        fl, fn = t.ref_forces_f32(eps)
        F = (fl + fn).astype(np.float32)
        v_old = v.copy()
        v = v + (F / m32) * dt32
        x = x + v_old * dt32
        del t
    return x, v


def direct(pos, q=None, m=None, eps=0.01, G=1.0, targets=None, nthreads=None):
    """FP64 softened direct sum: (acc, pot) for the targets (default all)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    n = pos.shape[0]
    q = np.ones(n) if q is None else np.ascontiguousarray(q, dtype=np.float64)
    m = q.copy() if m is None else np.ascontiguousarray(m, dtype=np.float64)
    nthreads = nthreads or min(os.cpu_count() or 1, 32)
    if targets is None:
        nt, tp = n, None
        tgt = None
    else:
        tgt = np.ascontiguousarray(targets, dtype=np.int64)
        nt, tp = tgt.shape[0], tgt.ctypes.data
    acc = np.zeros(3 * max(nt, 1))
    pot = np.zeros(max(nt, 1))
    lib().orc_direct(n, pos.reshape(-1), q, m, eps, G, nt, tp, acc, pot.ctypes.data, nthreads)
    return acc[: 3 * nt].reshape(-1, 3), pot[:nt]


def leapfrog(pos, vel, q, m, eps, G, dt, steps, nthreads=None):
    """FP64 direct-sum kick-drift-kick leapfrog; returns (pos, vel, acc)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1).copy()
    n = pos.shape[0] // 3
    acc = np.zeros(3 * n)
    q = np.ascontiguousarray(q, dtype=np.float64)
    m = np.ascontiguousarray(m, dtype=np.float64)
    lib().orc_leapfrog(n, pos, vel, q, m, eps, G, dt, steps, acc, 0, nthreads or min(os.cpu_count() or 1, 32))
    return pos.reshape(-1, 3), vel.reshape(-1, 3), acc.reshape(-1, 3)


def adaptive_dt(acc, eta, length, dt_min, dt_max):
    """The adaptive step rule of nbody_set_timestep_control: clamp(eta * sqrt(length / max|a|), dt_min,
    dt_max), with max|a|^2 summed per particle as x*x + y*y + z*z.  The reference only lists a variable
    time step as a goal (its TODO file), so this restates the library's own rule."""
    acc = np.asarray(acc, dtype=np.float64).reshape(-1, 3)
    a2 = float(np.max(acc[:, 0] * acc[:, 0] + acc[:, 1] * acc[:, 1] + acc[:, 2] * acc[:, 2])) if len(acc) else 0.0
    dt = eta * np.sqrt(length / np.sqrt(a2)) if a2 > 0.0 else dt_max
    if not dt >= dt_min:
        dt = dt_min
    return min(dt, dt_max)


def leapfrog_adaptive(pos, vel, q, m, eps, G, eta, length, dt_min, dt_max, steps, nthreads=None):
    """FP64 direct-sum kick-drift-kick leapfrog whose step n takes adaptive_dt of the accelerations at
    its start (length <= 0: eps); returns (pos, vel, acc, dts)."""
    pos = np.array(pos, dtype=np.float64).reshape(-1, 3)
    vel = np.array(vel, dtype=np.float64).reshape(-1, 3)
    length = length if length > 0.0 else eps
    acc = direct(pos, q, m, eps, G, nthreads=nthreads)[0]
    dts = []
    for _ in range(steps):
        dt = adaptive_dt(acc, eta, length, dt_min, dt_max)
        vel = vel + (0.5 * dt) * acc
        pos = pos + dt * vel
        acc = direct(pos, q, m, eps, G, nthreads=nthreads)[0]
        vel = vel + (0.5 * dt) * acc
        dts.append(dt)
    return pos, vel, acc, np.array(dts)


def block_level(acc, eta, length, dt_max, K):
    """Level k of each particle for block steps: the smallest k in 0..K with dt_max 2^-k <=
    eta sqrt(length / |a|), |a|^2 summed as x*x + y*y + z*z (the library's rule; the reference only
    lists a variable time step as a goal)."""
    acc = np.asarray(acc, dtype=np.float64).reshape(-1, 3)
    a2 = acc[:, 0] * acc[:, 0] + acc[:, 1] * acc[:, 1] + acc[:, 2] * acc[:, 2]
    k = np.zeros(len(a2), np.int64)
    pos = a2 > 0
    want = np.full(len(a2), np.inf)
    want[pos] = eta * np.sqrt(length / np.sqrt(a2[pos]))
    for _ in range(K):
        step = np.ldexp(dt_max, -k)
        k = np.where((k < K) & (step > want), k + 1, k)
    return k


def leapfrog_block(pos, vel, q, m, eps, G, eta, length, dt_max, K, steps, nthreads=None, stats=None):
    """FP64 direct-sum kick-drift-kick leapfrog with individual power-of-two steps (the library's
    NBODY_DT_BLOCK scheme): per base step dt_max, 2^K substeps of dt_max 2^-K; every particle drifts
    every substep; a particle's step of dt_max 2^-k starts with a half kick and ends with one, and
    its level comes from block_level at the start of each of its steps, no coarser than the substep
    grid allows there.  Returns (pos, vel, acc, levels of the last steps).  With a dict `stats`,
    stats["evaluations"] = substeps of the last base step at which some particle's step ended (the
    ones that need forces)."""
    x = np.array(pos, dtype=np.float64).reshape(-1, 3)
    v = np.array(vel, dtype=np.float64).reshape(-1, 3)
    length = length if length > 0.0 else eps
    a = direct(x, q, m, eps, G, nthreads=nthreads)[0]
    S = 1 << K
    lv = None
    for _ in range(steps):
        lv = block_level(a, eta, length, dt_max, K)
        v = v + np.ldexp(dt_max, -(lv + 1))[:, None] * a
        evaluations = 0
        for s in range(1, S + 1):
            x = x + np.ldexp(dt_max, -K) * v
            a = direct(x, q, m, eps, G, nthreads=nthreads)[0]
            end = (s & ((1 << (K - lv)) - 1)) == 0
            evaluations += bool(end.any())
            v = v + np.where(end, np.ldexp(dt_max, -(lv + 1)), 0.0)[:, None] * a
            if s < S:
                tz = (s & -s).bit_length() - 1
                new = np.maximum(block_level(a, eta, length, dt_max, K), K - tz)
                lv = np.where(end, new, lv)
                v = v + np.where(end, np.ldexp(dt_max, -(lv + 1)), 0.0)[:, None] * a
        if stats is not None:
            stats["evaluations"] = evaluations
    return x, v, a, lv


def direct_vjp(pos, q, m, mu, eps=0.01, G=1.0, nthreads=None):
    """FP64 direct-sum VJP of S = sum_i mu_i . a_i: (dS/dx, dS/dq, dS/dm)."""
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1)
    n = pos.shape[0] // 3
    gx, gq, gm = np.zeros(3 * n), np.zeros(n), np.zeros(n)
    lib().orc_direct_vjp(n, pos, np.ascontiguousarray(q, np.float64), np.ascontiguousarray(m, np.float64), eps, G,
                         np.ascontiguousarray(mu, np.float64).reshape(-1), gx, gq, gm,
                         nthreads or min(os.cpu_count() or 1, 32))
    return gx.reshape(-1, 3), gq, gm


def leapfrog_adjoint(pos, vel, q, m, eps, G, dt, steps, gxT, gvT, nthreads=None):
    """FP64 direct-sum leapfrog adjoint: (dL/dx0, dL/dv0, dL/dq, dL/dm)."""
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1)
    n = pos.shape[0] // 3
    gx0, gv0, gq, gm = np.zeros(3 * n), np.zeros(3 * n), np.zeros(n), np.zeros(n)
    lib().orc_leapfrog_adjoint(n, pos, np.ascontiguousarray(vel, np.float64).reshape(-1),
                               np.ascontiguousarray(q, np.float64), np.ascontiguousarray(m, np.float64), eps, G, dt,
                               steps, np.ascontiguousarray(gxT, np.float64).reshape(-1),
                               np.ascontiguousarray(gvT, np.float64).reshape(-1), gx0, gv0, gq, gm,
                               nthreads or min(os.cpu_count() or 1, 32))
    return gx0.reshape(-1, 3), gv0.reshape(-1, 3), gq, gm


def naive_steps(pos4, vel4, mass, charge, G, dt, steps, fix_delta=False):
    """Port of the reference CPU path (src/naive_simulation.cpp:7-46)."""
    p = np.ascontiguousarray(pos4, dtype=np.float32).copy()
    v = np.ascontiguousarray(vel4, dtype=np.float32).copy()
    t = lib().orc_naive_steps(p.shape[0], p.reshape(-1), v.reshape(-1), np.ascontiguousarray(mass, np.float32),
                              np.ascontiguousarray(charge, np.float32), G, dt, steps, int(fix_delta))
    return p, v, t


def ref_naive_steps(pos4, vel4, mass, charge, G, dt, steps):
    """The reference's own src/naive_simulation.cpp (only where it was built)."""
    R = ref_lib()
    if R is None:
        return None
    p = np.ascontiguousarray(pos4, dtype=np.float32).copy()
    v = np.ascontiguousarray(vel4, dtype=np.float32).copy()
    t = R.ref_naive_steps(p.shape[0], p.reshape(-1), v.reshape(-1), np.ascontiguousarray(mass, np.float32),
                          np.ascontiguousarray(charge, np.float32), G, dt, steps)
    return p, v, t


def ref_fmm_run(pos_sorted, vel_sorted, mass_sorted, charge_sorted, nodes, box, dt):
    """Run the reference's FMM kernels (src/*.cl) on the CPU over a given tree.

    Inputs are in sorted (leaf) order, float32.  Returns dict with leaf/node
    interaction pairs (breadth-first node ids), per-particle leaf and node
    forces and the explicit-Euler-stepped state, all in sorted order.
    """
    R = ref_lib()
    if R is None:
        return None
    n = pos_sorted.shape[0]
    cap = 8 * 1024 * 1024
    lp = np.zeros(2 * cap, np.int32)
    npairs = np.zeros(2 * cap, np.int32)
    nl, nn = C.c_int(0), C.c_int(0)
    fl = np.zeros(3 * n, np.float32)
    fn = np.zeros(3 * n, np.float32)
    po = np.zeros(3 * n, np.float32)
    vo = np.zeros(3 * n, np.float32)
    rc = R.ref_fmm_run(n, np.ascontiguousarray(pos_sorted, np.float32).reshape(-1),
                       np.ascontiguousarray(vel_sorted, np.float32).reshape(-1),
                       np.ascontiguousarray(mass_sorted, np.float32), np.ascontiguousarray(charge_sorted, np.float32),
                       nodes.shape[0], np.ascontiguousarray(nodes, np.int32).reshape(-1),
                       np.ascontiguousarray(box, np.float64), dt, cap, C.byref(nl), lp, C.byref(nn), npairs,
                       fl, fn, po, vo)
    if rc != 0:
        raise RuntimeError(f"ref_fmm_run failed rc={rc}")
    return {
        "leaf_pairs": lp[: 2 * nl.value].reshape(-1, 2).copy(),
        "node_pairs": npairs[: 2 * nn.value].reshape(-1, 2).copy(),
        "f_leaf": fl.reshape(-1, 3), "f_node": fn.reshape(-1, 3),
        "pos": po.reshape(-1, 3), "vel": vo.reshape(-1, 3),
    }


def both_orientations(pairs):
    """Unordered (a, b) pairs -> set of ordered (t, s) tuples in both directions."""
    s = set()
    for a, b in np.asarray(pairs).tolist():
        s.add((a, b))
        s.add((b, a))
    return s
