"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference is mounted and oracle/_ref was built
(``make -C oracle ref``).  Outputs:

ref_fmm_plummer1k.npz  Plummer N=1,024 shifted into [0,64)^3 (bounds 64),
                       leaf capacity 8, theta 0.5, eps 0.01 (the reference's
                       defaults), charge = mass; interaction sets, leaf/node
                       forces and one explicit-Euler step computed by the
                       reference kernels src/{moment,interaction,field,force}.cl.
ref_fmm_cube2k.npz     N=2,048 uniform in [0,1)^3 (bounds 1) with the
                       mass/charge ranges of src/main.cpp:23-27 (mass 1..10,
                       charge 0.1..1), same kernels.
ref_naive_256.npz      N=256, three steps of src/naive_simulation.cpp.

Inputs are seeded; positions are rounded to float32 (the reference's
vector_t) before anything is computed.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from nbody_gb300 import ics  # noqa: E402


def pair_array(pairs):
    a = np.array(sorted(O.both_orientations(pairs)), dtype=np.int32).reshape(-1, 2)
    return a


def fmm_case(name, pos, vel, mass, charge, bounds, cap=8, dt=1e-3):
    pos = pos.astype(np.float32).astype(np.float64)
    vel = vel.astype(np.float32).astype(np.float64)
    mass = mass.astype(np.float32).astype(np.float64)
    charge = charge.astype(np.float32).astype(np.float64)
    box = np.array([0.0, 0.0, 0.0, float(bounds)])
    t = O.Tree(pos, charge, mass, box=box, cap=cap)
    srt = t.perm
    r = O.ref_fmm_run(pos[srt], vel[srt], mass[srt], charge[srt], t.nodes, box, dt)
    inv = np.argsort(srt)
    out = dict(
        pos=pos, vel=vel, mass=mass, charge=charge, box=box, cap=np.int32(cap), theta=np.float64(0.5),
        eps=np.float64(0.01), dt=np.float64(dt),
        nodes=t.nodes, perm=srt.astype(np.int64), keys=t.keys,
        m2l=pair_array(r["node_pairs"]), p2p=pair_array(r["leaf_pairs"]),
        f_leaf=r["f_leaf"][inv], f_node=r["f_node"][inv],
        pos1=r["pos"][inv], vel1=r["vel"][inv],
    )
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name, "n", pos.shape[0], "nodes", t.nnodes, "m2l", len(out["m2l"]), "p2p", len(out["p2p"]))


def main():
    if O.ref_lib() is None:
        O.build(ref=True)
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref/libnbody_ref.so is not available (reference not mounted?)")

    p, v, m = ics.plummer(1024, seed=11)
    fmm_case("ref_fmm_plummer1k.npz", p + 32.0, v, m, m, 64.0)

    rng = np.random.Generator(np.random.PCG64(12))
    n = 2048
    pos = rng.uniform(0.0, 1.0, (n, 3))
    theta = 2 * np.pi * rng.uniform(0, 1, n)
    phi = np.arccos(2.0 * (rng.uniform(0, 1, n) - 0.5))
    vel = 0.1 * np.stack([np.sin(phi) * np.cos(theta), np.sin(phi) * np.sin(theta), np.cos(phi)], axis=1)
    mass = 1.0 + 9.0 * rng.uniform(0, 1, n)
    charge = 0.1 + 0.9 * rng.uniform(0, 1, n)
    fmm_case("ref_fmm_cube2k.npz", pos, vel, mass, charge, 1.0)

    rng = np.random.Generator(np.random.PCG64(13))
    n = 256
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = rng.uniform(0.0, 1.0, (n, 3))
    vel4 = np.zeros((n, 4), np.float32)
    vel4[:, :3] = rng.normal(0.0, 0.1, (n, 3))
    mass = rng.uniform(1.0, 10.0, n).astype(np.float32)
    charge = rng.uniform(0.1, 1.0, n).astype(np.float32)
    p1, v1, t1 = O.ref_naive_steps(pos4, vel4, mass, charge, 1.0, 1e-3, 3)
    np.savez_compressed(os.path.join(HERE, "ref_naive_256.npz"), pos4=pos4, vel4=vel4, mass=mass, charge=charge,
                        G=np.float32(1.0), dt=np.float32(1e-3), steps=np.int32(3), pos_out=p1, vel_out=v1,
                        t_out=np.float32(t1))
    print("ref_naive_256.npz t", t1)


if __name__ == "__main__":
    main()
