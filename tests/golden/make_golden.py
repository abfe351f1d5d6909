"""Writes the golden fixtures of tests/golden/ from the FP64 CPU oracle.

TEST INFRASTRUCTURE ONLY.  The reference ships no tests and no golden vectors, and
its build needs submodules (Eigen, nlohmann/json, libigl) that are not vendored, so
the fixtures are the oracle's output on small, seeded versions of the benchmark
workloads.  They freeze the oracle (a change to it shows up as a CPU test failure)
and let the GPU tests check the CUDA path against stored vectors without running the
oracle.  Each fixture holds, for one case:

* ``pos0_sha256``: hash of the generated initial positions (detects a case-generator change);
* after initialisation (``MpsParticleSystem`` set-up, src/main.cpp:158-166): per-particle
  neighbour count, sum of neighbour indices, ``pndSmall``, ``npcd²`` and the boundary flag;
* after ``STEPS`` whole steps (src/main.cpp:221-469) with the PPE solved to 1e-12:
  particle count, positions, velocities, pressure, neighbour counts, boundary flags and
  the per-step PPE iterations and relative residual.

Usage: ``python tests/golden/make_golden.py`` (one oracle thread, a few seconds).
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from polymps_gb300 import abi, cases  # noqa: E402

STEPS = 3
TOL = 1e-12

# small versions of the four workloads: 2D particle walls, 3D weakly compressible and
# incompressible polygon tanks, tank with obstacle, collision and shifting
CASES = {
    "cfg1_2d_particle_walls": lambda: cases.config(1, jitter=0.02),
    "cfg2_3d_wc_polygon": lambda: cases.config(2, jitter=0.02, scale=3.0),
    "cfg3_3d_inc_polygon": lambda: cases.config(3, jitter=0.02, scale=5.0),
    "cfg5_3d_obstacle_shifting": lambda: cases.config(5, jitter=0.02, scale=10.0),
}


def pos_hash(pos):
    return hashlib.sha256(np.ascontiguousarray(pos, dtype=np.float64).tobytes()).hexdigest()


def neighbor_sums(counts, nbr):
    """Per-particle sum of neighbour indices (int64): with the count, a compact
    fingerprint of the neighbour set."""
    start = np.concatenate(([0], np.cumsum(counts, dtype=np.int64)))
    csum = np.concatenate(([0], np.cumsum(nbr.astype(np.int64))))
    return csum[start[1:]] - csum[start[:-1]]


def record(sim, c, steps=STEPS):
    """Runs ``sim`` (the oracle, or any object with the same methods) over the golden
    protocol and returns the fixture arrays."""
    out = {"pos0_sha256": np.array(pos_hash(c.pos)), "steps": np.array(steps)}
    sim.initialize()
    counts, nbr = sim.neighbors()
    out["init_numneigh"] = counts.astype(np.int32)
    out["init_nbrsum"] = neighbor_sums(counts, nbr)
    out["init_pndsmall"] = sim.get(abi.F_PNDSMALL)
    out["init_npcd2"] = sim.get(abi.F_NPCD2)
    out["init_bc"] = sim.get(abi.F_BC).astype(np.int32)
    its, res = [], []
    for _ in range(steps):
        st = sim.step()
        its.append(st.ppeIterations)
        res.append(st.ppeRelResidual)
    out["n"] = np.array(sim.n)
    out["ppe_iters"] = np.array(its, dtype=np.int32)
    out["ppe_res"] = np.array(res)
    out["pos"] = sim.get(abi.F_POS)
    out["vel"] = sim.get(abi.F_VEL)
    out["press"] = sim.get(abi.F_PRESS)
    out["numneigh"] = sim.get(abi.F_NUMNEIGH).astype(np.int32)
    out["bc"] = sim.get(abi.F_BC).astype(np.int32)
    return out


def oracle_record(oracle_mod, name):
    c = CASES[name]()
    o = oracle_mod.Oracle(c, threads=1)
    try:
        o.set_solver(TOL)
        return record(o, c)
    finally:
        o.close()


def path(name):
    return os.path.join(HERE, name + ".npz")


def main():
    import oracle as O
    O.build()
    for name in CASES:
        d = oracle_record(O, name)
        np.savez_compressed(path(name), **d)
        print("%-28s n=%6d  iters=%s  %7.1f KB" % (name, int(d["n"]), d["ppe_iters"].tolist(),
                                                   os.path.getsize(path(name)) / 1024))


if __name__ == "__main__":
    main()
