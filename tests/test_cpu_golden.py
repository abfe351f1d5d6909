"""Golden fixtures on the CPU (tests/golden/*.npz, written by tests/golden/make_golden.py
from the FP64 oracle on seeded small versions of the four workloads): the case generator
and the oracle still reproduce the stored vectors, and every stored incompressible step
reached the 1e-12 PPE residual it was solved to.  The GPU side is test_gpu_zgolden.py."""
import hashlib
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def golden_module():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


G = golden_module()

NAMES = list(G.CASES)
INT_KEYS = ("init_numneigh", "init_nbrsum", "numneigh")


def load(name):
    with np.load(G.path(name)) as f:
        return {k: f[k] for k in f.files}


def relerr(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("name", NAMES)
def test_case_generator_unchanged(name):
    c = G.CASES[name]()
    assert hashlib.sha256(np.ascontiguousarray(c.pos, dtype=np.float64).tobytes()).hexdigest() \
        == str(load(name)["pos0_sha256"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(oracle_mod, name):
    ref = load(name)
    got = G.oracle_record(oracle_mod, name)
    assert int(got["n"]) == int(ref["n"])
    for k in INT_KEYS + ("init_bc", "bc", "ppe_iters"):
        assert np.array_equal(got[k], ref[k]), k
    for k in ("init_pndsmall", "init_npcd2", "pos", "vel", "press"):
        assert relerr(got[k], ref[k]) <= 1e-13, k


@pytest.mark.parametrize("name", NAMES)
def test_golden_solver_converged(name):
    ref = load(name)
    if name.startswith("cfg2"):          # weakly compressible: no PPE
        assert np.all(ref["ppe_iters"] == 0)
    else:
        assert np.all(ref["ppe_iters"] > 0)
        assert np.all(ref["ppe_res"] <= G.TOL)

