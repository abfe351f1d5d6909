"""Golden fixtures on the GPU: the plain FP64 drop-in tier, driven through the C ABI over
the protocol of tests/golden/make_golden.py, matches the vectors the FP64 oracle stored.
Tolerances are those of the oracle-side parity tests:
* neighbour counts and index sums, particle counts: exact;
* boundary flags: exact except particles within 1e-6 relative of the PND or NPCD threshold;
* ``pndSmall`` after initialisation: normwise relative error <= 1e-10;
* after three free-running steps: positions <= 1e-10, velocities and pressure <= 1e-6
  (PPE to 1e-12 on both sides; the residual left by the solver feeds the velocities).
"""
import numpy as np
import pytest

from test_cpu_golden import G, INT_KEYS, NAMES, load, relerr

pytestmark = pytest.mark.gpu


def _bc_mismatch(got, ref, pnd, npcd2, p):
    bad = np.nonzero(got != ref)[0]
    amb = (np.abs(pnd[bad] - p.betaPnd) <= 1e-6 * p.betaPnd) | \
          (np.abs(npcd2[bad] - p.delta2) <= 1e-6 * p.delta2)
    return bad[~amb]


@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(mps_lib, name):
    from polymps_gb300 import mps
    ref = load(name)
    c = G.CASES[name]()
    with mps.MpsGpu(c, tol=G.TOL) as g:
        got = G.record(g, c, steps=int(ref["steps"]))
        p = g.params
    assert int(got["n"]) == int(ref["n"])
    for k in INT_KEYS:
        assert np.array_equal(got[k], ref[k]), k
    bad = _bc_mismatch(got["init_bc"], ref["init_bc"], ref["init_pndsmall"], ref["init_npcd2"], p)
    assert len(bad) == 0, "init_bc differs at %s" % bad[:10]
    assert relerr(got["init_pndsmall"], ref["init_pndsmall"]) <= 1e-10
    assert relerr(got["pos"], ref["pos"]) <= 1e-10
    assert relerr(got["vel"], ref["vel"]) <= 1e-6
    assert relerr(got["press"], ref["press"]) <= 1e-6
    assert np.all(got["ppe_res"] <= G.TOL)
