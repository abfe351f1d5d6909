"""Dynamic particle collision (collision type 1: MpsParticleCollision::
checkDynamicParticleCollisions, src/MpsParticleCollision.cpp:120-292) against the oracle."""
import numpy as np
import pytest

from polymps_gb300 import abi, cases

from test_gpu_parity import relerr, step_ops, sync

pytestmark = pytest.mark.gpu


def _case(base):
    c = cases.config(3, jitter=0.02, scale=5.0) if base == 3 else cases.config(1, jitter=0.02)
    c.params.update(collisionType=1, lambdaCollision=0.2)
    return c


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
@pytest.mark.parametrize("base", [3, 1])
def test_dpc_teacher_forced(oracle_mod, mps_lib, base, precision):
    from polymps_gb300 import mps
    c = _case(base)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12, precision=precision)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(3):
        o.step()
    # a velocity kick so that both branches (approaching and separating pairs) act
    v = o.get(abi.F_VEL)
    o.set(abi.F_VEL, v + 0.05 * np.random.default_rng(4).standard_normal(v.shape))
    ops = step_ops(o.params)
    sync(o, g)
    o.run_op("UPDATE_BUCKETS")
    g.run_op("UPDATE_BUCKETS")
    for op in ops[1: ops.index("COLLISION")]:
        o.run_op(op)
    sync(o, g)
    x0 = o.get(abi.F_POS)
    o.run_op("COLLISION")
    g.run_op("COLLISION")
    assert np.abs(o.get(abi.F_POS) - x0).max() > 0   # DPC moves positions
    for f in (abi.F_VEL, abi.F_POS):
        assert relerr(g.get(f), o.get(f)) <= 1e-12, abi.FIELD_NAMES[f]
    # the lists after the collision follow the moved positions
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert np.array_equal(co, cg) and np.array_equal(no, ng)
    g.close()


@pytest.mark.parametrize("base", [3, 1])
def test_dpc_free_running(oracle_mod, mps_lib, base):
    from polymps_gb300 import mps
    c = _case(base)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12)
    o.set_solver(1e-12)
    o.initialize()
    g.initialize()
    for _ in range(6):
        so = o.step()
        sg = g.step()
        assert sg.numParticles == so.numParticles
    assert relerr(g.get(abi.F_POS), o.get(abi.F_POS)) < 1e-10
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-6
    g.close()
