"""ARC free-surface detection (free-surface type 2: MpsShifting::calcNormalParticles and
calcWallNormalParticles, src/MpsShifting.cpp:106-166, :319-420; MpsBoundaryCondition::
updateParticleBC, src/MpsBoundaryCondition.cpp:205-395) against the oracle."""
import numpy as np
import pytest

from polymps_gb300 import abi, cases

from test_gpu_parity import relerr, step_ops, sync

pytestmark = pytest.mark.gpu


def _case(base):
    c = cases.config(3, jitter=0.02, scale=5.0) if base == 3 else cases.config(1, jitter=0.02)
    c.params.update(freeSurfType=2)
    return c


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
@pytest.mark.parametrize("base", [3, 1])
def test_arc_teacher_forced(oracle_mod, mps_lib, base, precision):
    from polymps_gb300 import mps
    c = _case(base)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12, precision=precision)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(4):
        o.step()
    ops = step_ops(o.params)
    sync(o, g)
    o.run_op("UPDATE_BUCKETS")
    g.run_op("UPDATE_BUCKETS")
    for op in ops[1: ops.index("UPDATE_BC")]:
        o.run_op(op)
    sync(o, g)
    o.run_op("UPDATE_BC")
    g.run_op("UPDATE_BC")
    assert relerr(g.get(abi.F_NORMAL), o.get(abi.F_NORMAL)) <= 1e-10
    bo, bg = o.get(abi.F_BC), g.get(abi.F_BC)
    assert np.array_equal(bg, bo), np.nonzero(bg != bo)[0][:10]
    p = o.params
    assert np.sum(bo == p.surface) > 0 and np.sum(bo == p.inner) > 0
    g.close()


@pytest.mark.parametrize("base", [3, 1])
def test_arc_free_running(oracle_mod, mps_lib, base):
    from polymps_gb300 import mps
    c = _case(base)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12)
    o.set_solver(1e-12)
    o.initialize()
    g.initialize()
    assert np.array_equal(g.get(abi.F_BC), o.get(abi.F_BC))
    for _ in range(6):
        so = o.step()
        sg = g.step()
        assert sg.numParticles == so.numParticles
    assert relerr(g.get(abi.F_POS), o.get(abi.F_POS)) < 1e-10
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-6
    g.close()
