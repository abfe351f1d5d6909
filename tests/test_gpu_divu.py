"""The PND + div u pressure source (mps_type 3: MpsPressure::calcVelDivergence and the wall
divergences, src/MpsPressure.cpp:479-790, solvePressurePoissonPndDivU :289-421) and the
BiCGSTAB solver (solver_type 1, :448-468) against the oracle."""
import numpy as np
import pytest

from polymps_gb300 import abi, cases

from test_gpu_parity import relerr, step_ops, sync

pytestmark = pytest.mark.gpu

VARIANTS = {
    "divu_cg_noslip": dict(mpsType=3, solverType=0),
    "divu_cg_slip": dict(mpsType=3, solverType=0, slipCondition=1),
    "divu_bicgstab": dict(mpsType=3, solverType=1),
    "pnd_bicgstab": dict(mpsType=2, solverType=1),
}


def _case(name, base):
    c = cases.config(3, jitter=0.02, scale=5.0) if base == 3 else cases.config(1, jitter=0.02)
    c.params.update(VARIANTS[name])
    return c


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
@pytest.mark.parametrize("base", [3, 1])
@pytest.mark.parametrize("name", list(VARIANTS))
def test_pressure_variants_teacher_forced(oracle_mod, mps_lib, name, base, precision):
    from polymps_gb300 import mps
    c = _case(name, base)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12, precision=precision)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(3):
        o.step()
    ops = step_ops(o.params)
    sync(o, g)
    o.run_op("UPDATE_BUCKETS")
    g.run_op("UPDATE_BUCKETS")
    for op in ops[1: ops.index("CALC_PRESS")]:
        o.run_op(op)
    sync(o, g)
    o.run_op("CALC_PRESS")
    g.run_op("CALC_PRESS")
    st = g.last_stats()
    assert st.ppeRelResidual <= 1e-12
    tol = 1e-10 if precision == abi.PRECISION_FP64 else 1e-8
    if c.params["mpsType"] == 3:
        dv = o.get(abi.F_VELDIV)
        assert np.abs(dv).max() > 0
        assert relerr(g.get(abi.F_VELDIV), dv) <= tol
    ro, co, vo, bo = o.ppe()
    rg, cg, vg, bg = g.ppe()
    assert np.array_equal(ro, rg) and np.array_equal(co, cg)
    assert relerr(bg, bo) <= 1e-7
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-6
    g.close()


@pytest.mark.parametrize("name", list(VARIANTS))
def test_pressure_variants_free_running(oracle_mod, mps_lib, name):
    from polymps_gb300 import mps
    c = _case(name, 3)
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
