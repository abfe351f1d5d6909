"""DF32 tier (float-float neighbour arithmetic) against the FP64 CPU oracle.

Stated tolerances of the tier:
* neighbour sets, entry masks, integer fields: bit-exact (every radius / mirror-side /
  collision decision near its threshold is taken in FP64, as the reference takes it);
* free-surface flags: equal except particles within 1e-6 relative of a threshold;
* FP64 fields after one operator from an identical state (teacher forcing):
  normwise relative error <= 1e-8 (float-float pair arithmetic is ~1e-11 relative;
  pressure-dependent fields amplify it through the solver);
* pressure of the PPE (solved to 1e-12): within 1e-6 relative of the oracle's.
"""
import numpy as np
import pytest

from polymps_gb300 import abi, cases

from test_gpu_parity import CASES, INT, SCA, VEC, relerr, step_ops, sync

pytestmark = pytest.mark.gpu

DF_RTOL = 1e-8


def _pair(oracle_mod, mps, case, tol=1e-12):
    o = oracle_mod.Oracle(case)
    g = mps.MpsGpu(case, tol=tol, precision=abi.PRECISION_DF32)
    o.set_solver(tol)
    return o, g


def compare(o, g, where, fields=None, rtol=DF_RTOL):
    fields = fields or (VEC + SCA + INT)
    p = o.params
    for f in fields:
        a, b = g.get(f), o.get(f)
        name = abi.FIELD_NAMES[f]
        if f in abi.INT_FIELDS:
            bad = np.nonzero(a != b)[0]
            if f == abi.F_BC and len(bad):
                ps = o.get(abi.F_PNDSMALL)[bad]
                d2 = o.get(abi.F_NPCD2)[bad]
                amb = (np.abs(ps - p.betaPnd) <= 1e-6 * p.betaPnd) | (np.abs(d2 - p.delta2) <= 1e-6 * p.delta2)
                bad = bad[~amb]
            assert len(bad) == 0, "%s: %s differs at %s (gpu %s, oracle %s)" % (where, name, bad[:10], a[bad[:5]], b[bad[:5]])
        else:
            e = relerr(a, b)
            assert e <= rtol, "%s: %s rel err %.3e" % (where, name, e)


@pytest.mark.parametrize("name", list(CASES))
def test_df32_neighbor_sets_bit_exact(oracle_mod, mps_lib, name):
    from polymps_gb300 import mps
    o, g = _pair(oracle_mod, mps, CASES[name]())
    o.initialize()
    for _ in range(3):
        o.step()
    sync(o, g)
    for ob in (o, g):
        ob.run_op("UPDATE_BUCKETS")
        ob.run_op("VISCOSITY"); ob.run_op("ADD_GRAVITY"); ob.run_op("PREDICT")
    g.set(abi.F_POS, o.get(abi.F_POS))
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert np.array_equal(co, cg)
    assert np.array_equal(no, ng)


@pytest.mark.parametrize("kick", [0.0, 40.0])
@pytest.mark.parametrize("name", list(CASES))
def test_df32_skin_list_bit_exact(oracle_mod, mps_lib, name, kick):
    """The list of the predicted positions filtered from the start-of-step skin list (no
    kick) or, when particles move beyond half the skin (random velocities of 40 m/s), rebuilt
    by the fallback scan, equals the oracle's scan of the same positions through the same
    stale buckets."""
    from polymps_gb300 import mps
    o, g = _pair(oracle_mod, mps, CASES[name]())
    o.initialize()
    for _ in range(3):
        o.step()
    v = o.get(abi.F_VEL)
    o.set(abi.F_VEL, v + kick * np.random.default_rng(2).standard_normal(v.shape))
    sync(o, g)
    for ob in (o, g):
        for op in ("UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY", "PREDICT"):
            ob.run_op(op)
    compare(o, g, "after prediction", fields=[abi.F_ACC, abi.F_POS], rtol=1e-8)
    o.set(abi.F_POS, g.get(abi.F_POS))   # no field set on the GPU side since the skin list
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert np.array_equal(co, cg)
    assert np.array_equal(no, ng)


def test_df32_fused_correction_matrix(oracle_mod, mps_lib):
    """The correction matrix formed inside the PND sweep equals the separate kernel's, bit for
    bit (same entries, same order, same float-float arithmetic)."""
    from polymps_gb300 import mps
    c = CASES["cfg3_3d_inc_polygon"]()
    g = mps.MpsGpu(c, tol=1e-10, precision=abi.PRECISION_DF32)
    g.initialize()
    g.run(3)
    ops = step_ops(g.params)
    for op in ops[: ops.index("CORRECTION_MATRIX") + 1]:
        g.run_op(op)   # no field set since the PND sweep: the fused matrix is kept
    fused = [g.get(f) for f in (abi.F_CORR1, abi.F_CORR2, abi.F_CORR3)]
    g.set(abi.F_PRESS, g.get(abi.F_PRESS))   # any field set: the operator recomputes
    g.run_op("CORRECTION_MATRIX")
    sep = [g.get(f) for f in (abi.F_CORR1, abi.F_CORR2, abi.F_CORR3)]
    for a, b in zip(fused, sep):
        assert np.array_equal(a, b)
    assert np.abs(fused[0]).max() > 0
    g.close()


def test_df32_neighbor_sets_adversarial(oracle_mod, mps_lib):
    """Pairs at r^2 = reL^2 and within a few ulps of it: decided by the FP64 fallback."""
    from polymps_gb300 import mps
    c = cases.config(3, scale=5.0)
    p = oracle_mod.Oracle(c).params
    rng = np.random.default_rng(11)
    pos = c.pos.copy()
    n = len(pos)
    for k in range(0, n - 1, 5):
        d = rng.normal(size=3); d /= np.linalg.norm(d)
        r = p.reL * [1.0, 1.0 + 2e-16, 1.0 - 2e-16, 1.0 + 1e-13, 1.0 - 1e-13][k % 5]
        pos[k + 1] = pos[k] + r * d
    c2 = cases.Case(c.name, c.params, c.type, pos, c.mesh)
    o, g = _pair(oracle_mod, mps, c2)
    for ob in (o, g):
        ob.run_op("UPDATE_BUCKETS")
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert np.array_equal(co, cg)
    assert np.array_equal(no, ng)


@pytest.mark.parametrize("name", list(CASES))
def test_df32_operator_parity_teacher_forced(oracle_mod, mps_lib, name):
    from polymps_gb300 import mps
    o, g = _pair(oracle_mod, mps, CASES[name]())
    o.initialize()
    g.initialize()
    for _ in range(4):
        o.step()
    o.set_velmax(0.0)
    for s in range(3):
        sync(o, g)
        for op in step_ops(o.params):
            o.run_op(op)
            g.run_op(op)
            compare(o, g, "step %d op %s" % (s, op))
            sync(o, g)


@pytest.mark.parametrize("name", ["cfg3_3d_inc_polygon", "cfg1_2d_particle_walls"])
def test_df32_ppe_pressure(oracle_mod, mps_lib, name):
    """The pressure the DF32 tier's PPE yields stays within 1e-6 of the FP64 oracle."""
    from polymps_gb300 import mps
    o, g = _pair(oracle_mod, mps, CASES[name]())
    o.initialize()
    for _ in range(5):
        o.step()
    sync(o, g)
    for op in step_ops(o.params)[: step_ops(o.params).index("CALC_PRESS")]:
        o.run_op(op); g.run_op(op); sync(o, g)
    o.run_op("CALC_PRESS")
    g.run_op("CALC_PRESS")
    ro, co, vo, bo = o.ppe()
    rg, cg, vg, bg = g.ppe()
    assert np.array_equal(ro, rg) and np.array_equal(co, cg)
    assert relerr(vg, vo) < 1e-10
    assert relerr(bg, bo) < 1e-7
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-6


@pytest.mark.parametrize("name", list(CASES))
def test_df32_free_running_steps(oracle_mod, mps_lib, name):
    from polymps_gb300 import mps
    o, g = _pair(oracle_mod, mps, CASES[name]())
    o.initialize()
    g.initialize()
    for _ in range(10):
        so = o.step()
        sg = g.step()
        assert sg.numParticles == so.numParticles
    assert relerr(g.get(abi.F_POS), o.get(abi.F_POS)) < 1e-9
    assert relerr(g.get(abi.F_VEL), o.get(abi.F_VEL)) < 1e-5
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-5


@pytest.mark.parametrize("solver", [abi.SOLVER_PLAIN_FP64, abi.SOLVER_MIXED])
def test_extrapolated_warm_start(oracle_mod, mps_lib, solver):
    """Warm start 2 p_n - p_{n-1}: the same system solved from it reaches the tolerance in
    fewer iterations than from p_n, and the two solutions agree to the tolerance."""
    from polymps_gb300 import mps
    c = CASES["cfg3_3d_inc_polygon"]()
    g = mps.MpsGpu(c, solver=solver, tol=1e-10, precision=abi.PRECISION_DF32)
    g.initialize()
    g.run(8)
    for op in step_ops(g.params)[: step_ops(g.params).index("CALC_PRESS")]:
        g.run_op(op)
    pn, pp = g.get(abi.F_PRESSPPE), g.get(abi.F_PRESSPPE_PREV)
    out = {}
    for warm in (abi.WARM_PREVIOUS, abi.WARM_EXTRAP):
        g.set(abi.F_PRESSPPE, pn)
        g.set(abi.F_PRESSPPE_PREV, pp)
        g.set_solver(solver, warm, 1e-10, 20000)
        g.run_op("CALC_PRESS")
        st = g.last_stats()
        assert st.ppeRelResidual <= 1e-10
        out[warm] = (g.get(abi.F_PRESSPPE), st.ppeIterations, st.ppeInitialRelResidual)
    assert out[abi.WARM_EXTRAP][2] < out[abi.WARM_PREVIOUS][2]
    assert out[abi.WARM_EXTRAP][1] <= out[abi.WARM_PREVIOUS][1]
    assert relerr(out[abi.WARM_EXTRAP][0], out[abi.WARM_PREVIOUS][0]) < 1e-7
    g.close()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
@pytest.mark.parametrize("inner", [abi.SOLVER_MIXED_MATFREE, abi.SOLVER_MIXED_COMPACT])
def test_mixed_inner_operators(oracle_mod, mps_lib, precision, inner):
    """The mixed solver with the matrix-free FP32 or the compact FP16-stored inner operator
    reaches the FP64 residual of the assembled system and agrees with the plain FP64 CG
    within 1e-6."""
    from polymps_gb300 import mps
    c = CASES["cfg3_3d_inc_polygon"]()
    out = {}
    for solver in (abi.SOLVER_PLAIN_FP64, inner):
        g = mps.MpsGpu(c, solver=solver, tol=1e-10, precision=precision)
        g.initialize()
        st = g.run(4)
        assert st.ppeRelResidual <= 1e-10
        out[solver] = g.get(abi.F_PRESS)
        g.close()
    assert relerr(out[inner], out[abi.SOLVER_PLAIN_FP64]) < 1e-6


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
@pytest.mark.parametrize("stype", [1, 2])
def test_shifting_parity(oracle_mod, mps_lib, stype, precision):
    """Particle shifting (type 1: velocity correction; type 2: concentration gradient with
    the polygon-wall term) from an identical post-corrector state, tank with obstacle."""
    from polymps_gb300 import mps
    c = cases.config(5, jitter=0.02, scale=6.0)
    c.params.update(shiftingType=stype)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12, precision=precision)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(4):
        o.step()
    ops = step_ops(o.params)
    # both sides scan the bucket list of the start-of-step positions
    sync(o, g)
    o.run_op("UPDATE_BUCKETS")
    g.run_op("UPDATE_BUCKETS")
    for op in ops[1: ops.index("SHIFTING")]:
        o.run_op(op)
    assert o.n == g.n
    sync(o, g)
    f = abi.F_POS if stype == 2 else abi.F_VEL
    before = o.get(f)
    o.run_op("SHIFTING")
    g.run_op("SHIFTING")
    assert np.abs(o.get(f) - before).max() > 0.0   # the sweep moved something
    compare(o, g, "shifting %d" % stype, rtol=DF_RTOL if precision == abi.PRECISION_DF32 else 1e-10)
    g.close()
    o.close()


@pytest.mark.parametrize("stype", [1, 2])
def test_shifting_list_parity(oracle_mod, mps_lib, stype):
    """DF32 shifting over the list of the post-corrector positions filtered from the
    start-of-step skin list (the path of a full step) equals the oracle's scan from the
    same post-corrector state, tank with obstacle."""
    from polymps_gb300 import mps
    c = cases.config(5, jitter=0.02, scale=6.0)
    c.params.update(shiftingType=stype)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12, precision=abi.PRECISION_DF32)
    o.set_solver(1e-12)
    o.initialize()
    g.initialize()
    for _ in range(4):
        o.step()
    ops = step_ops(o.params)
    sync(o, g)
    k = ops.index("SHIFTING")
    for op in ops[:k]:   # the GPU builds its skin list in VISCOSITY, as in a step
        o.run_op(op)
        g.run_op(op)
    assert o.n == g.n
    sync(o, g)   # identical post-corrector state (moves within the skin keep the list usable)
    f = abi.F_POS if stype == 2 else abi.F_VEL
    before = o.get(f)
    o.run_op("SHIFTING")
    l0 = mps.MpsGpu.launch_count()
    g.run_op("SHIFTING")
    # filter path: positions (2), skin check, filter (2), masks, then the sweeps
    assert mps.MpsGpu.launch_count() - l0 == 6 + (3 if stype == 1 else 7)
    assert np.abs(o.get(f) - before).max() > 0.0
    compare(o, g, "shifting list %d" % stype, rtol=DF_RTOL)
    g.close()
    o.close()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
def test_dense_rows_over_64_entries(oracle_mod, mps_lib, precision):
    """Fluid compressed to 0.75 of its spacing (about 75 neighbours per particle, the second
    word of the entry masks in use): bit-exact neighbour sets and one teacher-forced step
    of every operator against the oracle."""
    from polymps_gb300 import mps
    from test_gpu_parity import FP64_RTOL
    c = cases.config(3, jitter=0.02, scale=5.0)
    o0 = oracle_mod.Oracle(c)
    fluid = c.type == o0.params.fluid
    o0.close()
    pos = c.pos.copy()
    ctr = pos[fluid].mean(axis=0)
    pos[fluid] = ctr + 0.75 * (pos[fluid] - ctr)
    c2 = cases.Case(c.name, c.params, c.type, pos, c.mesh)
    o = oracle_mod.Oracle(c2)
    g = mps.MpsGpu(c2, tol=1e-12, precision=precision)
    o.set_solver(1e-12)
    for ob in (o, g):
        ob.run_op("UPDATE_BUCKETS")
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert co.max() > 64
    assert np.array_equal(co, cg)
    assert np.array_equal(no, ng)
    o.initialize()
    g.initialize()
    o.set_velmax(0.0)
    sync(o, g)
    rtol = FP64_RTOL if precision == abi.PRECISION_FP64 else DF_RTOL
    for op in step_ops(o.params):
        o.run_op(op)
        g.run_op(op)
        compare(o, g, "dense op %s" % op, rtol=rtol)
        sync(o, g)
    g.close()
    o.close()
