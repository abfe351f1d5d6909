"""GPU parity tests: the CUDA path (through the C ABI) against the FP64 CPU oracle.

* neighbour sets: bit-exact (membership decided in exact FP64 on both sides);
* integer fields (numNeigh, nNeighWall, nearWall, bucket-derived): exact;
* FP64 fields after one operator from an identical state (teacher forcing):
  normwise relative error <= 1e-10 (summation order / FMA differ, nothing else);
* free-surface flags: equal except particles within 1e-6 relative of a threshold;
* PPE: same sparsity pattern and values to 1e-12, pressure to the solver tolerances.
"""
import numpy as np
import pytest

from polymps_gb300 import abi, cases

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
VEC = sorted(abi.VECTOR_FIELDS)
SCA = sorted(abi.SCALAR_FIELDS)
INT = sorted(abi.INT_FIELDS)

# small versions of the benchmark workloads (same parameters, coarser lattices)
CASES = {
    "cfg1_2d_particle_walls": lambda: cases.config(1, jitter=0.02),
    "cfg2_3d_wc_polygon": lambda: cases.config(2, jitter=0.02, scale=3.0),
    "cfg3_3d_inc_polygon": lambda: cases.config(3, jitter=0.02, scale=5.0),
    "cfg5_3d_obstacle_shifting": lambda: cases.config(5, jitter=0.02, scale=6.0),
    # relax_fact < 1: the prediction-step pressure gradient (src/main.cpp:271-276), with the
    # polygon wall and gradient type 2 (p_min sweep), and with particle walls
    "cfg3_relax_0.7_grad2": lambda: _relaxed(cases.config(3, jitter=0.02, scale=5.0), 0.7, gradientType=2),
    "cfg1_relax_0.8": lambda: _relaxed(cases.config(1, jitter=0.02), 0.8),
}


def _relaxed(c, relax, **kw):
    c.params.update(relaxPress=relax, **kw)
    c.name += "_relax%g" % relax
    return c


def _pair(oracle_mod, mps, case, tol=1e-12):
    o = oracle_mod.Oracle(case)
    g = mps.MpsGpu(case, tol=tol)
    o.set_solver(tol)
    return o, g


def sync(o, g):
    for f in VEC + SCA + INT:
        g.set(f, o.get(f))


def relerr(a, b):
    na = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (na if na > 0 else 1.0)


def compare(o, g, where, fields=None, ambiguous_ok=0):
    fields = fields or (VEC + SCA + INT)
    p = o.params
    for f in fields:
        a, b = g.get(f), o.get(f)
        name = abi.FIELD_NAMES[f]
        if f in abi.INT_FIELDS:
            bad = np.nonzero(a != b)[0]
            if f == abi.F_BC and len(bad):
                # flags decided by a FP threshold: tolerate particles within 1e-6 relative
                ps = o.get(abi.F_PNDSMALL)[bad]
                d2 = o.get(abi.F_NPCD2)[bad]
                amb = (np.abs(ps - p.betaPnd) <= 1e-6 * p.betaPnd) | (np.abs(d2 - p.delta2) <= 1e-6 * p.delta2)
                bad = bad[~amb]
            assert len(bad) == 0, "%s: %s differs at %s (gpu %s, oracle %s)" % (where, name, bad[:10], a[bad[:5]], b[bad[:5]])
        else:
            e = relerr(a, b)
            assert e <= FP64_RTOL, "%s: %s rel err %.3e" % (where, name, e)


def step_ops(p):
    ops = ["UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY"]
    if p.relaxPress < 1.0:
        ops += ["PREDICT_PRESS_GRADIENT"]
    ops += ["PREDICT", "OUT_OF_DOMAIN", "COLLISION"]
    if p.wallType == 1:
        ops += ["WALL_DISTANCE", "WALL_NPCD"]
    if p.gradientCorrection and (p.pndType == 2 or p.mpsType == 3):
        ops += ["CORRECTION_MATRIX"]
    ops += ["PND_NEIGH_NPCD"]
    if p.pndType == 2:
        ops += ["PND_DIFFUSIVE"]
    elif p.pndType == 1:
        ops += ["PND_MEAN"]
    ops += ["UPDATE_BC", "CALC_PRESS"]
    if p.wallType == 0:
        ops += ["EXTRAPOLATE_PRESS"]
    if p.gradientCorrection:
        ops += ["CORRECTION_MATRIX"]
    ops += ["PRESS_GRADIENT"]
    if p.wallType == 1:
        ops += ["WALL_PRESS_GRADIENT", "WALL_VISCOSITY"]
    ops += ["CORRECT", "OUT_OF_DOMAIN"]
    if p.shiftingType:
        ops += ["SHIFTING"]
    if p.wallType == 0:
        ops += ["DUMMY_VELOCITY"]
    ops += ["OUT_OF_DOMAIN"]
    return ops


@pytest.mark.parametrize("name", list(CASES))
def test_initialize_parity(oracle_mod, mps_lib, name):
    from polymps_gb300 import mps
    c = CASES[name]()
    o, g = _pair(oracle_mod, mps, c)
    o.initialize()
    g.initialize()
    compare(o, g, "initialize")


@pytest.mark.parametrize("name", list(CASES))
def test_neighbor_sets_bit_exact(oracle_mod, mps_lib, name):
    """The list every sweep walks, through the stale bucket list, after a prediction."""
    from polymps_gb300 import mps
    c = CASES[name]()
    o, g = _pair(oracle_mod, mps, c)
    o.initialize()
    for _ in range(3):
        o.step()
    sync(o, g)
    for ob in (o, g):
        ob.run_op("UPDATE_BUCKETS")
    # move particles as the predictor does (stale list, current positions)
    for ob in (o, g):
        ob.run_op("VISCOSITY"); ob.run_op("ADD_GRAVITY"); ob.run_op("PREDICT")
    compare(o, g, "predict", [abi.F_POS])
    g.set(abi.F_POS, o.get(abi.F_POS))
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert np.array_equal(co, cg)
    assert np.array_equal(no, ng)   # same sets in the same (reference) order


def test_neighbor_sets_adversarial(oracle_mod, mps_lib):
    """Pairs placed at r^2 = reL^2 and one ulp either side, and on bucket faces."""
    from polymps_gb300 import mps
    c = cases.config(3, scale=5.0)
    o0 = oracle_mod.Oracle(c)
    p = o0.params
    rng = np.random.default_rng(7)
    pos = c.pos.copy()
    n = len(pos)
    re = p.reL
    for k in range(0, n - 1, 7):
        d = rng.normal(size=3); d /= np.linalg.norm(d)
        r = re * [1.0, 1.0 + 2e-16, 1.0 - 2e-16, 1.0 + 1e-12][k % 4]
        pos[k + 1] = pos[k] + r * d
    # snap some particles onto bucket faces
    for k in range(3, n, 11):
        pos[k, 0] = p.domainMin[0] + np.round((pos[k, 0] - p.domainMin[0]) / p.bucketSide) * p.bucketSide
    c2 = cases.Case(c.name, c.params, c.type, pos, c.mesh)
    o, g = _pair(oracle_mod, mps, c2)
    for ob in (o, g):
        ob.run_op("UPDATE_BUCKETS")
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert np.array_equal(co, cg)
    assert np.array_equal(no, ng)


@pytest.mark.parametrize("name", list(CASES))
def test_operator_parity_teacher_forced(oracle_mod, mps_lib, name):
    """Every operator of the step, in the reference order, from an identical state."""
    from polymps_gb300 import mps
    c = CASES[name]()
    o, g = _pair(oracle_mod, mps, c)
    o.initialize()
    g.initialize()
    for s in range(4):
        o.step()
    # the wall repulsion uses velMax of the last corrector: the GPU has run none yet, so
    # start both from 0; from the second forced step on both carry their own (synced) value
    o.set_velmax(0.0)
    for s in range(3):
        sync(o, g)
        for op in step_ops(o.params):
            o.run_op(op)
            g.run_op(op)
            compare(o, g, "step %d op %s" % (s, op))
            sync(o, g)


@pytest.mark.parametrize("name", ["cfg3_relax_0.7_grad2", "cfg1_relax_0.8"])
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
def test_prediction_pressure_gradient(oracle_mod, mps_lib, name, precision):
    """The prediction-step gradient right after the start-of-step sweeps, with no state set
    in between: the GPU reads the start-of-step skin list built by the viscosity sweep (the
    teacher-forced test, which sets the state before every operator, covers the bucket
    scan).  FP64 in both tiers: the acceleration within 1e-10 of the oracle's once the
    viscosity term (the tier's own) is taken from the oracle."""
    from polymps_gb300 import mps
    c = CASES[name]()
    o = oracle_mod.Oracle(c)
    o.set_solver(1e-12)
    g = mps.MpsGpu(c, tol=1e-12, precision=precision)
    o.initialize()
    for _ in range(4):
        o.step()
    ops = step_ops(o.params)
    for s in range(2):
        sync(o, g)
        o.set_velmax(0.0)   # the GPU handle has run no corrector (wall repulsion reads velMax)
        for op in ("UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY"):
            o.run_op(op)
            g.run_op(op)
        acc0, gacc0 = o.get(abi.F_ACC), g.get(abi.F_ACC)
        assert relerr(gacc0, acc0) <= (FP64_RTOL if precision == abi.PRECISION_FP64 else 1e-8)
        o.run_op("PREDICT_PRESS_GRADIENT")
        g.run_op("PREDICT_PRESS_GRADIENT")
        term_o = o.get(abi.F_ACC) - acc0
        term_g = g.get(abi.F_ACC) - gacc0
        assert np.linalg.norm(term_o) > 0
        e = relerr(term_g, term_o)
        assert e <= FP64_RTOL, "step %d: prediction gradient rel err %.3e" % (s, e)
        for op in ops[ops.index("PREDICT"):]:   # finish the step, then one more
            o.run_op(op)
        o.step()
    g.close()
    o.close()


@pytest.mark.parametrize("layout", ["10", "0", "8"])
@pytest.mark.parametrize("name", ["cfg3_3d_inc_polygon", "cfg1_2d_particle_walls"])
def test_ppe_system_and_solution(oracle_mod, mps_lib, name, layout, monkeypatch):
    """The assembled system and its solution against the oracle, in each ELL layout of the
    library (MPSGPU_ELL_SLICE, read when a handle is created: 1024-row slices by default,
    column-major over all rows, 256-row slices)."""
    from polymps_gb300 import mps
    monkeypatch.setenv("MPSGPU_ELL_SLICE", layout)
    c = CASES[name]()
    o, g = _pair(oracle_mod, mps, c, tol=1e-12)
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
    assert relerr(vg, vo) < 1e-13
    assert relerr(bg, bo) < 1e-12
    assert relerr(g.get(abi.F_PRESSPPE), o.get(abi.F_PRESSPPE)) < 1e-9
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-9


@pytest.mark.parametrize("name", list(CASES))
def test_free_running_steps(oracle_mod, mps_lib, name):
    """Whole steps through mpsgpu_step vs the oracle: trajectories agree to the solver
    tolerance over a short window (they diverge chaotically over long ones)."""
    from polymps_gb300 import mps
    c = CASES[name]()
    o, g = _pair(oracle_mod, mps, c, tol=1e-12)
    o.initialize()
    g.initialize()
    for s in range(10):
        so = o.step()
        sg = g.step()
        assert sg.numParticles == so.numParticles
    assert relerr(g.get(abi.F_POS), o.get(abi.F_POS)) < 1e-10
    assert relerr(g.get(abi.F_VEL), o.get(abi.F_VEL)) < 1e-6
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-6


@pytest.mark.parametrize("layout", ["10", "0"])
def test_mixed_precision_solver(oracle_mod, mps_lib, layout, monkeypatch):
    """FP32 inner CG + FP64 refinement reaches the FP64 residual 1e-8 and its pressure
    stays within 1e-6 (normwise relative) of the FP64 oracle solved to 1e-12 (sliced and
    column-major ELL layouts)."""
    from polymps_gb300 import mps
    monkeypatch.setenv("MPSGPU_ELL_SLICE", layout)
    c = cases.config(3, jitter=0.02, scale=4.0)
    o, g = _pair(oracle_mod, mps, c, tol=1e-12)
    o.initialize()
    g.initialize()
    for s in range(6):
        o.step()
    g.set_solver(abi.SOLVER_MIXED, abi.WARM_PREVIOUS, 1e-8)
    sync(o, g)
    for op in step_ops(o.params)[: step_ops(o.params).index("CALC_PRESS")]:
        o.run_op(op); g.run_op(op); sync(o, g)
    o.run_op("CALC_PRESS")
    g.run_op("CALC_PRESS")
    st = g.last_stats()
    assert st.ppeRelResidual <= 1e-8
    assert st.ppeRefinements >= 1
    assert relerr(g.get(abi.F_PRESSPPE), o.get(abi.F_PRESSPPE)) < 1e-6
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-6
    st = g.step()   # a full mixed step must also converge
    assert st.ppeRelResidual <= 1e-8


def _bf16(x):
    """Round-to-nearest-even FP32 -> BF16 -> FP32 (numpy)."""
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


# GELU in its tanh form, as the kernels evaluate it (with the hardware tanh)
_K0, _K1 = np.sqrt(2.0 / np.pi), 0.044715


def _gelu(z):
    return 0.5 * z * (1.0 + np.tanh(_K0 * (z + _K1 * z ** 3)))


def _gelud(z):
    t = np.tanh(_K0 * (z + _K1 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _K0 * (1.0 + 3.0 * _K1 * z * z)


def _mlp_ref(params, norm, feat, want_grad=False, target=None):
    H, NF = 64, 16
    o = 0
    W1 = params[o:o + H * NF].reshape(H, NF); o += H * NF
    b1 = params[o:o + H]; o += H
    W2 = params[o:o + H * H].reshape(H, H); o += H * H
    b2 = params[o:o + H]; o += H
    W3 = params[o:o + H * H].reshape(H, H); o += H * H
    b3 = params[o:o + H]; o += H
    W4 = params[o:o + H]; o += H
    b4 = params[o]
    g = _gelu
    x = _bf16((feat - norm[:16]) * norm[16:32]).astype(np.float64)
    z1 = x @ _bf16(W1).T.astype(np.float64) + b1
    h1 = _bf16(g(z1))
    z2 = h1 @ _bf16(W2).T.astype(np.float64) + b2
    h2 = _bf16(g(z2))
    z3 = h2 @ _bf16(W3).T.astype(np.float64) + b3
    out = g(z3) @ _bf16(W4).astype(np.float64) + b4
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_mlp_forward_matches_cpu(mps_lib, seed):
    from polymps_gb300 import mps
    rng = np.random.default_rng(seed)
    c = cases.config(3, scale=8.0)
    g = mps.MpsGpu(c)
    params = (rng.normal(size=abi.MLP_NPARAM) * 0.2).astype(np.float32)
    norm = np.concatenate([rng.normal(size=16), 0.5 + rng.random(16), [0.0, 1.0]]).astype(np.float32)
    g.mlp_set_weights(params, norm)
    feat = rng.normal(size=(1000, 16)).astype(np.float32)
    out = g.mlp_forward(feat)
    ref = _mlp_ref(params.astype(np.float64), norm.astype(np.float64), feat.astype(np.float64))
    # BF16 activations and FP32 accumulation: 2^-8 relative per rounding
    assert np.max(np.abs(out - ref)) <= 2e-2 * (np.max(np.abs(ref)) + 1.0)


def _mlp_grad_ref(params, feat, target):
    """Exact backprop (FP64) of the network with BF16-rounded weights and hidden inputs,
    as the tensor-core kernels evaluate it; mean squared error over the samples."""
    H, NF = 64, 16
    sl = {}
    o = 0
    for name, size in (("W1", H * NF), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * H), ("b3", H), ("W4", H), ("b4", 1)):
        sl[name] = slice(o, o + size); o += size
    W1 = _bf16(params[sl["W1"]]).astype(np.float64).reshape(H, NF)
    W2 = _bf16(params[sl["W2"]]).astype(np.float64).reshape(H, H)
    W3 = _bf16(params[sl["W3"]]).astype(np.float64).reshape(H, H)
    W4 = _bf16(params[sl["W4"]]).astype(np.float64)
    b1, b2, b3, b4 = (params[sl[k]].astype(np.float64) for k in ("b1", "b2", "b3", "b4"))
    g, gd = _gelu, _gelud
    x = _bf16(feat).astype(np.float64)
    z1 = x @ W1.T + b1; h1 = _bf16(g(z1)).astype(np.float64)
    z2 = h1 @ W2.T + b2; h2 = _bf16(g(z2)).astype(np.float64)
    z3 = h2 @ W3.T + b3; h3 = g(z3)
    out = h3 @ W4 + b4[0]
    n = len(feat)
    e = out - target
    loss = np.mean(e * e)
    dout = 2 * e / n
    grad = np.zeros(len(params))
    grad[sl["W4"]] = dout @ h3
    grad[sl["b4"]] = dout.sum()
    dz3 = np.outer(dout, W4) * gd(z3)
    grad[sl["W3"]] = (dz3.T @ h2).ravel(); grad[sl["b3"]] = dz3.sum(0)
    dz2 = (dz3 @ W3) * gd(z2)
    grad[sl["W2"]] = (dz2.T @ h1).ravel(); grad[sl["b2"]] = dz2.sum(0)
    dz1 = (dz2 @ W2) * gd(z1)
    grad[sl["W1"]] = (dz1.T @ x).ravel(); grad[sl["b1"]] = dz1.sum(0)
    return grad, loss, sl


def test_mlp_gradient_matches_cpu(mps_lib):
    """Tensor-core backward (activation and weight gradients) against an FP64 numpy
    backprop of the same BF16-rounded network: every parameter block within 3%
    normwise (BF16 rounding of the staged gradients is 2^-9 relative)."""
    from polymps_gb300 import mps
    rng = np.random.default_rng(3)
    c = cases.config(3, scale=8.0)
    g = mps.MpsGpu(c)
    params = (rng.normal(size=abi.MLP_NPARAM) * 0.3).astype(np.float32)
    norm = np.concatenate([np.zeros(16), np.ones(16), [0.0, 1.0]]).astype(np.float32)
    g.mlp_set_weights(params, norm)
    n = 512
    feat = rng.normal(size=(n, 16)).astype(np.float32)
    target = rng.normal(size=n).astype(np.float32)
    grad, loss = g.mlp_gradient(feat, target)
    ref, loss_ref, sl = _mlp_grad_ref(params.astype(np.float64), feat.astype(np.float64), target.astype(np.float64))
    assert loss == pytest.approx(loss_ref, rel=1e-2)
    for name, s in sl.items():
        a, b = grad[s].astype(np.float64), ref[s]
        assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-7, name


@pytest.mark.parametrize("solver", [abi.SOLVER_PLAIN_FP64, abi.SOLVER_MIXED])
def test_ppe_launch_modes_agree(oracle_mod, mps_lib, solver):
    """The single cooperative launch (block-owned rows with the inner-CG vectors in shared
    memory, grid-stride rows with the vectors in global memory, the staged ELL tiles, the
    pipelined inner CG of the mixed solver) and the per-kernel launches solve the same
    system to the same tolerance (same method; rounding differs)."""
    from polymps_gb300 import mps
    c = CASES["cfg3_3d_inc_polygon"]()
    out = []
    for mode in (2, 1, 0, 3, 4):
        g = mps.MpsGpu(c, solver=solver, tol=1e-10)
        g.set_ppe_launch(mode)
        g.initialize()
        st = g.run(3)
        assert st.ppeRelResidual <= 1e-10
        out.append((g.get(abi.F_PRESS), st.ppeIterations))
        g.close()
    for k in (1, 2, 3, 4):
        assert relerr(out[0][0], out[k][0]) < 1e-8
        assert abs(out[0][1] - out[k][1]) <= 3 + 3 * (k == 3)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
def test_mixed_solver_storage_orders(mps_lib, precision):
    """108k particles in random storage order (matrix columns anywhere in the index range)
    and, after the bucket-order renumbering of the 20th rebuild, in bucket order: the mixed
    solution reaches the FP64 residual 1e-8 and stays within 1e-6 (normwise) of the FP64
    solve of the same system to 1e-12."""
    from polymps_gb300 import mps
    c = cases.config(3, jitter=0.02, scale=2.0)
    perm = np.random.default_rng(7).permutation(c.n)
    c = cases.Case(c.name, c.params, c.type[perm], c.pos[perm], c.mesh)
    g = mps.MpsGpu(c, precision=precision, solver=abi.SOLVER_MIXED, tol=1e-8)
    g.initialize()
    ops = step_ops(g.params)
    k = ops.index("CALC_PRESS")
    hist_f = (abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2)
    done = 0
    for upto in (2, 23):   # steps before the checked one
        g.run(upto - done)
        done = upto + 1
        for op in ops[:k]:
            g.run_op(op)
        hist = [g.get(f) for f in hist_f]
        g.set_solver(abi.SOLVER_PLAIN_FP64, abi.WARM_PREVIOUS, 1e-12, 20000)
        g.run_op("CALC_PRESS")
        p_ref = g.get(abi.F_PRESSPPE)
        for f, v in zip(hist_f, hist):
            g.set(f, v)
        g.set_solver(abi.SOLVER_MIXED, abi.WARM_PREVIOUS, 1e-8, 20000)
        g.run_op("CALC_PRESS")
        st = g.last_stats()
        assert st.ppeRelResidual <= 1e-8
        assert relerr(g.get(abi.F_PRESSPPE), p_ref) < 1e-6
        for op in ops[k + 1:]:
            g.run_op(op)
    g.close()


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
@pytest.mark.parametrize("name", ["cfg1_2d_particle_walls", "cfg3_3d_inc_polygon"])
def test_out_of_domain_removal(oracle_mod, mps_lib, name, precision):
    """Fluid particles pushed outside the domain margin (one of them the last index) are
    removed by the reference's swap-with-last replay; fields, counts and the neighbour
    lists read through the step's stale bucket list afterwards match the oracle."""
    from polymps_gb300 import mps
    c = CASES[name]()
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12, precision=precision)
    o.set_solver(1e-12)
    o.initialize()
    g.initialize()
    for _ in range(2):
        o.step()
    sync(o, g)
    for ob in (o, g):
        ob.run_op("UPDATE_BUCKETS")
    p = o.params
    pos = o.get(abi.F_POS)
    typ = o.get(abi.F_TYPE)
    fl = np.nonzero(typ == p.fluid)[0]
    pick = [fl[len(fl) // 3], fl[len(fl) // 2], fl[-1], fl[5]]
    for k in pick:
        pos[k, 0] = p.domainMax[0] - 0.5 * p.bucketSide
    for ob in (o, g):
        ob.set(abi.F_POS, pos)
        ob.run_op("OUT_OF_DOMAIN")
    # the last index is among the pushed ones: copied into an earlier freed index, it is not
    # re-checked (the reference's loop), so fewer than four leave
    assert g.n == o.n and len(pos) - 4 <= o.n < len(pos)
    compare(o, g, "out of domain")
    co, no = o.neighbors()
    cg, ng = g.neighbors()
    assert np.array_equal(co, cg)
    assert np.array_equal(no, ng)


def test_field_transfers_page_locked(mps_lib):
    """Fields read into and written from page-locked host arrays (the end-to-end bench's
    buffers) equal the transfers through pageable arrays, in both directions."""
    torch = pytest.importorskip("torch")
    from polymps_gb300 import mps
    c = CASES["cfg3_3d_inc_polygon"]()
    g = mps.MpsGpu(c)
    g.initialize()
    g.run(2)

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64 if a.dtype == np.float64 else torch.int32).pin_memory()
        v = t.numpy().reshape(a.shape)
        return v, t

    for f in (abi.F_POS, abi.F_VEL, abi.F_PRESS, abi.F_PRESSPPE, abi.F_BC, abi.F_NUMNEIGH):
        a = g.get(f)
        v, keep = pinned(a)
        g.get(f, out=v)
        assert np.array_equal(v, a), abi.FIELD_NAMES[f]
        if f in abi.INT_FIELDS:
            continue
        v[...] = a * 1.5 + 0.25
        g.set(f, v)
        assert np.array_equal(g.get(f), v), abi.FIELD_NAMES[f]
        g.set(f, a)
    st = g.step()
    assert st.ppeRelResidual <= 1e-8
    g.close()
