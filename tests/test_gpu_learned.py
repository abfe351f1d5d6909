"""What the trained warm-start network gains over the method without it.

The network is trained on the GPU by the library's own kernels (records of the plain FP64
solver on the 3D incompressible dam break, fused BF16 forward/backward, Adam), then the
same held-out PPE systems are solved by the FP32/FP64 refinement solver from three
starts: the previous-step pressure (the reference's warm start), the quadratic
extrapolation x_e = 3 p_n - 3 p_{n-1} + p_{n-2} (the learned start without the network),
and the learned start x_e + theta c (network correction c, residual-minimising step theta).
Every start's pressure (FP64 residual 1e-8) must lie within 1e-6 relative of the CPU
oracle's Jacobi-PCG of the same system solved to 1e-12 (src/MpsPressure.cpp:424-445).
"""
import os

import numpy as np
import pytest

from polymps_gb300 import abi, cases

pytestmark = pytest.mark.gpu

OPS_BEFORE = ["UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY", "PREDICT", "OUT_OF_DOMAIN", "COLLISION",
              "WALL_DISTANCE", "WALL_NPCD", "PND_NEIGH_NPCD", "UPDATE_BC"]
OPS_AFTER = ["CORRECTION_MATRIX", "PRESS_GRADIENT", "WALL_PRESS_GRADIENT", "WALL_VISCOSITY", "CORRECT",
             "OUT_OF_DOMAIN"]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_learned_warm_start_gain(oracle_mod, mps_lib):
    from polymps_gb300 import mps, train_warmstart as tw
    c = cases.config(4, scale=2.0)   # l0 = 0.02 m
    g = mps.MpsGpu(c, solver=abi.SOLVER_PLAIN_FP64, tol=1e-10, max_iter=20000, precision=abi.PRECISION_DF32)
    g.initialize()
    g.run(10)
    for s in range(80):
        g.mlp_record(s % 2 == 0)
        g.step()
    g.mlp_record(False)
    assert g.mlp_num_records() > 100000
    rng = np.random.default_rng(5)
    g.mlp_set_weights(tw.init_params(rng), np.concatenate([np.zeros(16), np.ones(16), [0.0, 1.0]]).astype(np.float32))
    g.mlp_fit_normalization()
    p0, norm = g.mlp_get_weights()
    g.mlp_set_weights(p0, norm)
    first = float(np.mean(g.mlp_train(200, 4096, 2e-3, seed=1)))
    last = float(np.mean(g.mlp_train(800, 4096, 1e-3, seed=2)))
    assert last < first   # the network learns the correction on its own kernels

    rows = []
    for s in range(8):   # held-out systems: later steps of the same run
        for op in OPS_BEFORE:
            g.run_op(op)
        xp, xq, xr = g.get(abi.F_PRESSPPE), g.get(abi.F_PRESSPPE_PREV), g.get(abi.F_PRESSPPE_PREV2)
        out = {}
        for name, solver, warm, tol in (("assemble", abi.SOLVER_PLAIN_FP64, abi.WARM_PREVIOUS, 1e-8),
                                        ("previous", abi.SOLVER_MIXED, abi.WARM_PREVIOUS, 1e-8),
                                        ("extrapolated", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 1e-8),
                                        ("learned", abi.SOLVER_MIXED, abi.WARM_MLP, 1e-8)):
            g.set(abi.F_PRESSPPE, xp)
            g.set(abi.F_PRESSPPE_PREV, xq)
            g.set(abi.F_PRESSPPE_PREV2, xr)
            g.set_solver(solver, warm, tol, 20000)
            g.run_op("CALC_PRESS")
            st = g.last_stats()
            assert st.ppeRelResidual <= tol
            out[name] = (st.ppeInitialRelResidual, st.ppeIterations, g.get(abi.F_PRESSPPE))
            if name == "assemble":
                # the oracle's Jacobi-PCG (Eigen's CG restated) on the same system, to 1e-12
                rowptr, col, val, rhs = g.ppe()
                x_orc, _, err = oracle_mod.pcg_csr(rowptr, col, val, rhs, xp, 1e-12, 20000)
                assert err <= 1e-12
        for name in ("previous", "extrapolated", "learned"):
            assert _rel(out[name][2], x_orc) < 1e-6
        rows.append({k: v[:2] for k, v in out.items() if k != "assemble"})
        for op in OPS_AFTER:
            g.run_op(op)
    g.close()
    r0 = {k: np.array([r[k][0] for r in rows]) for k in ("previous", "extrapolated", "learned")}
    it = {k: np.array([r[k][1] for r in rows]) for k in ("previous", "extrapolated", "learned")}
    print("initial relative residual (mean): previous %.3e  extrapolated %.3e  learned %.3e"
          % (r0["previous"].mean(), r0["extrapolated"].mean(), r0["learned"].mean()))
    print("inner iterations (mean): previous %.2f  extrapolated %.2f  learned %.2f"
          % (it["previous"].mean(), it["extrapolated"].mean(), it["learned"].mean()))
    print("network gain over the extrapolated start: residual x%.3f, iterations %+.2f"
          % (r0["extrapolated"].mean() / r0["learned"].mean(), it["extrapolated"].mean() - it["learned"].mean()))
    # the residual-minimising step never leaves a larger residual than the extrapolation
    assert np.all(r0["learned"] <= r0["extrapolated"] * (1.0 + 1e-6))
    # and the learned start beats the reference's previous-step start
    assert r0["learned"].mean() < r0["previous"].mean()



def _system_after_steps(mps, steps=12):
    """A PPE system of the 3D dam break at l0 = 0.02 m after a few steps (the operators
    before the pressure run) and the warm-start history of its unclamped solutions."""
    c = cases.config(4, scale=2.0)
    g = mps.MpsGpu(c, solver=abi.SOLVER_MIXED, tol=1e-8, max_iter=20000, precision=abi.PRECISION_DF32)
    w = np.load(os.path.join(os.path.dirname(mps.__file__), "mlp_warmstart.npz"))
    g.mlp_set_weights(w["params"], w["norm"])
    g.initialize()
    g.run(steps)
    for op in OPS_BEFORE:
        g.run_op(op)
    hist = [g.get(f) for f in (abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2)]
    return g, w, hist


def _solve(mps, g, hist, solver, warm, max_iter):
    """CALC_PRESS from the same history; returns the status code, the stats and pressurePPE."""
    for f, v in zip((abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2), hist):
        g.set(f, v)
    g.set_solver(solver, warm, 1e-8, max_iter)
    code = 0
    try:
        g.run_op("CALC_PRESS")
    except mps.MpsError as err:
        code = err.code
    return code, g.last_stats(), g.get(abi.F_PRESSPPE)


def test_learned_start_with_a_broken_network(mps_lib):
    """Non-finite network weights: the residual-minimising step rejects the correction
    (theta = 0), the start is the quadratic extrapolation, and the solve converges to the
    extrapolated start's pressure."""
    from polymps_gb300 import mps
    g, w, hist = _system_after_steps(mps)
    code_e, st_e, x_e = _solve(mps, g, hist, abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 20000)
    bad = np.array(w["params"], dtype=np.float32)
    bad[-1] = np.nan   # output bias
    g.mlp_set_weights(bad, w["norm"])
    code_l, st_l, x_l = _solve(mps, g, hist, abi.SOLVER_MIXED, abi.WARM_MLP, 20000)
    g.close()
    assert code_e == 0 and code_l == 0
    assert st_l.ppeRelResidual <= 1e-8 and st_l.ppeFallback == 0
    assert st_l.ppeInitialRelResidual == pytest.approx(st_e.ppeInitialRelResidual, rel=1e-9)
    assert _rel(x_l, x_e) < 1e-9


@pytest.mark.parametrize("warm", [abi.WARM_MLP, abi.WARM_PREVIOUS])
def test_mixed_solve_falls_back_to_plain_cg(mps_lib, warm):
    """A mixed solve that misses the tolerance within max_iter is redone by the plain FP64
    CG from the previous unclamped solution (the reference's solver): with the same budget
    the result is the plain solver's own, bit for bit, the stats report the fallback, and
    the status reports that the plain CG missed the tolerance as well."""
    from polymps_gb300 import mps
    g, w, hist = _system_after_steps(mps)
    code_m, st_m, _ = _solve(mps, g, hist, abi.SOLVER_MIXED, warm, 20000)
    assert code_m == 0 and st_m.ppeFallback == 0 and st_m.ppeRelResidual <= 1e-8
    short = 3
    assert st_m.ppeIterations > short
    code_s, st_s, x_s = _solve(mps, g, hist, abi.SOLVER_PLAIN_FP64, abi.WARM_PREVIOUS, short)
    code_f, st_f, x_f = _solve(mps, g, hist, abi.SOLVER_MIXED, warm, short)
    g.close()
    assert code_s == abi.ERR_NOT_CONVERGED and st_s.ppeFallback == 0
    assert code_f == abi.ERR_NOT_CONVERGED and st_f.ppeFallback == 1
    assert np.array_equal(x_f, x_s)


def test_learned_start_matches_host_reconstruction(mps_lib):
    """The learned start of the single-launch mixed solve (features from the FP64 start x_e
    and its FP64 residual, which the solver's set-up then starts from) against the same
    start rebuilt step by step on the host: the recorded-feature definitions (FP32 residual
    pass), the system scale sigma, the network on those inputs, c, the residual-minimising
    step theta = (r_e . A c) / (A c . A c) with the exported FP64 system, and the initial
    relative residual ||r_e - theta A c|| / ||b||."""
    from polymps_gb300 import mps
    inner = cases.config(4, scale=2.0).params["inner"]
    g, w, hist = _system_after_steps(mps)
    code_e, st_e, _ = _solve(mps, g, hist, abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 20000)
    code_l, st_l, _ = _solve(mps, g, hist, abi.SOLVER_MIXED, abi.WARM_MLP, 20000)
    assert code_e == 0 and code_l == 0 and st_l.ppeFallback == 0
    for f, v in zip((abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2), hist):
        g.set(f, v)
    feat = g.ppe_features()
    rowptr, col, val, rhs = g.ppe()
    eq = g.get(abi.F_BC).reshape(-1) == inner
    _, norm = g.mlp_get_weights()
    xe = np.where(eq, 3.0 * (hist[0] - hist[1]) + hist[2], 0.0)
    n = len(rhs)
    rows = np.repeat(np.arange(n), np.diff(rowptr))

    def matvec(x):
        return np.bincount(rows, weights=val[:rowptr[-1]] * x[col[:rowptr[-1]]], minlength=n)

    r = rhs - matvec(xe)
    sig = float(np.sqrt(np.mean(feat[eq, 7].astype(np.float64) ** 2)))
    fs = feat.copy()
    fs[:, [1, 5, 7, 14]] *= np.float32(1.0 / sig)
    g_out = g.mlp_forward(fs).astype(np.float64)
    g.close()
    c = np.where(eq, (g_out / norm[2 * 16 + 1] + norm[2 * 16]) * sig, 0.0)
    q = matvec(c)
    theta = float(r @ q) / float(q @ q)
    r0_host = float(np.linalg.norm(r - theta * q) / np.linalg.norm(rhs))
    r0_extrap = float(np.linalg.norm(r) / np.linalg.norm(rhs))
    print("initial relative residual: extrapolated %.4e (GPU %.4e), learned host %.4e GPU %.4e, theta %.3f"
          % (r0_extrap, st_e.ppeInitialRelResidual, r0_host, st_l.ppeInitialRelResidual, theta))
    assert st_e.ppeInitialRelResidual == pytest.approx(r0_extrap, rel=1e-6)
    assert r0_host < 0.95 * r0_extrap   # the network moves the start, so the comparison below means something
    assert st_l.ppeInitialRelResidual == pytest.approx(r0_host, rel=1e-2)
