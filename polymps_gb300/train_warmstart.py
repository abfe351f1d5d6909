"""Train the learned PPE warm start on the GPU with libmpsgpu's own kernels.

1. Run the 3D incompressible polygon dam break at l0 = 0.01 m (108,000 particles; or, with
   --config 3, at the evaluation resolution l0 = 0.005 m) with the
   plain FP64 solver (previous-step warm start, tolerance 1e-10) and record, for every
   inner row of every recorded step, the 16 features of the assembled system and the
   difference between the converged pressure and the temporal extrapolation
   3 p_n - 3 p_{n-1} + p_{n-2} of the three previous solutions (the network learns that
   correction).
2. Fit the feature normalisation on the recorded set, then run Adam on mini-batches with
   the fused BF16 tensor-core forward/backward kernel.
3. Evaluate on the l0 = 0.005 case (864,000 particles): PPE iterations and time to 1e-8
   with the learned warm start against the previous-step and the extrapolated warm
   starts, same systems.

    python -m polymps_gb300.train_warmstart [--steps 600] [--iters 3000] [--out PATH]
"""
import argparse
import json
import os
import time

import numpy as np

from . import abi, build, cases, mps

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "mlp_warmstart.npz")


def init_params(rng):
    """He-style initialisation, small output layer (the network starts near 'no change')."""
    H, NF = 64, 16
    p = []
    p.append(rng.normal(0, np.sqrt(2.0 / NF), size=H * NF)); p.append(np.zeros(H))
    p.append(rng.normal(0, np.sqrt(2.0 / H), size=H * H)); p.append(np.zeros(H))
    p.append(rng.normal(0, np.sqrt(2.0 / H), size=H * H)); p.append(np.zeros(H))
    p.append(rng.normal(0, 0.01, size=H)); p.append(np.zeros(1))
    return np.concatenate(p).astype(np.float32)


def record(steps, every, tol, scale=1.0, warmup=20, config=4):
    c = cases.config(config, scale=scale)
    g = mps.MpsGpu(c, solver=abi.SOLVER_PLAIN_FP64, tol=tol, max_iter=20000, precision=abi.PRECISION_DF32)
    g.initialize()
    g.run(warmup)
    t0 = time.perf_counter()
    for s in range(steps):
        g.mlp_record(s % every == 0)
        g.step()
    g.mlp_record(False)
    return g, c, time.perf_counter() - t0


def evaluate(params, norm, scale=1.0, steps=30, warmup=10, tol=1e-8):
    """Same systems, eight solves each: the plain FP64 CG and the FP32/FP64 refinement
    solver, each from the previous-step, the linear and quadratic extrapolation and the
    learned warm start."""
    c = cases.config(3, scale=scale)
    g = mps.MpsGpu(c, solver=abi.SOLVER_MIXED, tol=tol, max_iter=20000, precision=abi.PRECISION_DF32)
    g.mlp_set_weights(params, norm)
    g.set_solver(abi.SOLVER_MIXED, abi.WARM_EXTRAP2, tol, 20000)
    g.initialize()
    g.run(warmup)
    ops = ["UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY", "PREDICT", "OUT_OF_DOMAIN", "COLLISION",
           "WALL_DISTANCE", "WALL_NPCD", "PND_NEIGH_NPCD", "UPDATE_BC"]
    rows = []
    for s in range(steps):
        for op in ops:
            g.run_op(op)
        hist = [g.get(f) for f in (abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2)]
        res = {}
        for solver, sname in ((abi.SOLVER_PLAIN_FP64, "plain"), (abi.SOLVER_MIXED, "mixed")):
            for warm, wname in ((abi.WARM_PREVIOUS, "prev"), (abi.WARM_EXTRAP, "extrap"),
                                (abi.WARM_EXTRAP2, "extrap2"), (abi.WARM_MLP, "mlp")):
                for f, h in zip((abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2), hist):
                    g.set(f, h)
                g.set_solver(solver, warm, tol, 20000)
                g.run_op("CALC_PRESS")
                st = g.last_stats()
                res[sname + "_" + wname] = (st.ppeIterations, st.ppeSolveMs, st.ppeInitialRelResidual,
                                            st.ppeRelResidual)
        rows.append(res)
        # finish the step from the quadratic extrapolation with the refinement solver
        for f, h in zip((abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2), hist):
            g.set(f, h)
        g.set_solver(abi.SOLVER_MIXED, abi.WARM_EXTRAP2, tol, 20000)
        g.run_op("CALC_PRESS")
        for op in ["CORRECTION_MATRIX", "PRESS_GRADIENT", "WALL_PRESS_GRADIENT", "WALL_VISCOSITY", "CORRECT",
                   "OUT_OF_DOMAIN"]:
            g.run_op(op)
    g.close()
    summ = {}
    for k in rows[0]:
        it = np.array([r[k][0] for r in rows]); ms = np.array([r[k][1] for r in rows])
        r0 = np.array([r[k][2] for r in rows])
        summ[k] = {"iters_mean": float(it.mean()), "ms_mean": float(ms.mean()), "relres0_mean": float(r0.mean()),
                   "relres_max": float(max(r[k][3] for r in rows))}
    return summ


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--every", type=int, default=2)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--eval-steps", type=int, default=20)
    ap.add_argument("--eval-scale", type=float, default=1.0)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--config", type=int, default=4, choices=[3, 4],
                    help="recorded workload: 4 = l0 0.01 m (108k particles), 3 = l0 0.005 m (864k, the "
                         "evaluation resolution)")
    ap.add_argument("--warmup", type=int, default=20, help="steps before the first recorded one")
    a = ap.parse_args()
    build.build()
    rng = np.random.default_rng(a.seed)
    g, c, t_rec = record(a.steps, a.every, tol=1e-10, warmup=a.warmup, config=a.config)
    nrec = g.mlp_num_records()
    g.mlp_set_weights(init_params(rng), np.concatenate([np.zeros(16), np.ones(16), [0.0, 1.0]]).astype(np.float32))
    g.mlp_fit_normalization()
    p0, norm = g.mlp_get_weights()
    g.mlp_set_weights(p0, norm)
    t0 = time.perf_counter()
    losses = []
    lr = a.lr
    chunk = 500
    done = 0
    while done < a.iters:
        k = min(chunk, a.iters - done)
        losses.append(g.mlp_train(k, a.batch, lr, seed=a.seed + done))
        done += k
        lr *= 0.7
    t_train = time.perf_counter() - t0
    params, norm = g.mlp_get_weights()
    g.close()
    loss = np.concatenate(losses)
    np.savez(a.out, params=params, norm=norm)
    ev = evaluate(params, norm, scale=a.eval_scale, steps=a.eval_steps)
    report = {"records": int(nrec), "record_s": round(t_rec, 2), "train_s": round(t_train, 2),
              "loss_first": float(loss[:50].mean()), "loss_last": float(loss[-50:].mean()),
              "iters": a.iters, "batch": a.batch, "eval": ev, "out": a.out}
    print(json.dumps(report))


if __name__ == "__main__":
    main()
