"""Benchmark of the PolyMPS per-step particle path on GB300.

Workload: the 3D incompressible polygon dam break (tank 1.61 x 0.6 x 0.6 m, 12-triangle
closed box, fluid block 0.6 x 0.6 x 0.3 m at l0 = 0.005 m: 864,000 particles,
dt = 2.5e-4 s, PPE to relative residual 1e-8), synthetic lattice input (the reference's
.grid files are not available).  A step is one mainLoopOfSimulation iteration.

Metric: particle-steps/s (whole job), plus the PPE time-to-1e-8 of the plain FP64 CG,
the FP32/FP64 refinement solver and the learned warm start on the same systems.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Multi-GPU: the path is run as N independent replicas (one per rank, no collective on
the data path); value = sum of particle-steps over ranks / max time over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"
WORKLOADS = {2: "3D weakly compressible polygon dam break (cfg2)",
             3: "3D incompressible polygon dam break (cfg3)",
             5: "3D incompressible dam break with obstacle, collision and shifting (cfg5)"}
HBM_FALLBACK = 6800.0


# DRAM bytes (read + write) per launch of the single-launch PPE solve over the 100 timed
# steps of the default workload, from one ncu capture of exactly those launches
# (dram__bytes_read.sum + dram__bytes_write.sum, profiles/k_mx_solve_cfg3-864k.md).
MX_SOLVE_TRAFFIC = 4.814e9


def args_():
    a = argparse.ArgumentParser()
    a.add_argument("--gpus", type=int, default=1)
    a.add_argument("--steps", type=int, default=100)
    a.add_argument("--warmup", type=int, default=5)
    a.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    a.add_argument("--solver", default="mixed", choices=["mixed", "plain", "matfree", "compact"])
    a.add_argument("--precision", default="df32", choices=["df32", "fp64"],
                   help="neighbour-sweep arithmetic: float-float (df32) or FP64")
    a.add_argument("--warm", default="auto", choices=["auto", "prev", "mlp", "extrap", "extrap2"],
                   help="auto: quadratic extrapolation (the fastest measured); the learned start is "
                        "timed in the PPE comparison when its weights are present")
    a.add_argument("--scale", type=float, default=1.0, help="l0 multiplier (1 = 864k particles)")
    a.add_argument("--config", type=int, default=3, choices=[2, 3, 5],
                   help="workload: 3 = 864k-particle incompressible dam break (the headline), "
                        "5 = 9.375M particles with obstacle and shifting, 2 = 108k weakly compressible")
    a.add_argument("--e2e-steps", type=int, default=3)
    a.add_argument("--no-cpu-baseline", action="store_true")
    a.add_argument("--cpu-steps", type=int, default=1)
    a.add_argument("--ppe-compare", type=int, default=1)
    a.add_argument("--ppe-steps", type=int, default=0,
                   help="steps the PPE comparison runs on (0: to the workload's configured length)")
    a.add_argument("--presort", action="store_true",
                   help="number the input particles in bucket order (input renumbering only)")
    return a.parse_args()


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# Algorithmic bytes per call of each timed class (each distinct element read or written
# once; neighbour re-reads assumed cache resident).  N particles, E neighbour entries,
# Z off-diagonal PPE non-zeros; df = float-float tier (hi/lo FP32 copies, no weight cache).
def algo_bytes(cls, N, E, Z, mixed, df, st=None, matfree=False, compact=False):
    if cls == "PPE_SOLVE" and st is not None and st.runPpeSolves:
        # one launch = one whole solve; per call averages of the timed run
        it = st.runPpeIterations / st.runPpeSolves
        rf = st.runPpeRefinements / st.runPpeSolves
        if mixed and compact:
            # compact inner iteration: FP16 value + 16-bit offset per entry; wide flag, y, Ap,
            # p per row; update (x_f, p, r_f, Ap, z); once per solve the compact copy (FP32
            # value + column read, FP16 value + offset written) and the scaling
            return it * (49 * N + 4 * Z) + (rf + 1) * (84 * N + 12 * Z) + 12 * Z + 17 * N
        if mixed and matfree:
            # inner iteration with the matrix-free operator: neighbour index per entry; mask,
            # diagonal, own hi/lo position, z, Ap, p per row; update as below
            return it * (96 * N + 4 * Z) + (rf + 1) * (80 * N + 12 * Z)
        if mixed:
            # inner FP32 iteration: SpMV (valf + col per entry; diag, len, z, Ap, p per row)
            # + update (x_f, p, r_f, Ap, M^-1, z per row); per refinement: FP64 residual
            # (val + col per entry; b, r, x, diag, len per row), x update, inner start
            return it * (60 * N + 8 * Z) + (rf + 1) * (80 * N + 12 * Z)
        # FP64 iteration: SpMV (val + col; diag, len, z, Ap, p) + update (x, p, r, Ap, M^-1, z);
        # setup and final residual
        return it * (116 * N + 12 * Z) + 2 * (60 * N + 12 * Z)
    if cls == "PPE_SPMV":
        return N * (16 if mixed else 28) + Z * (8 if mixed else 12)
    if cls == "PPE_VECTOR":
        return N * (4 * 9 if mixed else 8 * 9)
    if cls == "NEIGHBOR_LIST":
        # FP32 copies (pos -> posf/posLo, bucket-ordered copies), list build (+ weights)
        copies = N * (32 + 32) + N * (4 + 32 + 32)
        return copies + N * (32 + 16 + 16 + 4) + (4 * E if df else 20 * E)
    if cls == "PPE_ASSEMBLE":
        return N * (32 + 4 + 4 + 8 + 8 + 4 + 8 + 8) + Z * 12 + (4 * E if df else 12 * E)
    if cls == "PRESS_GRADIENT":
        return N * (32 + 8 + 8 + 3 * 32 + 32) + (N * 16 if df else 0) + (4 * E if df else 12 * E)
    if cls == "PND_NEIGH_NPCD":
        return N * (32 + 8 + 4 + 32 + 32 + 8 * 5 + 4) + (4 * E if df else 12 * E)
    if cls == "CORRECTION_MATRIX":
        return N * (32 + 8 + 4 + 3 * 32) + (4 * E if df else 12 * E)
    if cls == "VISCOSITY":
        return N * (32 + 16 + 16 + 32 + 4 + 32) + (N * 64 if df else 0)
    if cls == "COLLISION":
        return N * (32 + 32 + 32 + 4 + 32) + 4 * E + (N * 64 if df else 0)
    return None


def run_gb300(a, rank, world, local):
    import torch
    from polymps_gb300 import abi, build, cases, mps, replicas
    if world > 1:
        import torch.distributed as dist_
        dist_.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    build.build()
    case = cases.config(a.config, scale=a.scale)
    N = case.n
    if a.presort:
        p0 = mps.derive(case.mps_params(), case.n, case.pos)
        b = np.floor((case.pos - np.array(p0.domainMin[:3])) / p0.bucketSide).astype(np.int64)
        key = (b[:, 2] * p0.numBucketsY + b[:, 1]) * p0.numBucketsX + b[:, 0]
        perm = np.argsort(key, kind="stable")
        case = cases.Case(case.name, case.params, case.type[perm], case.pos[perm], case.mesh)
    solver = {"mixed": abi.SOLVER_MIXED, "plain": abi.SOLVER_PLAIN_FP64, "matfree": abi.SOLVER_MIXED_MATFREE,
              "compact": abi.SOLVER_MIXED_COMPACT}[a.solver]
    mlp_path = os.path.join(ROOT, "polymps_gb300", "mlp_warmstart.npz")
    have_mlp = os.path.exists(mlp_path)
    use_mlp = a.warm == "mlp"
    prec = abi.PRECISION_DF32 if a.precision == "df32" else abi.PRECISION_FP64
    g = mps.MpsGpu(case, solver=solver, tol=1e-8, max_iter=20000, precision=prec)
    warm = {"prev": abi.WARM_PREVIOUS, "extrap": abi.WARM_EXTRAP}.get(a.warm, abi.WARM_EXTRAP2)
    if have_mlp:
        w = np.load(mlp_path)
        g.mlp_set_weights(w["params"], w["norm"])
    if use_mlp:
        warm = abi.WARM_MLP
    g.set_solver(solver, warm, 1e-8, 20000)
    g.initialize()
    g.run(a.warmup)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(local)
    clocks.start()
    g.profile(True)
    l0 = mps.MpsGpu.launch_count()
    t0 = time.perf_counter()
    st = g.run(a.steps)
    wall = time.perf_counter() - t0
    launches = mps.MpsGpu.launch_count() - l0
    prof = g.profile_get()
    g.profile(False)
    clk = clocks.stop()
    torch.cuda.synchronize()
    # replicas: particle-steps of all ranks over the slowest rank's device time
    units, dev_s = replicas.aggregate(N * a.steps, st.stepMs / 1e3, world, device="cuda")
    replicas.barrier(world)
    value = units / dev_s

    # state of the end of the timed run, uploaded every step of the end-to-end section from
    # page-locked host arrays (and the results read back into page-locked arrays)
    def pinned_like(a):
        t = torch.empty(a.size, dtype=torch.float64).pin_memory()
        v = t.numpy().reshape(a.shape)
        v[...] = a
        return v, t
    host, keep = {}, []
    for f in (abi.F_POS, abi.F_VEL, abi.F_PRESS, abi.F_PRESSPPE):
        v, t = pinned_like(g.get(f))
        host[f] = v
        keep.append(t)
    # e2e through the C ABI with host arrays: upload the state from pinned host memory,
    # step, download the result, every step
    h2d = sum(v.nbytes for v in host.values())
    d2h = h2d   # the step's state comes back: positions, velocities, pressure and the unclamped solution
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        for f, v in host.items():
            g.set(f, v)
        g.step()
        g.get(abi.F_POS, out=host[abi.F_POS])
        g.get(abi.F_VEL, out=host[abi.F_VEL])
        g.get(abi.F_PRESS, out=host[abi.F_PRESS])
        g.get(abi.F_PRESSPPE, out=host[abi.F_PRESSPPE])
    e2e_s = time.perf_counter() - t0
    e2e_units, e2e_s = replicas.aggregate(N * a.e2e_steps, e2e_s, world, device="cuda")
    e2e = e2e_units / e2e_s

    # PPE time-to-1e-8 on identical systems along the rest of the run: plain FP64 vs mixed vs
    # warm starts
    ppe = None
    if a.ppe_compare and rank == 0:
        done = a.warmup + a.steps + a.e2e_steps   # steps taken so far (initialisation is step 0)
        steps = a.ppe_steps if a.ppe_steps > 0 else max(getattr(case, "steps", 1000) - done, 40)
        ppe = ppe_compare(g, abi, have_mlp, g.params, (solver, warm, 1e-8, 20000), steps=steps,
                          every=max(1, steps // 36), start=done)
    # dominant class and its roofline
    hbm, hbm_src = peaks()
    E, Z = st.nbrEntries, max(st.ppeNnz - N, 0)
    mixed = solver != abi.SOLVER_PLAIN_FP64
    leaf = {k: v for k, v in prof.items() if k not in ("CALC_PRESS",)}
    dom = max(leaf, key=lambda k: leaf[k][0]) if leaf else None
    roof = None
    if dom:
        ms, calls = leaf[dom]
        b = algo_bytes(dom, N, E, Z, mixed, prec == abi.PRECISION_DF32, st, solver == abi.SOLVER_MIXED_MATFREE,
                       solver == abi.SOLVER_MIXED_COMPACT)
        if b:
            ach = b / (ms / calls / 1e3) / 1e9
            traffic = None
            if (dom == "PPE_SOLVE" and a.config == 3 and a.scale == 1.0 and a.solver == "mixed"
                    and a.precision == "df32" and a.warm in ("auto", "extrap2") and a.steps == 100 and a.warmup == 5):
                traffic = MX_SOLVE_TRAFFIC
            roof = {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(ach / hbm, 4), "peak_source": hbm_src, "traffic": traffic,
                    "algo_bytes_per_launch": int(b), "launch_ms": round(ms / calls, 4),
                    "share_of_step": round(ms / st.stepMs, 3)}

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "particle-steps/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(st.stepMs / a.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("df32" if prec == abi.PRECISION_DF32 else "f64") + ("+f32/f64 PPE" if mixed else "+f64 PPE"),
        "data": "synthetic",
        "config": {"workload": WORKLOADS[a.config], "particles": N,
                   "l0": case.params["partDist"], "dt": case.params["timeStep"],
                   "ppe_tol": 1e-8, "solver": a.solver, "precision": a.precision,
                   "warm_start": {abi.WARM_MLP: "learned", abi.WARM_EXTRAP: "extrapolated",
                                  abi.WARM_EXTRAP2: "quadratic extrapolation", abi.WARM_PREVIOUS: "previous"}[warm],
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "working set > L2 (no flush needed)", "wall_s": round(wall, 3)},
        "e2e": {"value": round(e2e, 1), "unit": "particle-steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": a.e2e_steps},
        "roofline": roof,
        "clocks": clk,
        "gpu_launches": int(launches),
        "ppe": ppe,
        "profile_ms": {k: round(v[0], 3) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
        "last_step": {"ppe_iters": st.ppeIterations, "ppe_relres": st.ppeRelResidual, "velMax": st.velMax},
    }
    g.close()
    # the smooth start of the flow (steps 7-86, every second system) on a fresh simulation:
    # extrapolated and learned starts gain most there
    if a.ppe_compare and rank == 0 and a.ppe_steps == 0:
        g2 = mps.MpsGpu(case, solver=solver, tol=1e-8, max_iter=20000, precision=prec)
        if have_mlp:
            w = np.load(mlp_path)
            g2.mlp_set_weights(w["params"], w["norm"])
        g2.set_solver(solver, warm, 1e-8, 20000)
        g2.initialize()
        g2.run(6)
        out["ppe_early"] = ppe_compare(g2, abi, have_mlp, g2.params, (solver, warm, 1e-8, 20000), steps=80,
                                       every=2, start=7)
        g2.close()
    if rank == 0 and not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(case, a.cpu_steps)
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def _hist_get(g, abi):
    return [g.get(f) for f in (abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2)]


def _hist_set(g, abi, h):
    for f, v in zip((abi.F_PRESSPPE, abi.F_PRESSPPE_PREV, abi.F_PRESSPPE_PREV2), h):
        g.set(f, v)


def _solve(g, abi, hist, solver, warm, mode=1):
    g.set_ppe_launch(mode)
    _hist_set(g, abi, hist)
    g.set_solver(solver, warm, 1e-8, 20000)
    g.run_op("CALC_PRESS")
    st = g.last_stats()
    return {"ms": st.ppeSolveMs, "iters": st.ppeIterations, "refinements": st.ppeRefinements,
            "relres": st.ppeRelResidual, "relres0": st.ppeInitialRelResidual}


def ppe_compare(g, abi, use_mlp, params, default, steps=40, every=4, start=0):
    """PPE time-to-1e-8 of the solvers and warm starts on the same systems, sampled along
    `steps` further steps of the run (every `every`-th system): each sampled system is
    solved by every variant from the same warm-start state, then the step is finished
    with the bench's own solver."""
    before = ["UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY", "PREDICT", "OUT_OF_DOMAIN", "COLLISION"]
    if params.wallType == 1:
        before += ["WALL_DISTANCE", "WALL_NPCD"]
    before += ["PND_NEIGH_NPCD", "UPDATE_BC"]
    after = ["CORRECTION_MATRIX", "PRESS_GRADIENT"] if params.gradientCorrection else ["PRESS_GRADIENT"]
    if params.wallType == 1:
        after += ["WALL_PRESS_GRADIENT", "WALL_VISCOSITY"]
    after += ["CORRECT", "OUT_OF_DOMAIN"] + (["SHIFTING"] if params.shiftingType else []) + ["OUT_OF_DOMAIN"]
    main = [("plain_fp64", abi.SOLVER_PLAIN_FP64, abi.WARM_PREVIOUS),
            ("plain_fp64_extrapolated", abi.SOLVER_PLAIN_FP64, abi.WARM_EXTRAP),
            ("plain_fp64_quadratic_extrapolated", abi.SOLVER_PLAIN_FP64, abi.WARM_EXTRAP2),
            ("fp32_fp64_refinement", abi.SOLVER_MIXED, abi.WARM_PREVIOUS),
            ("extrapolated_fp32_fp64", abi.SOLVER_MIXED, abi.WARM_EXTRAP),
            ("quadratic_extrapolated_fp32_fp64", abi.SOLVER_MIXED, abi.WARM_EXTRAP2)]
    if use_mlp:
        main.append(("learned_fp32_fp64", abi.SOLVER_MIXED, abi.WARM_MLP))
    # launch-form and inner-operator options: first sampled system only (best of three)
    alt = [("quadratic_fp32_fp64_staged_tiles", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 2),
           ("quadratic_fp32_fp64_pipelined", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 3),
           ("quadratic_compact_fp32_fp64", abi.SOLVER_MIXED_COMPACT, abi.WARM_EXTRAP2, 1),
           ("quadratic_matfree_fp32_fp64", abi.SOLVER_MIXED_MATFREE, abi.WARM_EXTRAP2, 1),
           ("plain_fp64_per_kernel_launch", abi.SOLVER_PLAIN_FP64, abi.WARM_PREVIOUS, 0),
           ("quadratic_fp32_fp64_per_kernel_launch", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 0)]
    samples = {k: [] for k, _, _ in main}
    trace = []
    alt_res = {}
    err = {k: 0.0 for k, _, _ in main}
    first = None
    for s in range(steps):
        for op in before:
            g.run_op(op)
        hist = _hist_get(g, abi)
        if s % every == 0:
            if first is None:
                first = s
            p_ref = None
            row = {"step": start + s}
            for name, solver, warm in main:
                r = _solve(g, abi, hist, solver, warm)
                samples[name].append(r)
                row[name] = round(r["ms"], 3)
                p = g.get(abi.F_PRESSPPE)
                if p_ref is None:
                    p_ref = p
                else:
                    err[name] = max(err[name], float(np.linalg.norm(p - p_ref) / np.linalg.norm(p_ref)))
            trace.append(row)
            if s == first:
                for name, solver, warm, mode in alt:
                    best = min((_solve(g, abi, hist, solver, warm, mode) for _ in range(3)), key=lambda r: r["ms"])
                    alt_res[name] = {k: (round(v, 3) if k == "ms" else v) for k, v in best.items()}
            g.set_ppe_launch(1)
        _hist_set(g, abi, hist)
        g.set_solver(*default)
        g.run_op("CALC_PRESS")
        for op in after:
            g.run_op(op)
    res = {}
    for name, _, _ in main:
        v = samples[name]
        res[name] = {"ms": round(float(np.mean([r["ms"] for r in v])), 3),
                     "iters": round(float(np.mean([r["iters"] for r in v])), 2),
                     "refinements": round(float(np.mean([r["refinements"] for r in v])), 2),
                     "relres0": float(np.mean([r["relres0"] for r in v])),
                     "relres_max": float(max(r["relres"] for r in v))}
        if name != "plain_fp64":
            res[name]["rel_err_vs_fp64_max"] = err[name]
    base = res["plain_fp64"]["ms"]
    for k in res:
        res[k]["speedup_vs_plain"] = round(base / res[k]["ms"], 3) if res[k]["ms"] > 0 else None
    for k, v in alt_res.items():
        v["speedup_vs_plain"] = round(samples["plain_fp64"][0]["ms"] / v["ms"], 3) if v["ms"] > 0 else None
    res["options_first_system"] = alt_res
    res["systems"] = len(samples["plain_fp64"])
    res["steps_sampled"] = "every %d-th step of steps %d-%d of the run" % (every, start, start + steps - 1)
    # the flow's phases differ: early systems are smooth in time (extrapolated starts gain
    # most), later ones carry particle-scale pressure noise
    half = len(trace) // 2
    for tag, part in (("first_half", trace[:half]), ("second_half", trace[half:])):
        if part:
            res[tag] = {k: round(float(np.mean([r[k] for r in part])), 3) for k in part[0] if k != "step"}
            res[tag]["steps"] = "%d-%d" % (part[0]["step"], part[-1]["step"])
    res["trace_ms"] = trace
    res["assemble_ms"] = round(g.last_stats().ppeAssembleMs, 3)
    return res


def cpu_baseline(case, steps):
    """The FP64 CPU oracle (a restatement of the reference path; the reference itself
    cannot be built here) on the host cores: a bounded sample of `steps` steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the checker / CPU baseline
    cores = os.cpu_count() or 1
    o = oracle.Oracle(case, threads=cores)
    o.set_solver(1e-8)
    o.initialize()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    o.close()
    out = {"value": round(case.n * steps / dt, 1), "unit": "particle-steps/s", "cores": cores, "kind": "port",
           "sample": "%d step(s) of the %d-particle workload after initialisation (%.1f s)" % (steps, case.n, dt)}
    # the same sample on one host thread
    o = oracle.Oracle(case, threads=1)
    o.set_solver(1e-8)
    o.initialize()
    t0 = time.perf_counter()
    o.step()
    d1 = time.perf_counter() - t0
    o.close()
    out["single_thread"] = {"value": round(case.n / d1, 1), "cores": 1,
                            "sample": "1 step of the %d-particle workload (%.1f s)" % (case.n, d1)}
    # the 2D particle-wall dam break (1,922 particles) run to its configured 200 steps
    from polymps_gb300 import cases
    c1 = cases.config(1)
    full = {}
    for th in (cores, 1):
        o = oracle.Oracle(c1, threads=th)
        o.set_solver(1e-8)
        o.initialize()
        t0 = time.perf_counter()
        for _ in range(c1.steps):
            o.step()
        d = time.perf_counter() - t0
        o.close()
        full["threads_%d" % th] = {"s": round(d, 3), "value": round(c1.n * c1.steps / d, 1)}
    out["full_run_2d_particle_walls"] = {"particles": c1.n, "steps": c1.steps, **full}
    # a fixed window of the 3D weakly compressible dam break (108,000 particles), all threads
    c2 = cases.config(2)
    o = oracle.Oracle(c2, threads=cores)
    o.set_solver(1e-8)
    o.initialize()
    t0 = time.perf_counter()
    for _ in range(5):
        o.step()
    d = time.perf_counter() - t0
    o.close()
    out["window_3d_weakly_compressible"] = {"particles": c2.n, "steps": 5, "s": round(d, 3),
                                            "value": round(c2.n * 5 / d, 1), "cores": cores}
    return out


def run_reference(a, rank, world):
    if rank != 0:
        return None
    from polymps_gb300 import cases
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    case = cases.config(a.config, scale=a.scale)
    cores = os.cpu_count() or 1
    o = oracle.Oracle(case, threads=cores)
    o.set_solver(1e-8)
    o.initialize()
    # W warm-up and up to K timed steps of the full workload, capped so the run stays within
    # a few minutes (each step of the 864k-particle case takes seconds on the host cores)
    budget = 150.0
    t0 = time.perf_counter()
    w = 0
    while w < a.warmup and time.perf_counter() - t0 < budget / 4:
        o.step()
        w += 1
    t0 = time.perf_counter()
    k = 0
    while k < a.steps and (k == 0 or time.perf_counter() - t0 < budget):
        o.step()
        k += 1
    dt = time.perf_counter() - t0
    v = case.n * k / dt
    return {"metric": METRIC, "value": round(v, 1), "unit": "particle-steps/s", "n_gpus": world, "steps": k,
            "warmup": w, "ms_per_step": round(dt / k * 1e3, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOADS[a.config], "particles": case.n,
                       "ppe_tol": 1e-8},
            "cpu_baseline": {"value": round(v, 1), "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": "%d timed step(s) after %d warm-up step(s)" % (k, w)},
            "e2e": {"value": round(v, 1), "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    a = args_()
    rank, world, local = dist()
    if a.impl == "reference":
        out = run_reference(a, rank, world)
    else:
        out = run_gb300(a, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
