"""Benchmark of the PolyMPS per-step particle path on GB300.

Workload: the 3D incompressible polygon dam break (tank 1.61 x 0.6 x 0.6 m, 12-triangle
closed box, fluid block 0.6 x 0.6 x 0.3 m at l0 = 0.005 m: 864,000 particles,
dt = 2.5e-4 s, PPE to relative residual 1e-8), synthetic lattice input (the reference's
.grid files are not available).  A step is one mainLoopOfSimulation iteration.

Metric: particle-steps/s (whole job), plus the PPE time-to-1e-8 of the plain FP64 CG,
the FP32/FP64 refinement solver and the learned warm start on the same systems.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The last stdout line is one JSON object of about 1.5 KB at most; the per-system PPE
traces, the per-class profile and the longer CPU baseline go to the --detail file.

Multi-GPU: the path is run as N independent replicas (one per rank, no collective on
the data path); value = sum of particle-steps over ranks / max time over ranks.  With
--gpus N > 1 and no torchrun environment, bench.py starts the N ranks itself (torchrun
on 127.0.0.1, one GPU per rank).
"""
import argparse
import json
import os
import socket
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s"
WORKLOADS = {2: "3D WC polygon dam break, 108k (cfg2)",
             3: "3D INC polygon dam break, 864k (cfg3)",
             5: "3D INC dam break + obstacle, collision, shifting, 9.4M (cfg5)"}
HBM_FALLBACK = 6800.0
LINE_MAX = 1500
# DRAM bytes (read + write) of the single-launch mixed PPE solve per inner-iteration
# equivalent, from one ncu capture of the 20 timed solves of the 864k workload
# (3.634e9 B per launch at 18 inner iterations and 1 refinement: the setup and each
# refinement's FP64 passes counted as two inner iterations each; k_mx_own_cfg3-864k.md)
MX_TRAFFIC_PER_ITER = 3.634e9 / (18 + 2 * 2)


def args_(argv=None):
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
    a.add_argument("--e2e-steps", type=int, default=10)
    a.add_argument("--fp64-steps", type=int, default=0,
                   help="timed steps of the FP64 drop-in tier (0: as --steps; -1: not timed)")
    a.add_argument("--no-cpu-baseline", action="store_true")
    a.add_argument("--cpu-steps", type=int, default=1)
    a.add_argument("--ppe-compare", type=int, default=1)
    a.add_argument("--ppe-steps", type=int, default=0,
                   help="steps the PPE comparison runs on (0: to the workload's configured length)")
    a.add_argument("--ppe-options", action="store_true",
                   help="also time the measured-and-rejected launch forms and inner operators")
    a.add_argument("--detail", default=os.path.join(ROOT, "bench_detail.json"),
                   help="file for the per-system PPE traces, the per-class profile and the long CPU baseline")
    a.add_argument("--mlp", default=os.path.join(ROOT, "polymps_gb300", "mlp_warmstart.npz"),
                   help="weights of the learned warm start (npz with params, norm)")
    a.add_argument("--presort", action="store_true",
                   help="number the input particles in bucket order (input renumbering only)")
    return a.parse_args(argv)


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def launch_ranks(n, argv):
    """Re-run this script as n ranks under torchrun on this node (127.0.0.1); returns the
    launcher's exit status.  Rank 0 prints the line."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.abspath(__file__)] + argv
    return subprocess.call(cmd)


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
                                          "--format=csv,noheader,nounits", "-lms", "20"],
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
def algo_bytes(cls, N, E, Z, mixed, df, st=None, matfree=False, compact=False, own=False):
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
        if mixed and own:
            # block-owned rows (x_f, r_f, p, Ap in shared memory): inner iteration = SpMV
            # (valf + col per entry; z, diag, len per row) + update (M^-1 read, z written);
            # per refinement: FP64 residual (val + col per entry; b, x, r, diag, len per row),
            # x update (x read and written), inner start (r, M^-1 read, z written)
            return it * (20 * N + 8 * Z) + (rf + 1) * (68 * N + 12 * Z)
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


def owned_rows(n, sms=152):
    """Whether the mixed solve keeps its vectors in shared memory (the library's rule: the
    grid-stride rounds of a 1024-thread block per SM fit its 13,312 row slots)."""
    return (n // (sms * 1024) + 1) * 1024 <= 13312


def _timed_run(g, steps, world, rank, clocks=None):
    """K steps bracketed by a barrier and a device synchronise on both sides; returns
    (stats, wall seconds, launches)."""
    import torch
    from polymps_gb300 import mps, replicas
    torch.cuda.synchronize()
    replicas.barrier(world)
    if clocks:
        clocks.start()
    l0 = mps.MpsGpu.launch_count()
    t0 = time.perf_counter()
    st = g.run(steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    launches = mps.MpsGpu.launch_count() - l0
    replicas.barrier(world)
    return st, wall, launches


def run_gb300(a, rank, world, local):
    import torch
    from polymps_gb300 import abi, build, cases, mps, replicas
    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device visible (the GB300 path has no CPU fallback)")
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist_
        dist_.init_process_group("nccl", device_id=torch.device("cuda", local))
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
    mlp_path = a.mlp
    have_mlp = os.path.exists(mlp_path)
    prec = abi.PRECISION_DF32 if a.precision == "df32" else abi.PRECISION_FP64
    warm = {"prev": abi.WARM_PREVIOUS, "extrap": abi.WARM_EXTRAP, "mlp": abi.WARM_MLP}.get(a.warm, abi.WARM_EXTRAP2)

    def handle(precision, solver_, warm_):
        g = mps.MpsGpu(case, solver=solver_, tol=1e-8, max_iter=20000, precision=precision)
        if have_mlp:
            w = np.load(mlp_path)
            g.mlp_set_weights(w["params"], w["norm"])
        g.set_solver(solver_, warm_, 1e-8, 20000)
        g.initialize()
        return g

    g = handle(prec, solver, warm)
    g.run(a.warmup)
    # clocks are sampled from the start of the timed run to the end of the FP64 tier's
    # timed run (both timed regions; the end-to-end steps lie between them)
    clocks = Clocks(local)
    g.profile(True)
    st, wall, launches = _timed_run(g, a.steps, world, rank, clocks)
    prof = g.profile_get()
    g.profile(False)
    # replicas: particle-steps of all ranks over the slowest rank's device time
    units, dev_s = replicas.aggregate(N * a.steps, st.stepMs / 1e3, world, device="cuda")
    value = units / dev_s

    # e2e through the C ABI with host arrays: the state of the end of the timed run is
    # uploaded every step from page-locked host arrays, stepped, and read back into them
    def pinned_like(x):
        t = torch.empty(x.size, dtype=torch.float64).pin_memory()
        v = t.numpy().reshape(x.shape)
        v[...] = x
        return v, t
    host, keep = {}, []
    for f in (abi.F_POS, abi.F_VEL, abi.F_PRESS, abi.F_PRESSPPE):
        v, t = pinned_like(g.get(f))
        host[f] = v
        keep.append(t)
    h2d = sum(v.nbytes for v in host.values())
    d2h = h2d   # the step's state comes back: positions, velocities, pressure and the unclamped solution
    torch.cuda.synchronize()
    replicas.barrier(world)
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        for f, v in host.items():
            g.set(f, v)
        g.step()
        for f in host:
            g.get(f, out=host[f])
    e2e_s = time.perf_counter() - t0
    e2e_units, e2e_s = replicas.aggregate(N * a.e2e_steps, e2e_s, world, device="cuda")
    e2e = e2e_units / e2e_s

    # dominant class of the per-class profile and its roofline
    hbm, hbm_src = peaks()
    E, Z = st.nbrEntries, max(st.ppeNnz - N, 0)
    mixed = solver != abi.SOLVER_PLAIN_FP64
    leaf = {k: v for k, v in prof.items() if k not in ("CALC_PRESS",)}
    dom = max(leaf, key=lambda k: leaf[k][0]) if leaf else None
    roof = None
    if dom:
        ms, calls = leaf[dom]
        b = algo_bytes(dom, N, E, Z, mixed, prec == abi.PRECISION_DF32, st, solver == abi.SOLVER_MIXED_MATFREE,
                       solver == abi.SOLVER_MIXED_COMPACT, own=owned_rows(N))
        if b:
            ach = b / (ms / calls / 1e3) / 1e9
            traffic = None
            if dom == "PPE_SOLVE" and mixed and solver == abi.SOLVER_MIXED and owned_rows(N) and st.runPpeSolves:
                it = st.runPpeIterations / st.runPpeSolves
                rf = st.runPpeRefinements / st.runPpeSolves
                traffic = int(MX_TRAFFIC_PER_ITER * (it + 2 * (rf + 1)) * N / 864000)
            roof = {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(ach / hbm, 4), "peak_source": hbm_src, "traffic": traffic,
                    "algo_bytes": int(b), "launch_ms": round(ms / calls, 4),
                    "share": round(ms / st.stepMs, 3)}
    iters = st.runPpeIterations / max(st.runPpeSolves, 1)
    detail = {"profile_ms": {k: [round(v[0], 3), v[1]] for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
              "timed_run": {"wall_s": round(wall, 3), "ppe_iters_per_solve": round(iters, 2),
                            "ppe_refinements_per_solve": round(st.runPpeRefinements / max(st.runPpeSolves, 1), 2),
                            "last_relres": st.ppeRelResidual, "velMax": st.velMax}}

    # the FP64 drop-in tier (every pair in FP64, plain FP64 PPE from the previous solution)
    # on the same workload
    ppe_done = a.warmup + a.steps + a.e2e_steps
    fp64 = None
    if not (a.precision == "fp64" and a.solver == "plain") and a.fp64_steps >= 0:
        g64 = handle(abi.PRECISION_FP64, abi.SOLVER_PLAIN_FP64, abi.WARM_PREVIOUS)
        g64.run(max(3, min(a.warmup, 5)))
        k64 = a.fp64_steps or a.steps
        st64, _, _ = _timed_run(g64, k64, world, rank)
        u64, s64 = replicas.aggregate(N * k64, st64.stepMs / 1e3, world, device="cuda")
        fp64 = {"value": round(u64 / s64, 1), "ms_per_step": round(st64.stepMs / k64, 3), "steps": k64}
        g64.close()
    clk = clocks.stop()

    # PPE time-to-1e-8 on identical systems along the rest of the run
    ppe = ppe_early = None
    if a.ppe_compare and rank == 0 and case.params.get("mpsType", 2) == 2:
        steps = a.ppe_steps if a.ppe_steps > 0 else max(getattr(case, "steps", 1000) - ppe_done, 40)
        ppe = ppe_compare(g, abi, have_mlp, g.params, (solver, warm, 1e-8, 20000), steps=steps,
                          every=max(1, steps // 36), start=ppe_done, options=a.ppe_options)
    g.close()
    # the smooth start of the flow (steps 7-86, every second system) on a fresh simulation:
    # extrapolated and learned starts gain most there
    if a.ppe_compare and rank == 0 and a.ppe_steps == 0 and case.params.get("mpsType", 2) == 2:
        g2 = handle(prec, solver, warm)
        g2.run(6)
        ppe_early = ppe_compare(g2, abi, have_mlp, g2.params, (solver, warm, 1e-8, 20000), steps=80, every=2,
                                start=7)
        g2.close()
    cpu = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu, cpu_more = cpu_baseline(case, a.cpu_steps)
        detail["cpu_baseline_more"] = cpu_more
    if world > 1:
        torch.distributed.destroy_process_group()

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "particle-steps/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(st.stepMs / a.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("df32" if prec == abi.PRECISION_DF32 else "f64") + ("+f32/f64 PPE" if mixed else "+f64 PPE"),
        "data": "synthetic",
        "config": {"workload": WORKLOADS[a.config], "particles": N, "l0": case.params["partDist"],
                   "ppe_tol": 1e-8, "solver": a.solver, "precision": a.precision,
                   "warm_start": {abi.WARM_MLP: "learned", abi.WARM_EXTRAP: "linear", abi.WARM_EXTRAP2: "quadratic",
                                  abi.WARM_PREVIOUS: "previous"}[warm],
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "working set > L2, no flush"},
        "e2e": {"value": round(e2e, 1), "unit": "particle-steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "value_fp64": fp64,
        "roofline": roof,
        "clocks": clk,
        "gpu_launches": int(launches),
        "ppe": _ppe_summary(ppe, ppe_early),
        "cpu_baseline": cpu,
    }
    if rank == 0:
        detail.update({"line": out, "ppe": ppe, "ppe_early": ppe_early})
        try:
            with open(a.detail, "w") as f:
                json.dump(detail, f, indent=1)
            out["detail"] = os.path.relpath(a.detail, ROOT)
        except OSError:
            pass
    return out


def _ppe_summary(ppe, early):
    """Mean PPE time-to-1e-8 of the plain FP64 CG (previous-step start) and each FP32/FP64
    refinement variant's speed-up over it, by warm start: quadratic or linear
    extrapolation, learned, previous step."""
    if not ppe:
        return None
    keep = {"quadratic": "quadratic_extrapolated_fp32_fp64", "learned": "learned_fp32_fp64",
            "previous": "fp32_fp64_refinement", "linear": "extrapolated_fp32_fp64"}
    def sp(x):   # the printed line carries speed-ups to 2 decimals (3 in the detail file)
        return None if x is None else round(x, 2)
    s = {"systems": ppe["systems"], "steps": ppe["steps_sampled"], "plain_fp64_ms": round(ppe["plain_fp64"]["ms"], 2),
         "plain_fp64_iters": ppe["plain_fp64"]["iters"],
         "speedup_vs_plain": {k: sp(ppe[v]["speedup_vs_plain"]) for k, v in keep.items() if v in ppe},
         "max_rel_err_vs_plain": float("%.2g" % max(ppe[v].get("rel_err_vs_fp64_max", 0.0) for v in keep.values()
                                                    if v in ppe))}
    if early:
        s["early"] = {"systems": early["systems"], "steps": early["steps_sampled"],
                      "plain_fp64_ms": round(early["plain_fp64"]["ms"], 2),
                      "speedup_vs_plain": {k: sp(early[v]["speedup_vs_plain"]) for k, v in keep.items() if v in early}}
    return s


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


def ppe_compare(g, abi, use_mlp, params, default, steps=40, every=4, start=0, options=False):
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
            ("fp32_fp64_refinement", abi.SOLVER_MIXED, abi.WARM_PREVIOUS),
            ("extrapolated_fp32_fp64", abi.SOLVER_MIXED, abi.WARM_EXTRAP),
            ("quadratic_extrapolated_fp32_fp64", abi.SOLVER_MIXED, abi.WARM_EXTRAP2)]
    if use_mlp:
        main.append(("learned_fp32_fp64", abi.SOLVER_MIXED, abi.WARM_MLP))
    # launch-form and inner-operator options (measured and not the default): first sampled
    # system only (best of three), with --ppe-options
    alt = [("quadratic_fp32_fp64_grid_stride", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 4),
           ("plain_fp64_extrapolated", abi.SOLVER_PLAIN_FP64, abi.WARM_EXTRAP, 1),
           ("plain_fp64_quadratic_extrapolated", abi.SOLVER_PLAIN_FP64, abi.WARM_EXTRAP2, 1),
           ("quadratic_fp32_fp64_staged_tiles", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 2),
           ("quadratic_fp32_fp64_pipelined", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 3),
           ("quadratic_compact_fp32_fp64", abi.SOLVER_MIXED_COMPACT, abi.WARM_EXTRAP2, 1),
           ("quadratic_matfree_fp32_fp64", abi.SOLVER_MIXED_MATFREE, abi.WARM_EXTRAP2, 1),
           ("plain_fp64_per_kernel_launch", abi.SOLVER_PLAIN_FP64, abi.WARM_PREVIOUS, 0),
           ("quadratic_fp32_fp64_per_kernel_launch", abi.SOLVER_MIXED, abi.WARM_EXTRAP2, 0)] if options else []
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
    if alt_res:
        res["options_first_system"] = alt_res
    res["systems"] = len(samples["plain_fp64"])
    res["steps_sampled"] = "%d-%d every %d" % (start, start + steps - 1, every)
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


def _oracle_steps(case, threads, steps, tol=1e-8):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the checker / CPU baseline
    o = oracle.Oracle(case, threads=threads)
    o.set_solver(tol)
    o.initialize()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    o.close()
    return dt


def cpu_baseline(case, steps):
    """The FP64 CPU oracle (a restatement of the reference path; the reference itself
    cannot be built here) on the host cores: a bounded sample of `steps` steps of the same
    workload on all cores, and one step on one core.  Returns (line entry, longer record)."""
    from polymps_gb300 import cases
    cores = os.cpu_count() or 1
    dt = _oracle_steps(case, cores, steps)
    d1 = _oracle_steps(case, 1, 1)
    out = {"value": round(case.n * steps / dt, 1), "unit": "particle-steps/s", "cores": cores, "kind": "port",
           "sample": "%d step(s) of this workload (%.1f s)" % (steps, dt),
           "single_thread": round(case.n / d1, 1)}
    more = {"single_thread_sample": "1 step (%.1f s)" % d1}
    # the 2D particle-wall dam break run to its configured 200 steps, and a window of the
    # 3D weakly compressible dam break (108,000 particles)
    c1 = cases.config(1)
    more["full_run_2d_particle_walls"] = {"particles": c1.n, "steps": c1.steps}
    for th in (cores, 1):
        d = _oracle_steps(c1, th, c1.steps)
        more["full_run_2d_particle_walls"]["threads_%d" % th] = {"s": round(d, 3),
                                                                 "value": round(c1.n * c1.steps / d, 1)}
    c2 = cases.config(2)
    d = _oracle_steps(c2, cores, 5)
    more["window_3d_weakly_compressible"] = {"particles": c2.n, "steps": 5, "s": round(d, 3),
                                             "value": round(c2.n * 5 / d, 1), "cores": cores}
    return out, more


def run_reference(a, rank, world):
    """The reference arm: the reference's own CPU implementation of the path cannot be
    built here (its Eigen, libigl and nlohmann/json submodules are empty), so its FP64
    restatement (the oracle port) is timed on all host cores, rank 0 only."""
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
            "config": {"workload": WORKLOADS[a.config], "particles": case.n, "ppe_tol": 1e-8},
            "cpu_baseline": {"value": round(v, 1), "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": "%d timed step(s) after %d warm-up step(s)" % (k, w)},
            "e2e": {"value": round(v, 1), "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def compact(out):
    """The printed line: drop optional detail until it fits in LINE_MAX bytes."""
    s = json.dumps(out, separators=(",", ":"))
    for key in (("ppe", "early"), ("clocks", "samples"), ("cpu_baseline", "sample"), ("roofline", "peak_source")):
        if len(s) <= LINE_MAX:
            break
        d = out.get(key[0])
        if isinstance(d, dict):
            d.pop(key[1], None)
        s = json.dumps(out, separators=(",", ":"))
    return s


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    a = args_(argv)
    rank, world, local = dist()
    if "WORLD_SIZE" not in os.environ and a.gpus > 1:
        sys.exit(launch_ranks(a.gpus, argv))
    if "WORLD_SIZE" in os.environ and world != a.gpus:
        sys.exit("bench.py: --gpus %d but WORLD_SIZE=%d: launch one rank per GPU (torchrun --nproc-per-node %d)"
                 % (a.gpus, world, a.gpus))
    if a.impl == "reference":
        out = run_reference(a, rank, world)
    else:
        out = run_gb300(a, rank, world, local)
    if rank == 0 and out is not None:
        print(compact(out), flush=True)


if __name__ == "__main__":
    main()
