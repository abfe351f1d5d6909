"""bench.py's launch contract on the CPU: --gpus N starts N ranks, a world size that
disagrees with --gpus is refused, and the printed line stays short enough to be read back
whole."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BENCH = os.path.join(ROOT, "bench.py")


def _env():
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env["OMP_NUM_THREADS"] = "2"
    return env


def test_gpus_two_starts_two_ranks():
    """--gpus 2 without a torchrun environment re-launches itself as two ranks (the
    reference arm: rank 0 times the CPU path and prints the line, rank 1 exits)."""
    r = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0", "--scale", "4"], capture_output=True, text=True, timeout=900,
                       env=_env(), cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["impl"] == "reference"
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"]


def test_world_size_must_match_gpus():
    env = _env()
    env.update(WORLD_SIZE="2", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, BENCH, "--gpus", "3"], capture_output=True, text=True, timeout=300,
                       env=env, cwd=ROOT)
    assert r.returncode != 0
    assert "WORLD_SIZE=2" in r.stderr


def test_printed_line_is_short():
    sys.path.insert(0, ROOT)
    import bench
    ppe = {"systems": 37, "steps": "every 27-th of steps 28-999", "plain_fp64_ms": 3.123, "plain_fp64_iters": 26.31,
           "speedup_vs_plain": {"quadratic_extrapolated_fp32_fp64": 1.723, "learned_fp32_fp64": 1.512,
                                "fp32_fp64_refinement": 1.456, "extrapolated_fp32_fp64": 1.702},
           "max_rel_err_vs_plain": 1.234e-08,
           "early": {"systems": 40, "plain_fp64_ms": 2.881,
                     "speedup_vs_plain": {"quadratic_extrapolated_fp32_fp64": 2.251, "learned_fp32_fp64": 1.781,
                                          "fp32_fp64_refinement": 1.601, "extrapolated_fp32_fp64": 2.013}}}
    out = {"metric": "particle-steps/s", "value": 173456789.1, "unit": "particle-steps/s", "n_gpus": 1, "steps": 100,
           "warmup": 5, "ms_per_step": 4.987, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "df32+f32/f64 PPE", "data": "synthetic",
           "config": {"workload": bench.WORKLOADS[3], "particles": 864000, "l0": 0.005, "ppe_tol": 1e-8,
                      "solver": "mixed", "precision": "df32", "warm_start": "quadratic", "parallelism": "single",
                      "l2": "working set > L2, no flush"},
           "e2e": {"value": 141234567.8, "unit": "particle-steps/s", "h2d_bytes_per_step": 55296000,
                   "d2h_bytes_per_step": 55296000},
           "value_fp64": {"value": 45712345.6, "ms_per_step": 18.901, "steps": 100},
           "roofline": {"bound": "hbm", "kernel": "PPE_SOLVE", "achieved": 4871.2, "peak": 6785.5, "unit": "GB/s",
                        "frac": 0.7179, "peak_source": "measured", "traffic": None, "algo_bytes": 6480000000,
                        "launch_ms": 1.3301, "share": 0.267},
           "clocks": {"sm_mhz": 1995.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 53},
           "gpu_launches": 12345, "ppe": ppe,
           "cpu_baseline": {"value": 450097.9, "unit": "particle-steps/s", "cores": 16, "kind": "port",
                            "sample": "1 step(s) of the 864000-particle workload after initialisation (1.9 s)",
                            "single_thread": 127523.6},
           "detail": "bench_detail.json"}
    s = bench.compact(out)
    assert len(s) <= bench.LINE_MAX
    d = json.loads(s)
    for k in ("value", "e2e", "roofline", "cpu_baseline", "clocks", "value_fp64", "ppe"):
        assert d[k] is not None
