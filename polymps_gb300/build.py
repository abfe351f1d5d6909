"""In-tree build of libmpsgpu.so (sm_103a) and the C++ host driver.

Each CUDA translation unit is compiled by nvcc in parallel for
``-gencode arch=compute_103a,code=sm_103a`` only; host C++ is compiled with
``-ffp-contract=off`` so derived constants are the IEEE results of the reference's
expressions on both x86_64 and aarch64.  Outputs go to ``polymps_gb300/_build``.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["mps_cells.cu", "mps_ops.cu", "mps_ops_df.cu", "mps_wall.cu", "mps_ppe.cu", "mps_mlp.cu", "mps_mlp_tc.cu",
      "mps_api.cu", "mps_static.cu"]
CPP = ["mps_host.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, ptxas_verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(PKG, "..", "include", "mpsgpu.h"))
    jobs = []
    objs = []
    for f in CU:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f.replace(".cu", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [nvcc, *GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-c", src, "-o", obj]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for f in CPP:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f.replace(".cpp", ".o"))
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c", src, "-o", obj])
    logs = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    lib = os.path.join(OUT, "libmpsgpu.so")
    if jobs or not os.path.exists(lib):
        _run([nvcc, *GENCODE, "-shared", "-o", lib] + objs + ["-Xcompiler", "-fPIC"])
    # host driver (JSON/.grid/.stl in, .vtu/.pvd out) linked against the library
    drv_src = [os.path.join(HOST, f) for f in ("mps_driver.cpp", "mps_io.cpp")
               if os.path.exists(os.path.join(HOST, f))]
    if len(drv_src) == 2:
        exe = os.path.join(OUT, "mps_gb300")
        if _stale(exe, drv_src + [os.path.join(HOST, "mps_io.h"), lib]):
            _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-o", exe] + drv_src +
                 ["-I" + os.path.join(PKG, "..", "include"), "-L" + OUT, "-lmpsgpu",
                  "-Wl,-rpath,$ORIGIN"])
    if verbose:
        sys.stdout.write("".join(logs))
    return lib


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)
    print("built", os.path.join(OUT, "libmpsgpu.so"))
