"""Python host mirror of PolyMPS's stepping interface over libmpsgpu.so (ctypes).

The reference drives its operators as ``Class::method(MpsParticleSystem*, MpsParticle*,
MpsBucket*)`` calls from ``mainLoopOfSimulation`` (src/main.cpp:221-469); ``MpsGpu``
exposes the same operators (``run_op``), the whole step (``step``), the step-0 sequence
(``initialize``) and field access in the reference's array layout.  There is no CPU
path: if the CUDA library is missing or no GPU is visible, construction raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_lib = None

EXPORTS = [
    "mpsgpu_params_derive", "mpsgpu_create", "mpsgpu_destroy", "mpsgpu_initialize", "mpsgpu_step",
    "mpsgpu_run", "mpsgpu_run_op", "mpsgpu_set_solver", "mpsgpu_set_precision", "mpsgpu_set_ppe_launch", "mpsgpu_get_field", "mpsgpu_set_field",
    "mpsgpu_num_particles", "mpsgpu_time", "mpsgpu_get_neighbors", "mpsgpu_get_ppe",
    "mpsgpu_mlp_set_weights", "mpsgpu_mlp_get_weights", "mpsgpu_ppe_features", "mpsgpu_mlp_record",
    "mpsgpu_mlp_num_records", "mpsgpu_mlp_fit_normalization", "mpsgpu_mlp_train", "mpsgpu_mlp_forward",
    "mpsgpu_mlp_gradient", "mpsgpu_stream", "mpsgpu_last_error", "mpsgpu_abi_sizes",
    "mpsgpu_profile", "mpsgpu_profile_get", "mpsgpu_profile_name", "mpsgpu_launch_count",
    "mpsgpu_last_stats", "mpsgpu_pcg_solve_static", "mpsgpu_pcg_static_error", "mpsgpu_write_vtu",
    "mpsgpu_check_params",
]
PROF_NCLASS = len(abi.OPS) + 6


class MpsError(RuntimeError):
    def __init__(self, where, code, msg=""):
        super().__init__("%s failed with status %d%s" % (where, code, (": " + msg) if msg else ""))
        self.code = code


def lib(path=None):
    """Load libmpsgpu.so (built in-tree by polymps_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or abi.LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libmpsgpu.so not built (%s): run polymps_gb300.build.build()" % path)
    L = C.CDLL(path)
    vp, P = C.c_void_p, C.POINTER
    L.mpsgpu_params_derive.argtypes = [P(abi.MpsParams), C.c_int, P(C.c_double)]
    L.mpsgpu_check_params.argtypes = [P(abi.MpsParams)]
    L.mpsgpu_create.argtypes = [P(abi.MpsParams), C.c_int, P(C.c_int), P(C.c_double), P(C.c_double),
                                P(C.c_double), P(abi.MpsMesh), P(vp)]
    for f in ("mpsgpu_destroy", "mpsgpu_initialize", "mpsgpu_mlp_fit_normalization"):
        getattr(L, f).argtypes = [vp]
    L.mpsgpu_step.argtypes = [vp, P(abi.MpsStepStats)]
    L.mpsgpu_run.argtypes = [vp, C.c_int, P(abi.MpsStepStats)]
    L.mpsgpu_run_op.argtypes = [vp, C.c_int]
    L.mpsgpu_set_solver.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_int]
    L.mpsgpu_set_precision.argtypes = [vp, C.c_int]
    L.mpsgpu_set_ppe_launch.argtypes = [vp, C.c_int]
    L.mpsgpu_write_vtu.argtypes = [vp, C.c_char_p, C.c_uint]
    L.mpsgpu_get_field.argtypes = [vp, C.c_int, vp]
    L.mpsgpu_set_field.argtypes = [vp, C.c_int, vp]
    L.mpsgpu_num_particles.argtypes = [vp, P(C.c_int)]
    L.mpsgpu_time.argtypes = [vp, P(C.c_double), P(C.c_int)]
    L.mpsgpu_get_neighbors.argtypes = [vp, P(C.c_int), P(C.c_int), C.c_longlong]
    L.mpsgpu_get_ppe.argtypes = [vp, P(C.c_longlong), P(C.c_longlong), P(C.c_int), P(C.c_double), P(C.c_double)]
    L.mpsgpu_mlp_set_weights.argtypes = [vp, P(C.c_float), P(C.c_float)]
    L.mpsgpu_mlp_get_weights.argtypes = [vp, P(C.c_float), P(C.c_float)]
    L.mpsgpu_ppe_features.argtypes = [vp, P(C.c_float)]
    L.mpsgpu_mlp_record.argtypes = [vp, C.c_int]
    L.mpsgpu_mlp_num_records.argtypes = [vp, P(C.c_longlong)]
    L.mpsgpu_mlp_train.argtypes = [vp, C.c_int, C.c_int, C.c_float, C.c_ulonglong, P(C.c_float)]
    L.mpsgpu_mlp_forward.argtypes = [vp, P(C.c_float), C.c_int, P(C.c_float)]
    L.mpsgpu_mlp_gradient.argtypes = [vp, P(C.c_float), P(C.c_float), C.c_int, P(C.c_float), P(C.c_float)]
    L.mpsgpu_stream.argtypes = [vp, P(vp)]
    L.mpsgpu_last_error.argtypes = [vp]
    L.mpsgpu_last_error.restype = C.c_char_p
    L.mpsgpu_abi_sizes.argtypes = [P(C.c_int)] * 3
    L.mpsgpu_profile.argtypes = [vp, C.c_int]
    L.mpsgpu_profile_get.argtypes = [vp, C.c_int, P(C.c_double), P(C.c_longlong)]
    L.mpsgpu_profile_name.argtypes = [C.c_int]
    L.mpsgpu_profile_name.restype = C.c_char_p
    L.mpsgpu_launch_count.argtypes = [P(C.c_longlong)]
    L.mpsgpu_last_stats.argtypes = [vp, P(abi.MpsStepStats)]
    L.mpsgpu_pcg_solve_static.argtypes = [C.c_int, vp, vp, vp, vp, vp, C.c_double, C.c_int, vp,
                                          P(C.c_int), P(C.c_double)]
    L.mpsgpu_pcg_static_error.restype = C.c_char_p
    _lib = L
    return L


def _check(where, code, h=None):
    if code:
        msg = lib().mpsgpu_last_error(h).decode(errors="replace") if _lib is not None else ""
        raise MpsError(where, code, msg)


def derive(params, n, pos):
    """MpsParticle::setParameters + MpsBucket::allocateMemory on a copy of params."""
    p = abi.MpsParams.from_buffer_copy(params)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    _check("mpsgpu_params_derive", lib().mpsgpu_params_derive(C.byref(p), int(n), abi.dptr(pos)))
    return p


class MpsGpu:
    """One particle system on the GPU (one handle, one CUDA stream)."""

    def __init__(self, case, solver=abi.SOLVER_PLAIN_FP64, warm=abi.WARM_PREVIOUS, tol=1e-8, max_iter=0,
                 precision=abi.PRECISION_FP64):
        L = lib()
        self.case = case
        self.params = derive(case.mps_params(), case.n, case.pos)
        self._mesh, self._tri = abi.make_mesh(case.mesh)
        h = C.c_void_p()
        _check("mpsgpu_create", L.mpsgpu_create(
            C.byref(self.params), case.n, abi.iptr(case.type), abi.dptr(case.pos), abi.dptr(case.vel),
            abi.dptr(case.press), C.byref(self._mesh) if self._mesh is not None else None, C.byref(h)))
        self.h = h
        self.set_solver(solver, warm, tol, max_iter)
        self.set_precision(precision)

    # ------------------------------------------------------------- lifecycle
    def close(self):
        if getattr(self, "h", None):
            lib().mpsgpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------- stepping
    def initialize(self):
        _check("mpsgpu_initialize", lib().mpsgpu_initialize(self.h), self.h)

    def step(self):
        st = abi.MpsStepStats()
        _check("mpsgpu_step", lib().mpsgpu_step(self.h, C.byref(st)), self.h)
        return st

    def run(self, nsteps):
        st = abi.MpsStepStats()
        _check("mpsgpu_run", lib().mpsgpu_run(self.h, int(nsteps), C.byref(st)), self.h)
        return st

    def run_op(self, op):
        if isinstance(op, str):
            op = abi.OP[op]
        _check("mpsgpu_run_op(%s)" % abi.OPS[op], lib().mpsgpu_run_op(self.h, op), self.h)

    def last_stats(self):
        st = abi.MpsStepStats()
        _check("mpsgpu_last_stats", lib().mpsgpu_last_stats(self.h, C.byref(st)), self.h)
        return st

    def set_precision(self, precision=abi.PRECISION_FP64):
        """FP64 (reference arithmetic) or DF32 (float-float pair arithmetic, same decisions)."""
        _check("mpsgpu_set_precision", lib().mpsgpu_set_precision(self.h, precision), self.h)

    def set_ppe_launch(self, mode=1):
        """PPE launch: 0 one launch per kernel, 1 (default) one cooperative launch per solve
        (block-owned rows, inner-CG vectors in shared memory), 2 as 1 with the FP32 matrix
        streamed through shared memory by bulk copies, 3 as 1 with the pipelined inner CG,
        4 as 1 with grid-stride rows and the vectors in global memory."""
        _check("mpsgpu_set_ppe_launch", lib().mpsgpu_set_ppe_launch(self.h, int(mode)), self.h)

    def write_vtu(self, path, groups=0):
        """Binary .vtu of the current state (abi.VTU_* optional array groups)."""
        _check("mpsgpu_write_vtu", lib().mpsgpu_write_vtu(self.h, str(path).encode(), int(groups)), self.h)

    def set_solver(self, solver=abi.SOLVER_PLAIN_FP64, warm=abi.WARM_PREVIOUS, tol=1e-8, max_iter=0):
        _check("mpsgpu_set_solver", lib().mpsgpu_set_solver(self.h, solver, warm, tol, max_iter), self.h)

    # ------------------------------------------------------------- state
    @property
    def n(self):
        v = C.c_int()
        _check("mpsgpu_num_particles", lib().mpsgpu_num_particles(self.h, C.byref(v)), self.h)
        return v.value

    def time(self):
        t, it = C.c_double(), C.c_int()
        lib().mpsgpu_time(self.h, C.byref(t), C.byref(it))
        return t.value, it.value

    def get(self, field, out=None):
        """Field in the reference's host layout; out: a preallocated (e.g. page-locked) array."""
        buf = abi.field_buffer(field, self.n) if out is None else out
        _check("mpsgpu_get_field", lib().mpsgpu_get_field(self.h, field, buf.ctypes.data), self.h)
        return buf

    def set(self, field, arr):
        shape, dtype = abi.field_spec(field, self.n)
        arr = np.ascontiguousarray(arr, dtype=dtype).reshape(shape)   # no copy for a matching array
        _check("mpsgpu_set_field", lib().mpsgpu_set_field(self.h, field, arr.ctypes.data), self.h)

    def neighbors(self):
        n = self.n
        counts = np.zeros(n, dtype=np.int32)
        _check("mpsgpu_get_neighbors", lib().mpsgpu_get_neighbors(self.h, abi.iptr(counts), None, 0), self.h)
        tot = int(counts.sum())
        nbr = np.zeros(max(tot, 1), dtype=np.int32)
        _check("mpsgpu_get_neighbors",
               lib().mpsgpu_get_neighbors(self.h, abi.iptr(counts), abi.iptr(nbr), tot), self.h)
        return counts, nbr[:tot]

    def ppe(self):
        nnz = C.c_longlong()
        _check("mpsgpu_get_ppe", lib().mpsgpu_get_ppe(self.h, C.byref(nnz), None, None, None, None), self.h)
        n = self.n
        rowptr = np.zeros(n + 1, dtype=np.int64)
        col = np.zeros(max(nnz.value, 1), dtype=np.int32)
        val = np.zeros(max(nnz.value, 1), dtype=np.float64)
        rhs = np.zeros(n, dtype=np.float64)
        _check("mpsgpu_get_ppe", lib().mpsgpu_get_ppe(
            self.h, C.byref(nnz), rowptr.ctypes.data_as(C.POINTER(C.c_longlong)), abi.iptr(col),
            abi.dptr(val), abi.dptr(rhs)), self.h)
        return rowptr, col[:nnz.value], val[:nnz.value], rhs

    # ------------------------------------------------------------- timing
    def profile(self, enable=True):
        _check("mpsgpu_profile", lib().mpsgpu_profile(self.h, int(bool(enable))), self.h)

    def profile_get(self):
        """{class name: (device ms, calls)} accumulated since profiling was enabled."""
        out = {}
        for k in range(PROF_NCLASS):
            ms, calls = C.c_double(), C.c_longlong()
            lib().mpsgpu_profile_get(self.h, k, C.byref(ms), C.byref(calls))
            if calls.value:
                out[lib().mpsgpu_profile_name(k).decode()] = (ms.value, calls.value)
        return out

    @staticmethod
    def launch_count():
        v = C.c_longlong()
        lib().mpsgpu_launch_count(C.byref(v))
        return v.value

    # ------------------------------------------------------------- learned warm start
    def mlp_set_weights(self, params, norm):
        params = np.ascontiguousarray(params, dtype=np.float32)
        norm = np.ascontiguousarray(norm, dtype=np.float32)
        assert params.size == abi.MLP_NPARAM and norm.size == abi.MLP_NNORM
        _check("mpsgpu_mlp_set_weights", lib().mpsgpu_mlp_set_weights(self.h, abi.fptr(params), abi.fptr(norm)), self.h)

    def mlp_get_weights(self):
        params = np.zeros(abi.MLP_NPARAM, dtype=np.float32)
        norm = np.zeros(abi.MLP_NNORM, dtype=np.float32)
        _check("mpsgpu_mlp_get_weights", lib().mpsgpu_mlp_get_weights(self.h, abi.fptr(params), abi.fptr(norm)), self.h)
        return params, norm

    def ppe_features(self):
        f = np.zeros((self.n, abi.MLP_NFEAT), dtype=np.float32)
        _check("mpsgpu_ppe_features", lib().mpsgpu_ppe_features(self.h, abi.fptr(f)), self.h)
        return f

    def mlp_record(self, enable=True):
        _check("mpsgpu_mlp_record", lib().mpsgpu_mlp_record(self.h, int(bool(enable))), self.h)

    def mlp_num_records(self):
        v = C.c_longlong()
        lib().mpsgpu_mlp_num_records(self.h, C.byref(v))
        return v.value

    def mlp_fit_normalization(self):
        _check("mpsgpu_mlp_fit_normalization", lib().mpsgpu_mlp_fit_normalization(self.h), self.h)

    def mlp_train(self, iters, batch=8192, lr=1e-3, seed=1):
        loss = np.zeros(iters, dtype=np.float32)
        _check("mpsgpu_mlp_train", lib().mpsgpu_mlp_train(self.h, int(iters), int(batch), float(lr), int(seed),
                                                          abi.fptr(loss)), self.h)
        return loss

    def mlp_forward(self, feat):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        out = np.zeros(len(feat), dtype=np.float32)
        _check("mpsgpu_mlp_forward", lib().mpsgpu_mlp_forward(self.h, abi.fptr(feat), len(feat), abi.fptr(out)), self.h)
        return out

    def mlp_gradient(self, feat, target):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        grad = np.zeros(abi.MLP_NPARAM, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check("mpsgpu_mlp_gradient", lib().mpsgpu_mlp_gradient(self.h, abi.fptr(feat), abi.fptr(target), len(feat),
                                                                abi.fptr(grad), abi.fptr(loss)), self.h)
        return grad, float(loss[0])
