"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU oracle (oracle/mps_oracle.cpp).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by
the product package.  The oracle restates the reference algorithm in FP64; see the
header of mps_oracle.cpp for what is restated from third-party documentation (Eigen CG,
libigl closest point) and is therefore unpinned.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from polymps_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libmps_oracle.so")
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.orc_params_derive.argtypes = [C.POINTER(abi.MpsParams), C.c_int, C.POINTER(C.c_double)]
        L.orc_create.argtypes = [C.POINTER(abi.MpsParams), C.c_int, C.POINTER(C.c_int),
                                 C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(abi.MpsMesh), C.POINTER(vp)]
        for f in ("orc_destroy", "orc_initialize"):
            getattr(L, f).argtypes = [vp]
        L.orc_step.argtypes = [vp, C.POINTER(abi.MpsStepStats)]
        L.orc_run_op.argtypes = [vp, C.c_int]
        L.orc_set_solver.argtypes = [vp, C.c_double, C.c_int]
        L.orc_num_particles.argtypes = [vp, C.POINTER(C.c_int)]
        L.orc_state.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.orc_set_velmax.argtypes = [vp, C.c_double]
        L.orc_get_field.argtypes = [vp, C.c_int, vp]
        L.orc_set_field.argtypes = [vp, C.c_int, vp]
        L.orc_get_neighbors.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_longlong]
        L.orc_get_ppe.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_wall_tables.argtypes = [vp] + [C.POINTER(C.c_double)] * 3 + [C.POINTER(C.c_int)]
        L.orc_pcg_csr.argtypes = [C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_int),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.c_double, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def derive(params, n, pos):
    p = abi.MpsParams.from_buffer_copy(params)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    e = lib().orc_params_derive(C.byref(p), n, abi.dptr(pos))
    if e:
        raise RuntimeError("orc_params_derive failed: %d" % e)
    return p


class Oracle:
    """FP64 CPU restatement of the reference step, with the same field/op vocabulary as
    the GPU library."""

    def __init__(self, case, threads=None):
        L = lib()
        if threads:
            L.orc_set_threads(int(threads))
        self.case = case
        self.params = derive(case.mps_params(), case.n, case.pos)
        self._mesh, self._tri = abi.make_mesh(case.mesh)
        h = C.c_void_p()
        e = L.orc_create(C.byref(self.params), case.n, abi.iptr(case.type), abi.dptr(case.pos),
                         abi.dptr(case.vel), abi.dptr(case.press),
                         C.byref(self._mesh) if self._mesh is not None else None, C.byref(h))
        if e:
            raise RuntimeError("orc_create failed: %d" % e)
        self.h = h

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        v = C.c_int()
        lib().orc_num_particles(self.h, C.byref(v))
        return v.value

    def initialize(self):
        e = lib().orc_initialize(self.h)
        if e:
            raise RuntimeError("orc_initialize: %d" % e)

    def step(self):
        st = abi.MpsStepStats()
        e = lib().orc_step(self.h, C.byref(st))
        if e:
            raise RuntimeError("orc_step: %d" % e)
        return st

    def run_op(self, op):
        if isinstance(op, str):
            op = abi.OP[op]
        e = lib().orc_run_op(self.h, op)
        if e:
            raise RuntimeError("orc_run_op(%s): %d" % (abi.OPS[op], e))

    def set_solver(self, tol, max_iter=-1):
        lib().orc_set_solver(self.h, tol, max_iter)

    def set_velmax(self, v):
        lib().orc_set_velmax(self.h, v)

    def state(self):
        t, it, vm, si, se = C.c_double(), C.c_int(), C.c_double(), C.c_int(), C.c_double()
        lib().orc_state(self.h, C.byref(t), C.byref(it), C.byref(vm), C.byref(si), C.byref(se))
        return dict(time=t.value, iterations=it.value, velMax=vm.value, solverIter=si.value,
                    solverError=se.value)

    def get(self, field):
        buf = abi.field_buffer(field, self.n)
        e = lib().orc_get_field(self.h, field, buf.ctypes.data)
        if e:
            raise RuntimeError("orc_get_field %d: %d" % (field, e))
        return buf

    def set(self, field, arr):
        ref = abi.field_buffer(field, self.n)
        arr = np.ascontiguousarray(arr, dtype=ref.dtype).reshape(ref.shape)
        e = lib().orc_set_field(self.h, field, arr.ctypes.data)
        if e:
            raise RuntimeError("orc_set_field %d: %d" % (field, e))

    def neighbors(self):
        n = self.n
        counts = np.zeros(n, dtype=np.int32)
        lib().orc_get_neighbors(self.h, abi.iptr(counts), None, 0)
        tot = int(counts.sum())
        nbr = np.zeros(max(tot, 1), dtype=np.int32)
        e = lib().orc_get_neighbors(self.h, abi.iptr(counts), abi.iptr(nbr), tot)
        if e:
            raise RuntimeError("orc_get_neighbors: %d" % e)
        return counts, nbr[:tot]

    def ppe(self):
        nnz = C.c_longlong()
        lib().orc_get_ppe(self.h, C.byref(nnz), None, None, None, None)
        n = self.n
        rowptr = np.zeros(n + 1, dtype=np.int64)
        col = np.zeros(max(nnz.value, 1), dtype=np.int32)
        val = np.zeros(max(nnz.value, 1), dtype=np.float64)
        rhs = np.zeros(n, dtype=np.float64)
        lib().orc_get_ppe(self.h, C.byref(nnz), rowptr.ctypes.data_as(C.POINTER(C.c_longlong)),
                          abi.iptr(col), abi.dptr(val), abi.dptr(rhs))
        return rowptr, col[:nnz.value], val[:nnz.value], rhs

    def wall_tables(self):
        a, b, c = (np.zeros(50) for _ in range(3))
        d = np.zeros(50, dtype=np.int32)
        e = lib().orc_wall_tables(self.h, abi.dptr(a), abi.dptr(b), abi.dptr(c), abi.iptr(d))
        if e:
            raise RuntimeError("no wall tables")
        return a, b, c, d


def pcg_csr(rowptr, col, val, b, x0, tol, max_iter=-1):
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.array(x0, dtype=np.float64, copy=True)
    it, err = C.c_int(), C.c_double()
    lib().orc_pcg_csr(len(b), rowptr.ctypes.data_as(C.POINTER(C.c_longlong)), abi.iptr(col),
                      abi.dptr(val), abi.dptr(b), abi.dptr(x), tol, max_iter, C.byref(it), C.byref(err))
    return x, it.value, err.value
