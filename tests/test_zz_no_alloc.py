"""Allocation-free pressure solve (mpsgpu_pcg_solve_static) against the handle's solver.

The PPE system of a step is read back from the library, placed on the device with
torch (device memory only), and solved twice in a row through the C-ABI entry point
that keeps its work vectors in a static device array.  Both solutions must match the
handle's plain FP64 PCG solution of the same system within the pressure tolerance of
the parity tests (relative 1e-9 at solver tolerance 1e-12) and each other bit for bit
(the entry point's reductions are in a fixed order).
"""
import ctypes as C

import numpy as np
import pytest

from polymps_gb300 import abi, cases

pytestmark = pytest.mark.gpu

CASES = {
    "cfg1_2d_particle_walls": lambda: cases.config(1, jitter=0.0),
    "cfg3_3d_inc_polygon": lambda: cases.config(3, jitter=0.02, scale=5.0),
}


def relerr(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _system(mps, case):
    g = mps.MpsGpu(case, tol=1e-12)
    g.initialize()
    for _ in range(3):
        g.step()
    g.run_op("CALC_PRESS")
    rowptr, col, val, rhs = g.ppe()
    x_ref = g.get(abi.F_PRESSPPE)
    g.close()
    return rowptr, col, val, rhs, x_ref


def _solve(L, torch, rowptr, col, val, rhs, tol=1e-12, max_iter=20000):
    dev = torch.device("cuda:0")
    d_rowptr = torch.from_numpy(rowptr.astype(np.int32)).to(dev)
    d_col = torch.from_numpy(np.ascontiguousarray(col, dtype=np.int32)).to(dev)
    d_val = torch.from_numpy(np.ascontiguousarray(val, dtype=np.float64)).to(dev)
    d_b = torch.from_numpy(np.ascontiguousarray(rhs, dtype=np.float64)).to(dev)
    d_x = torch.zeros(rhs.size, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    iters, relres = C.c_int(), C.c_double()
    rc = L.mpsgpu_pcg_solve_static(rhs.size, d_rowptr.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                                   d_b.data_ptr(), d_x.data_ptr(), tol, max_iter, None,
                                   C.byref(iters), C.byref(relres))
    assert rc == 0, L.mpsgpu_pcg_static_error().decode()
    torch.cuda.synchronize()
    return d_x.cpu().numpy(), iters.value, relres.value


@pytest.mark.parametrize("name", list(CASES))
def test_static_solver_matches_handle_solver(mps_lib, name):
    torch = pytest.importorskip("torch")
    from polymps_gb300 import mps
    rowptr, col, val, rhs, x_ref = _system(mps, CASES[name]())
    assert 0 < rhs.size <= abi.STATIC_MAX_ROWS
    x1, it1, rr1 = _solve(mps_lib, torch, rowptr, col, val, rhs)
    x2, it2, rr2 = _solve(mps_lib, torch, rowptr, col, val, rhs)
    assert it1 > 0 and rr1 < 1e-11
    assert relerr(x1, x_ref) < 1e-9
    assert relerr(x2, x_ref) < 1e-9
    assert it1 == it2 and np.array_equal(x1, x2)


def test_static_solver_rejects_oversize(mps_lib):
    # rejected on the host before any pointer is used
    dummy = C.c_void_p(16)
    rc = mps_lib.mpsgpu_pcg_solve_static(abi.STATIC_MAX_ROWS + 1, dummy, dummy, dummy, dummy, dummy,
                                         1e-8, 10, None, None, None)
    assert rc == abi.ERR_ARG
    assert b"rows outside" in mps_lib.mpsgpu_pcg_static_error()
