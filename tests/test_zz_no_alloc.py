"""Allocation-free pressure solve (mpsgpu_pcg_solve_static) through the C ABI.

Callers that cannot allocate device memory at solve time (an application whose device
memory belongs to another framework's pool, a stepping loop that forbids allocation once
it runs) use this entry point: its work vectors sit in a static device array.  The PPE
system of a step is read back from the library, placed on the device with torch, and
solved twice in a row.  Both solutions must match the CPU oracle's Jacobi-PCG of the same
system (the restatement of Eigen's ConjugateGradient, src/MpsPressure.cpp:424-445) within
the parity tests' pressure tolerance (1e-9 at solver tolerance 1e-12), each other bit for
bit, and the device's free memory must be the same before and after the two calls.
This file is collected last so that a failure here leaves every other test already run.
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
    g.close()
    return rowptr, col, val, rhs


class _Dev:
    """The system's arrays in device memory (torch tensors), allocated once."""

    def __init__(self, torch, rowptr, col, val, rhs, x0=None):
        dev = torch.device("cuda:0")
        self.rowptr = torch.from_numpy(np.ascontiguousarray(rowptr, dtype=np.int32)).to(dev)
        self.col = torch.from_numpy(np.ascontiguousarray(col, dtype=np.int32)).to(dev)
        self.val = torch.from_numpy(np.ascontiguousarray(val, dtype=np.float64)).to(dev)
        self.b = torch.from_numpy(np.ascontiguousarray(rhs, dtype=np.float64)).to(dev)
        x0 = np.zeros(rhs.size) if x0 is None else x0
        self.x0 = torch.from_numpy(np.ascontiguousarray(x0, dtype=np.float64)).to(dev)
        self.x = self.x0.clone()
        self.n = rhs.size


def _solve(L, torch, d, tol=1e-12, max_iter=20000):
    d.x.copy_(d.x0)
    torch.cuda.synchronize()
    iters, relres = C.c_int(), C.c_double()
    rc = L.mpsgpu_pcg_solve_static(d.n, d.rowptr.data_ptr(), d.col.data_ptr(), d.val.data_ptr(),
                                   d.b.data_ptr(), d.x.data_ptr(), tol, max_iter, None,
                                   C.byref(iters), C.byref(relres))
    torch.cuda.synchronize()
    return rc, d.x.cpu().numpy(), iters.value, relres.value


@pytest.mark.parametrize("name", list(CASES))
def test_static_solver_matches_oracle(oracle_mod, mps_lib, name):
    torch = pytest.importorskip("torch")
    from polymps_gb300 import mps
    rowptr, col, val, rhs = _system(mps, CASES[name]())
    assert 0 < rhs.size <= abi.STATIC_MAX_ROWS
    x_orc, it_orc, err_orc = oracle_mod.pcg_csr(rowptr, col, val, rhs, np.zeros(rhs.size), 1e-12, 20000)
    assert err_orc < 1e-12
    d = _Dev(torch, rowptr, col, val, rhs)
    _solve(mps_lib, torch, d)   # loads the library's device code (and its static array) once
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc1, x1, it1, rr1 = _solve(mps_lib, torch, d)
    rc2, x2, it2, rr2 = _solve(mps_lib, torch, d)
    free1 = torch.cuda.mem_get_info()[0]
    assert rc1 == 0 and rc2 == 0, mps_lib.mpsgpu_pcg_static_error().decode()
    assert free1 == free0, "device free memory changed by %d bytes" % (free0 - free1)
    assert it1 > 0 and rr1 < 1e-11
    assert relerr(x1, x_orc) < 1e-9
    assert relerr(x2, x_orc) < 1e-9
    assert abs(it1 - it_orc) <= 2
    assert it1 == it2 and np.array_equal(x1, x2)


def test_static_solver_zero_rhs_gives_zero(oracle_mod, mps_lib):
    """b = 0 with a non-zero initial guess: x = 0 and relres 0, as the oracle's CG."""
    torch = pytest.importorskip("torch")
    from polymps_gb300 import mps
    rowptr, col, val, rhs = _system(mps, CASES["cfg1_2d_particle_walls"]())
    b = np.zeros_like(rhs)
    x0 = np.random.default_rng(5).normal(size=rhs.size)
    x_orc, _, err_orc = oracle_mod.pcg_csr(rowptr, col, val, b, x0, 1e-12, 20000)
    assert np.all(x_orc == 0.0) and err_orc == 0.0
    d = _Dev(torch, rowptr, col, val, b, x0)
    for _ in range(2):
        rc, x, it, rr = _solve(mps_lib, torch, d)
        assert rc == 0, mps_lib.mpsgpu_pcg_static_error().decode()
        assert np.all(x == 0.0) and it == 0 and rr == 0.0


def test_static_solver_rejects_missing_diagonal(mps_lib):
    """A row with a zero diagonal entry is reported as an argument error naming the row;
    the initial guess is left as it was."""
    torch = pytest.importorskip("torch")
    n = 64
    # tridiagonal SPD system, then row 17's diagonal set to zero
    rows, cols, vals = [], [], []
    for i in range(n):
        for j, v in ((i - 1, -1.0), (i, 4.0), (i + 1, -1.0)):
            if 0 <= j < n:
                rows.append(i); cols.append(j); vals.append(0.0 if (i == 17 and j == 17) else v)
    rowptr = np.searchsorted(np.array(rows), np.arange(n + 1))
    x0 = np.full(n, 0.5)
    d = _Dev(torch, rowptr, np.array(cols), np.array(vals), np.ones(n), x0)
    rc, x, _, _ = _solve(mps_lib, torch, d)
    assert rc == abi.ERR_ARG
    assert b"row 17" in mps_lib.mpsgpu_pcg_static_error()
    assert np.array_equal(x, x0)


def test_static_solver_rejects_oversize(mps_lib):
    # rejected on the host before any pointer is used
    dummy = C.c_void_p(16)
    rc = mps_lib.mpsgpu_pcg_solve_static(abi.STATIC_MAX_ROWS + 1, dummy, dummy, dummy, dummy, dummy,
                                         1e-8, 10, None, None, None)
    assert rc == abi.ERR_ARG
    assert b"rows outside" in mps_lib.mpsgpu_pcg_static_error()
