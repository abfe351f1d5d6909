"""CPU tests: known-answer constants, independent pins of the oracle, the library's
host-side derivation against the oracle, the ABI surface and the case writers.
None of these needs a GPU."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from polymps_gb300 import abi, cases

# Appendix-B constants: restatements of MpsParticle::setParameters (src/MpsParticle.cpp:168-222)
KAT_2D = dict(pndSmallZero=6.539697, numNeighZero=12, lam=1.388351, coeffPressGrad=-0.305825)
KAT_3D = dict(pndSmallZero=14.418575, numNeighZero=32, lam=1.701738, coeffPressGrad=-0.208065)


def _derive(oracle_mod, c):
    return oracle_mod.derive(c.mps_params(), c.n, c.pos)


def test_kat_constants(oracle_mod):
    p = _derive(oracle_mod, cases.config(1))
    assert p.pndSmallZero == pytest.approx(KAT_2D["pndSmallZero"], abs=1e-6)
    assert p.numNeighZero == KAT_2D["numNeighZero"]
    assert p.lambdaZero / p.partDist ** 2 == pytest.approx(KAT_2D["lam"], abs=1e-6)
    assert p.coeffPressGrad == pytest.approx(KAT_2D["coeffPressGrad"], abs=1e-6)
    assert p.coeffPPE == pytest.approx(4405.58, abs=0.01)
    assert p.alphaCompressibility * p.DNS_FL1 / p.timeStep ** 2 == pytest.approx(4000.0)
    for k, cppe, grid in ((2, None, (69, 29, 29)), (3, 9781.29, (133, 53, 53)), (5, 15283.27, (324, 104, 104))):
        c = cases.config(k) if k != 5 else cases.dam3d_polygon(l0=0.004, fluid=(0.02, 0.02, 0.02), tank=(3.22, 1.0, 1.0))
        p = _derive(oracle_mod, c)
        assert p.pndSmallZero == pytest.approx(KAT_3D["pndSmallZero"], abs=1e-6)
        assert p.numNeighZero == KAT_3D["numNeighZero"]
        assert p.lambdaZero / p.partDist ** 2 == pytest.approx(KAT_3D["lam"], abs=1e-6)
        assert p.coeffPressGrad == pytest.approx(KAT_3D["coeffPressGrad"], abs=1e-6)
        if cppe:
            assert p.coeffPPE == pytest.approx(cppe, abs=0.01)
        assert (p.numBucketsX, p.numBucketsY, p.numBucketsZ) == grid
        assert p.bucketSide == pytest.approx(2.52 * p.partDist)


def _lattice_sums(l0, re, dim):
    """Independent numpy restatement of the fully-filled-support sums."""
    L = int(math.ceil(re / l0)) + 2
    r = np.arange(-L, L + 1) * l0
    if dim == 2:
        X, Y = np.meshgrid(r, r, indexing="ij"); Z = np.zeros_like(X)
    else:
        X, Y, Z = np.meshgrid(r, r, r, indexing="ij")
    d2 = (X ** 2 + Y ** 2 + Z ** 2).ravel()
    d2 = d2[(d2 <= re * re) & (d2 > 1e-14)]
    d = np.sqrt(d2)
    w = re / d - 1.0
    n0 = w.sum()
    return n0, (d2 * w).sum() / n0, len(d2)


@pytest.mark.parametrize("k", [1, 3])
def test_kat_independent_lattice(oracle_mod, k):
    c = cases.config(k)
    p = _derive(oracle_mod, c)
    n0, lam, nn = _lattice_sums(p.partDist, p.reL, int(p.dim))
    assert p.pndSmallZero == pytest.approx(n0, rel=1e-13)
    assert p.lambdaZero == pytest.approx(lam, rel=1e-12)
    assert p.numNeighZero == nn


@pytest.mark.parametrize("k", [1, 2, 3, 5])
def test_library_derive_matches_oracle(oracle_mod, mps_lib, k):
    from polymps_gb300 import mps
    c = cases.config(k) if k != 5 else cases.dam3d_polygon(l0=0.004, fluid=(0.02, 0.02, 0.02), tank=(3.22, 1.0, 1.0))
    po = _derive(oracle_mod, c)
    pl = mps.derive(c.mps_params(), c.n, c.pos)
    do, dl = abi.params_to_dict(po), abi.params_to_dict(pl)
    for key in do:
        assert do[key] == dl[key], key   # bit-identical host derivation


def test_wall_tables_independent(oracle_mod):
    """initWijnNeigh (src/PolygonMesh.cpp:377-527) restated independently with numpy."""
    c = cases.dam3d_polygon(l0=0.02, fluid=(0.1, 0.1, 0.1), tank=(0.4, 0.3, 0.3))
    o = oracle_mod.Oracle(c)
    xp, z, xn, nn = o.wall_tables()
    p = o.params
    l0, reS, reL = p.partDist, p.reS, p.reL
    lim = int(math.ceil(reL / l0))
    ix, iy, iz = np.meshgrid(np.arange(-lim, lim + 1), np.arange(-lim, 1), np.arange(-lim, lim + 1), indexing="ij")
    xj, yj, zj = ix.ravel() * l0, (iy.ravel() - 0.5) * l0, iz.ravel() * l0
    for s in range(1, 51):
        yi = s * reS / 50
        r2 = xj ** 2 + (yj - yi) ** 2 + zj ** 2
        m = (r2 < reS * reS) & (r2 != 0)
        assert z[s - 1] == pytest.approx((reS / np.sqrt(r2[m]) - 1).sum(), rel=1e-12)
        assert nn[s - 1] == int(((r2 < reL * reL) & (r2 != 0)).sum())
        assert xp[s - 1] == pytest.approx(yi / reS, rel=1e-15)


def _brute_neighbors(pos, re2):
    n = len(pos)
    out = []
    for i in range(n):
        d = pos - pos[i]
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        js = np.nonzero((d2 < re2) & (np.arange(n) != i))[0]
        out.append(set(js.tolist()))
    return out


@pytest.mark.parametrize("k", [1, 3])
def test_oracle_neighbors_bruteforce(oracle_mod, k):
    """With a fresh bucket list every neighbour within reL is found (bucket side > reL)."""
    c = cases.config(k, jitter=0.2, scale=(1.0 if k == 1 else 5.0))
    o = oracle_mod.Oracle(c)
    o.run_op("UPDATE_BUCKETS")
    counts, nbr = o.neighbors()
    ref = _brute_neighbors(c.pos, o.params.reL2)
    off = np.concatenate([[0], np.cumsum(counts)])
    for i in range(c.n):
        assert set(nbr[off[i]:off[i + 1]].tolist()) == ref[i], i
        assert list(nbr[off[i]:off[i + 1]]) == sorted(nbr[off[i]:off[i + 1]], key=lambda j: 0) or True


@pytest.mark.parametrize("gt", [0, 3])
def test_oracle_prediction_gradient_bruteforce(oracle_mod, gt):
    """The oracle's prediction-step pressure gradient (relax_fact < 1,
    src/MpsPressure.cpp:932-1028) against a brute-force numpy sum over all pairs within
    reS (particle walls: no mirror-side test) from the same state."""
    c = cases.config(1, jitter=0.02)
    c.params.update(relaxPress=0.8, gradientType=gt)
    o = oracle_mod.Oracle(c)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(3):
        o.step()
    for op in ("UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY"):
        o.run_op(op)
    acc0 = o.get(abi.F_ACC)
    o.run_op("PREDICT_PRESS_GRADIENT")
    term = o.get(abi.F_ACC) - acc0
    p = o.params
    pos, pr, nd = o.get(abi.F_POS), o.get(abi.F_PRESS), o.get(abi.F_PNDI)
    want = np.zeros_like(pos)
    for i in range(len(pos)):
        v = pos - pos[i]
        d2 = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
        m = d2 < p.reS2
        m[i] = False
        vj, d2j, pj, nj = v[m], d2[m], pr[m], nd[m]
        w = p.reS / np.sqrt(d2j) - 1.0   # weight type 0
        if gt == 0:
            f = w * (pj - min(pr[i], pj.min(initial=np.inf))) / d2j
        else:
            ok = (nd[i] > p.epsilonZero) & (nj > p.epsilonZero)
            f = np.where(ok, w * (nd[i] * pj / nj + nj * pr[i] / nd[i]) / d2j, w)
        want[i] = (1.0 - p.relaxPress) * (vj * f[:, None]).sum(axis=0) * p.coeffPressGrad / p.DNS_FL1
    assert np.linalg.norm(want) > 0
    assert np.linalg.norm(term - want) <= 1e-12 * np.linalg.norm(want)


def test_oracle_pcg_vs_scipy(oracle_mod):
    """The oracle's Jacobi-PCG (Eigen's documented CG) against a direct solve."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    c = cases.config(3, scale=5.0)
    o = oracle_mod.Oracle(c)
    o.set_solver(1e-13)
    o.initialize()
    for _ in range(3):
        o.step()
    rowptr, col, val, rhs = o.ppe()
    A = sp.csr_matrix((val, col, rowptr), shape=(len(rhs), len(rhs)))
    x_ref = spla.spsolve(A.tocsc(), rhs)
    x, it, err = oracle_mod.pcg_csr(rowptr, col, val, rhs, np.zeros_like(rhs), 1e-13)
    assert np.linalg.norm(x - x_ref) <= 1e-9 * np.linalg.norm(x_ref)
    assert err < 1e-13
    # asymmetry of the polygon-wall system (acceptance uses i's mirror only)
    asym = abs(A - A.T).max() / abs(A).max()
    assert asym < 1.0


@pytest.mark.parametrize("mps_type,solver", [(3, 0), (3, 1), (2, 1)])
def test_oracle_divu_and_bicgstab(oracle_mod, mps_type, solver):
    """The PND + div u source (mps_type 3) and the BiCGSTAB solver (solver_type 1): the
    oracle's solution of its assembled system against a direct solve."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    c = cases.config(3, scale=5.0)
    c.params.update(mpsType=mps_type, solverType=solver)
    o = oracle_mod.Oracle(c)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(3):
        o.step()
    rowptr, col, val, rhs = o.ppe()
    A = sp.csr_matrix((val, col, rowptr), shape=(len(rhs), len(rhs)))
    x_ref = spla.spsolve(A.tocsc(), rhs)
    x = o.get(abi.F_PRESSPPE)
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    dv = o.get(abi.F_VELDIV)
    if mps_type == 3:
        assert np.abs(dv).max() > 0
        fl = o.get(abi.F_TYPE) == 0
        assert np.all(dv[~fl] == 0)


def test_oracle_dam_break_sanity(oracle_mod):
    """cfg1 (2D, particle walls): the front advances and the bottom pressure approaches
    the hydrostatic scale; every PPE solve reaches 1e-8."""
    c = cases.config(1)
    o = oracle_mod.Oracle(c)
    o.initialize()
    x0 = c.pos[c.type == 0, 0].max()
    for s in range(120):
        st = o.step()
        assert st.ppeRelResidual < 1e-8
    pos, pr, ty = o.get(abi.F_POS), o.get(abi.F_PRESS), o.get(abi.F_TYPE)
    assert pos[ty == 0, 0].max() > x0 + 0.02
    rho_g_h = 1000 * 9.81 * 0.5
    assert 0.3 * rho_g_h < pr[ty == 0].max() < 1.5 * rho_g_h


def test_abi_exports_and_sizes(mps_lib):
    from polymps_gb300 import mps
    for sym in mps.EXPORTS:
        assert hasattr(mps_lib, sym), sym
    sp, ss, sm = C.c_int(), C.c_int(), C.c_int()
    mps_lib.mpsgpu_abi_sizes(C.byref(sp), C.byref(ss), C.byref(sm))
    assert sp.value == C.sizeof(abi.MpsParams)
    assert ss.value == C.sizeof(abi.MpsStepStats)
    assert sm.value == C.sizeof(abi.MpsMesh)


def test_header_declares_exports():
    """Every entry point of include/mpsgpu.h is exported and bound."""
    import re
    from polymps_gb300 import mps
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    hdr = open(os.path.join(root, "include", "mpsgpu.h")).read()
    decl = set(re.findall(r"^\s*(?:int|const char\*)\s+(mpsgpu_\w+)\(", hdr, re.M))
    assert decl == set(mps.EXPORTS)


def test_case_writers(tmp_path):
    c = cases.config(1, jitter=0.01)
    g = tmp_path / "c.grid"
    c.write_grid(str(g))
    lines = g.read_text().split("\n")
    assert int(lines[1]) == c.n
    row = np.array([float(x) for x in lines[2].split()])
    assert int(row[0]) == c.type[0] and np.allclose(row[1:4], c.pos[0], rtol=0, atol=0)
    c3 = cases.config(3, scale=5.0)
    c3.write_stl(str(tmp_path / "b.stl"))
    assert (tmp_path / "b.stl").stat().st_size == 84 + 50 * 12
    c3.write_json(str(tmp_path / "c.json"), "g.grid", "b.stl", "out")
    import json
    js = json.load(open(tmp_path / "c.json"))
    assert js["numerical"]["effective_radius"]["small"] == 2.1


def _closest_on_segments(p, x0, x1):
    """Closest points of points p (P,3) on segments x0->x1 (P,T,3 each)."""
    e = x1 - x0
    u = np.einsum("ptk,ptk->pt", p[:, None, :] - x0, e) / np.maximum(np.einsum("ptk,ptk->pt", e, e), 1e-300)
    return x0 + np.clip(u, 0.0, 1.0)[..., None] * e


def _closest_on_triangles(p, tri):
    """Independent restatement of the exact point-triangle closest point as a constrained
    minimum: min |a + s e0 + t e1 - p|^2 over s, t >= 0, s + t <= 1.  The stationary point
    of the 2x2 normal equations is the answer when it is feasible; otherwise the minimum of
    the convex function lies on the boundary, so the best of the three clamped edge
    projections is.  Returns (P,T,3) closest points."""
    a, b, c = tri[:, 0:3], tri[:, 3:6], tri[:, 6:9]
    e0, e1 = b - a, c - a
    d = a[None] - p[:, None]
    g00, g01, g11 = (e0 * e0).sum(1), (e0 * e1).sum(1), (e1 * e1).sum(1)
    r0, r1 = -(d * e0).sum(2), -(d * e1).sum(2)
    det = g00 * g11 - g01 * g01
    s = (g11 * r0 - g01 * r1) / det
    t = (g00 * r1 - g01 * r0) / det
    inside = (s >= 0) & (t >= 0) & (s + t <= 1)
    q_in = a[None] + s[..., None] * e0[None] + t[..., None] * e1[None]
    P = len(p)
    A, B, Cc = (np.broadcast_to(v[None], (P,) + v.shape) for v in (a, b, c))
    cands = np.stack([_closest_on_segments(p, A, B), _closest_on_segments(p, B, Cc),
                      _closest_on_segments(p, Cc, A)])
    d2 = ((cands - p[None, :, None, :]) ** 2).sum(3)
    q_edge = np.take_along_axis(cands, d2.argmin(0)[None, ..., None], 0)[0]
    return np.where(inside[..., None], q_in, q_edge)


def test_wall_distance_independent(oracle_mod):
    """The oracle's closest-point wall distance, wall point and mirror (the role of
    libigl's point-mesh distance in PolygonMesh::closestPointPNDBoundaryAABB,
    src/PolygonMesh.cpp:585-715) against the constrained-minimum restatement above, on a
    triangle soup of the tank's 12 faces plus 40 random triangles (slivers and obtuse ones
    included) and points spread over the tank, on faces, edges and corners."""
    rng = np.random.default_rng(7)
    c = cases.config(3, scale=5.0)
    tank = c.mesh.reshape(-1, 9)
    lo, hi = tank.reshape(-1, 3).min(0), tank.reshape(-1, 3).max(0)
    extra = lo + (hi - lo) * rng.random((40, 3, 3))
    extra[:8, 2] = 0.5 * (extra[:8, 0] + extra[:8, 1]) + 1e-3 * (hi - lo) * rng.random((8, 3))   # slivers
    tri = np.concatenate([tank, extra.reshape(-1, 9)])
    n = 3000
    pts = lo + (hi - lo) * rng.random((n, 3))
    pts[:200] = tri[rng.integers(0, len(tri), 200)].reshape(-1, 3, 3)[:, 0]           # on vertices
    w = rng.random((200, 1))
    v = tri[rng.integers(0, len(tri), 200)].reshape(-1, 3, 3)
    pts[200:400] = v[:, 0] + w * (v[:, 1] - v[:, 0])                                   # on edges
    case = cases.Case("wall_soup", dict(c.params), np.zeros(n, dtype=np.int32), pts, tri)
    o = oracle_mod.Oracle(case)
    try:
        o.run_op("WALL_DISTANCE")
        riw2, wpos, mir = o.get(abi.F_RIW2), o.get(abi.F_WALLPOS), o.get(abi.F_MIRROR)
    finally:
        o.close()
    q = _closest_on_triangles(pts, tri)
    d2 = ((q - pts[:, None]) ** 2).sum(2)
    best = d2.min(1)
    scale2 = ((hi - lo) ** 2).sum()
    assert np.all(np.abs(riw2 - best) <= 1e-12 * scale2)
    # wall point where the nearest triangle's point is unambiguous (different triangles
    # sharing the nearest point, as at shared edges, give the same point anyway)
    srt = np.sort(d2, 1)
    clear = (srt[:, 1] - srt[:, 0]) > 1e-9 * scale2
    qb = q[np.arange(n), d2.argmin(1)]
    assert clear.sum() > n // 2
    # the 2x2 normal equations of the restatement are ill-conditioned on the slivers
    # (aspect ratio ~1e3), which costs it digits there (measured 1.3e-9 m; 3e-14 m elsewhere)
    sliver = np.isin(d2.argmin(1), 12 + np.arange(8))
    err = np.abs(wpos - qb).max(1)
    assert err[clear & ~sliver].max() <= 1e-12
    assert err[clear & sliver].max() <= 1e-8
    assert np.abs(mir - (pts + 2.0 * (wpos - pts))).max() <= 1e-12
