"""Wall distance and mirror particles against the oracle's brute force over all triangles
(PolygonMesh::closestPointPNDBoundaryAABB, src/PolygonMesh.cpp:585-715): the triangle BVH
walk of meshes above 64 triangles bit for bit, the brute-force kernel bit for bit within
2 reL of the wall and to rounding beyond."""
import numpy as np
import pytest

from polymps_gb300 import abi, cases

from test_gpu_parity import step_ops, sync

pytestmark = pytest.mark.gpu


def subdivide(tri, k):
    """Midpoint subdivision, k times (4^k triangles per triangle, winding kept)."""
    t = np.asarray(tri, dtype=np.float64).reshape(-1, 3, 3)
    for _ in range(k):
        a, b, c = t[:, 0], t[:, 1], t[:, 2]
        ab, bc, ca = 0.5 * (a + b), 0.5 * (b + c), 0.5 * (c + a)
        t = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                      np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3, 3)
    return t.reshape(-1, 9)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_DF32])
@pytest.mark.parametrize("levels", [2, 4])
def test_wall_distance_large_mesh(oracle_mod, mps_lib, levels, precision):
    from polymps_gb300 import mps
    c = cases.config(3, jitter=0.02, scale=5.0)
    mesh = subdivide(c.mesh, levels)            # 192 or 3,072 triangles
    assert len(mesh) > 64
    c2 = cases.Case(c.name, c.params, c.type, c.pos, mesh)
    o = oracle_mod.Oracle(c2)
    g = mps.MpsGpu(c2, tol=1e-12, precision=precision)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(3):
        o.step()
    ops = step_ops(o.params)
    sync(o, g)
    for op in ops[: ops.index("WALL_DISTANCE")]:
        o.run_op(op)
    sync(o, g)
    o.run_op("WALL_DISTANCE")
    g.run_op("WALL_DISTANCE")
    for f in (abi.F_RIW2, abi.F_WALLPOS, abi.F_MIRROR, abi.F_POLYNORMAL, abi.F_PNDWALL, abi.F_NNEIGHWALL,
              abi.F_NEARWALL):
        assert np.array_equal(g.get(f), o.get(f)), abi.FIELD_NAMES[f]
    assert g.get(abi.F_NEARWALL).sum() > 0
    g.close()


@pytest.mark.parametrize("cfg,scale", [(3, 5.0), (5, 6.0)])
def test_wall_distance_near_exact_far_projected(oracle_mod, mps_lib, cfg, scale):
    """The brute-force kernel (meshes up to 64 triangles): within 2 reL of the wall (where
    mirrors enter the sweeps' decisions) wall point, mirror and squared distance are the
    oracle's bit for bit; farther out the FP64 projection on the nearest triangle agrees
    with Ericson's walk to rounding; flags, normals and the wall tables' values exactly."""
    from polymps_gb300 import mps
    c = cases.config(cfg, jitter=0.02, scale=scale)
    o = oracle_mod.Oracle(c)
    g = mps.MpsGpu(c, tol=1e-12)
    o.set_solver(1e-12)
    o.initialize()
    for _ in range(3):
        o.step()
    ops = step_ops(o.params)
    sync(o, g)
    for op in ops[: ops.index("WALL_DISTANCE")]:
        o.run_op(op)
    sync(o, g)
    o.run_op("WALL_DISTANCE")
    g.run_op("WALL_DISTANCE")
    near = o.get(abi.F_RIW2) < 4.0 * o.params.reL2
    assert 0 < near.sum() < len(near)
    for f in (abi.F_POLYNORMAL, abi.F_PNDWALL, abi.F_NNEIGHWALL, abi.F_NEARWALL):
        assert np.array_equal(g.get(f), o.get(f)), abi.FIELD_NAMES[f]
    for f in (abi.F_RIW2, abi.F_WALLPOS, abi.F_MIRROR):
        a, b = g.get(f), o.get(f)
        assert np.array_equal(a[near], b[near]), abi.FIELD_NAMES[f]
        tol = 1e-15 * 16 if f == abi.F_RIW2 else 1e-15 * 8
        assert np.max(np.abs(a[~near] - b[~near])) <= tol * max(1.0, np.max(np.abs(b))), abi.FIELD_NAMES[f]
    g.close()


def test_large_mesh_free_running(oracle_mod, mps_lib):
    """Ten steps on a 3,072-triangle tank: the state follows the oracle's."""
    from polymps_gb300 import mps
    c = cases.config(3, jitter=0.02, scale=5.0)
    c2 = cases.Case(c.name, c.params, c.type, c.pos, subdivide(c.mesh, 4))
    o = oracle_mod.Oracle(c2)
    g = mps.MpsGpu(c2, tol=1e-12)
    o.set_solver(1e-12)
    o.initialize()
    g.initialize()
    for _ in range(10):
        o.step()
        g.step()
    from test_gpu_parity import relerr
    assert relerr(g.get(abi.F_POS), o.get(abi.F_POS)) < 1e-10
    assert relerr(g.get(abi.F_PRESS), o.get(abi.F_PRESS)) < 1e-6
    g.close()
