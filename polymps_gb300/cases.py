"""Deterministic dam-break cases standing in for PolyMPS's missing ``.grid`` inputs.

Axis convention: x = length, y = width, z = up, g = (0, 0, -9.81) in 3D (as in
input/InputDamINC.json); 2D runs in the (x, y) plane with g = (0, -9.81)
(input/dam1610_h300_lo0p0050_INC.json).  Particle centres sit at (k + 1/2) l0 from the
walls, the half-offset lattice that PolygonMesh::initWijnNeigh assumes
(src/PolygonMesh.cpp:406, 463).  Optional jitter ~U(-a l0, a l0) per coordinate with a
recorded numpy PCG64 seed.  Velocity and pressure start at zero.

Writers produce the reference's own formats: ``.grid`` (the layout read by
MpsInputOutput::readMpsParticleFile, src/MpsInputOutput.cpp:659-776), binary ``.stl``
and the JSON schema of MpsInputOutput::readInputFile (src/MpsInputOutput.cpp:126-509).
"""
import json
import math
import struct

import numpy as np

from . import abi

SEED = 20261203

# particle / boundary IDs of the example inputs (input/InputDamINC.json particle_type)
GHOST, FLUID, WALL, DUMMY = -1, 0, 2, 3


def _base_params():
    """Defaults shared by the example inputs (input/InputDamINC.json)."""
    return dict(
        wallType=1, femOn=0, forcedOn=0, domainMin=[0.0, 0.0, 0.0], domainMax=[1.0, 1.0, 1.0],
        domainTypeBC=0, limitTypeBC=0, densityFluid=1000.0, densityWall=1000.0, KNM_VS1=1e-6,
        fluidType=0, gravity=[0.0, 0.0, -9.81], KNM_VS2=1e-6, DNS_FL1=1000.0, DNS_FL2=1540.0,
        dim=3.0, partDist=0.01, timeStep=2.5e-4, timeSimulation=1.0, iterOutput=100,
        cflNumber=0.2, weightType=0, slipCondition=0, reS=2.1, reL=2.1, gradientType=0,
        gradientCorrection=1, relaxPress=1.0, mpsType=2, soundSpeed=15.0, gamma=7.0,
        solverType=0, alphaCompressibility=1e-6, relaxPND=0.01, shiftingType=0, dri=0.01,
        coefA=2.0, machNumber=0.1, pndType=0, diffusiveCoef=0.35, repulsiveForceType=2,
        reRepulsiveForce=0.5, expectMaxVelocity=4.0, repForceCoefMitsume=40000000.0,
        repForceCoefLennardJones=2.0, repForceCoefMonaghanKajtar=1.0, EPS_RE=0.01,
        freeSurfType=1, pndThreshold=0.98, neighThreshold=0.85, npcdThreshold=0.2,
        thetaThreshold=45.0, normThreshold=0.2, collisionType=0, collisionRatio=0.2,
        distLimitRatio=0.85, lambdaCollision=0.2, ghost=GHOST, fluid=FLUID, wall=WALL,
        dummyWall=DUMMY, surface=1, inner=0, other=-1,
    )


def box_triangles(x0, y0, z0, x1, y1, z1):
    """Closed axis-aligned box as 12 triangles (outward winding), (12, 9) float64."""
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float64)
    faces = [(0, 2, 1), (0, 3, 2),   # bottom z0 (normal -z)
             (4, 5, 6), (4, 6, 7),   # top z1 (+z)
             (0, 1, 5), (0, 5, 4),   # y0 (-y)
             (3, 7, 6), (3, 6, 2),   # y1 (+y)
             (0, 4, 7), (0, 7, 3),   # x0 (-x)
             (1, 2, 6), (1, 6, 5)]   # x1 (+x)
    return np.array([np.concatenate([v[a], v[b], v[c]]) for a, b, c in faces])


def _lattice3(nx, ny, nz, l0, jitter, rng):
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # reference-like ordering: z fastest inside y inside x is arbitrary; use x-major slabs
    pos = np.stack([(ix.ravel() + 0.5) * l0, (iy.ravel() + 0.5) * l0, (iz.ravel() + 0.5) * l0], 1)
    if jitter > 0:
        pos = pos + rng.uniform(-jitter * l0, jitter * l0, size=pos.shape)
    return pos


class Case:
    """A generated case: params (dict of MpsParams inputs), particle arrays, mesh."""

    def __init__(self, name, params, ptype, pos, mesh=None, steps=1):
        self.name = name
        self.params = params
        self.type = np.ascontiguousarray(ptype, dtype=np.int32)
        self.pos = np.ascontiguousarray(pos, dtype=np.float64)
        self.vel = np.zeros_like(self.pos)
        self.press = np.zeros(len(self.pos), dtype=np.float64)
        self.mesh = None if mesh is None else np.ascontiguousarray(mesh, dtype=np.float64)
        self.steps = steps

    @property
    def n(self):
        return len(self.pos)

    def mps_params(self):
        return abi.params_from_dict(self.params)

    # ---------------------------------------------------------------- writers
    def write_grid(self, path):
        """``.grid`` file: '0', N, then 'type x y z vx vy vz p p_av' per particle."""
        with open(path, "w") as f:
            f.write("0\n%d\n" % self.n)
            data = np.column_stack([self.pos, self.vel, self.press, self.press])
            for t, row in zip(self.type, data):
                f.write("%d " % t + " ".join("%.17g" % x for x in row) + "\n")

    def write_stl(self, path):
        """Binary STL of the triangle soup (face normal from the winding)."""
        tri = self.mesh.reshape(-1, 3, 3)
        with open(path, "wb") as f:
            f.write(b"polymps_gb300 generated box".ljust(80, b"\0"))
            f.write(struct.pack("<I", len(tri)))
            for t in tri:
                nrm = np.cross(t[1] - t[0], t[2] - t[0])
                nrm = nrm / (np.linalg.norm(nrm) or 1.0)
                f.write(struct.pack("<12fH", *nrm, *t[0], *t[1], *t[2], 0))

    def write_json(self, path, grid_path, stl_path, out_dir, vtu_type=0):
        """JSON input in the reference schema (radii in units of l0, as in the examples);
        vtu_type 0 ASCII output, 1 binary."""
        p = self.params
        js = {
            "flags": {"wall_type": p["wallType"], "fem_MESH": False, "forced_MESH": False,
                      "output_VTU": {"type": vtu_type, "only_freeSurface": False, "pnd": True,
                                     "neigh": True, "deviation": False, "concentration": False,
                                     "auxiliar": False, "non_newtonian": False}},
            "pathNames": {"particle_grid_file": grid_path, "mesh_rigid_file": stl_path,
                          "vtu_output_folder": out_dir},
            "domain": {"min": dict(zip("xyz", p["domainMin"])), "max": dict(zip("xyz", p["domainMax"])),
                       "boundary": {"type": 0, "limit": p["limitTypeBC"],
                                    "direction": {"x": False, "y": False, "z": False}}},
            "physical": {"fluid_density": p["densityFluid"], "wall_density": p["densityWall"],
                         "kinematic_visc": p["KNM_VS1"], "fluid_type": 0,
                         "gravity": dict(zip("xyz", p["gravity"])),
                         "rheological": {"kinematic_visc_phase_2": p["KNM_VS2"],
                                         "fluid_density_phase_1": p["DNS_FL1"],
                                         "fluid_density_phase_2": p["DNS_FL2"]}},
            "numerical": {
                "dimension": int(p["dim"]), "particle_dist": p["partDist"], "time_step": p["timeStep"],
                "final_time": p["timeSimulation"], "iter_output": p["iterOutput"],
                "CFL_number": p["cflNumber"], "weight_type": p["weightType"],
                "slip_condition": p["slipCondition"],
                "effective_radius": {"small": p["reS"], "large": p["reL"]},
                "gradient": {"type": p["gradientType"], "correction": bool(p["gradientCorrection"]),
                             "relax_fact": p["relaxPress"]},
                "mps_type": p["mpsType"],
                "explicit_mps": {"equation_state": {"speed_sound": p["soundSpeed"], "gamma": p["gamma"]}},
                "semi_implicit_mps": {"solver_type": p["solverType"],
                                      "weak_compressibility": {"alpha": p["alphaCompressibility"]},
                                      "source_term": {"relax_pnd": p["relaxPND"]}},
                "particle_shifting": {"type": p["shiftingType"], "DRI": p["dri"], "coef_A": p["coefA"],
                                      "mach_number": p["machNumber"]},
                "pnd": {"type": p["pndType"], "diffusive_coeff": p["diffusiveCoef"]},
                "wall_repulsive_force": {"type": p["repulsiveForceType"], "re": p["reRepulsiveForce"],
                                         "maxVel": p["expectMaxVelocity"],
                                         "coefficient": {"Mitsume": p["repForceCoefMitsume"],
                                                         "Lennard-Jones": p["repForceCoefLennardJones"],
                                                         "Monaghan-Kajtar": p["repForceCoefMonaghanKajtar"]},
                                         "eps_re": p["EPS_RE"]},
                "free_surface_threshold": {"type": p["freeSurfType"], "pnd": p["pndThreshold"],
                                           "neigh": p["neighThreshold"], "NPCD": p["npcdThreshold"],
                                           "ARC": p["thetaThreshold"], "normal": p["normThreshold"]},
                "particle_collision": {"type": p["collisionType"], "ratio": p["collisionRatio"],
                                       "dist_limit_ratio": p["distLimitRatio"], "lambda": p["lambdaCollision"]},
                "particle_type": {"ghost": p["ghost"], "fluid": p["fluid"], "wall": p["wall"],
                                  "dummyWall": p["dummyWall"]},
                "boundary_type": {"free_surface": p["surface"], "inner": p["inner"], "other": p["other"]},
            },
        }
        with open(path, "w") as f:
            json.dump(js, f, indent=1)


def dam2d_particle_walls(l0=0.01, width=0.25, height=0.5, tank=(1.0, 0.6), jitter=0.0,
                         seed=SEED, dt=5e-4):
    """2D incompressible dam break with particle walls (one wall layer, ID 2, and two
    dummy layers, ID 3) on the fluid lattice; parameters of
    input/dam1610_h300_lo0p0050_INC.json with l0, dt and re_large = 2.1 as given."""
    rng = np.random.default_rng(seed)
    nxf, nyf = int(round(width / l0)), int(round(height / l0))
    fx, fy = np.meshgrid(np.arange(nxf), np.arange(nyf), indexing="ij")
    fluid = np.stack([(fx.ravel() + 0.5) * l0, (fy.ravel() + 0.5) * l0, np.zeros(fx.size)], 1)
    if jitter > 0:
        fluid[:, :2] += rng.uniform(-jitter * l0, jitter * l0, size=(len(fluid), 2))
    L, H = tank
    nx, ny = int(round(L / l0)), int(round(H / l0))
    walls, types = [], []
    for layer in range(3):  # layer 0 = wall, 1..2 = dummy
        t = WALL if layer == 0 else DUMMY
        o = layer + 0.5
        xs = np.arange(-layer - 1, nx + layer + 1)  # bottom row incl. corners
        for ix in xs:
            walls.append(((ix + 0.5) * l0, -o * l0)); types.append(t)
        for iy in range(0, ny):  # side columns up to the tank height
            walls.append((-o * l0, (iy + 0.5) * l0)); types.append(t)
            walls.append((L + o * l0, (iy + 0.5) * l0)); types.append(t)
    walls = np.array(walls)
    wpos = np.column_stack([walls, np.zeros(len(walls))])
    pos = np.vstack([fluid, wpos])
    ptype = np.concatenate([np.full(len(fluid), FLUID), np.array(types)])
    p = _base_params()
    p.update(wallType=0, dim=2.0, partDist=l0, timeStep=dt, reS=2.1, reL=2.1,
             domainMin=[-0.1, -0.1, 0.0], domainMax=[L + 0.1, H + 0.2, 0.0],
             gravity=[0.0, -9.81, 0.0], soundSpeed=10.0, relaxPND=0.05, freeSurfType=0,
             pndThreshold=0.97, gradientType=0, gradientCorrection=1, mpsType=2, pndType=0,
             shiftingType=0, iterOutput=200)
    return Case("dam2d_inc_particle_walls", p, ptype, pos, None, steps=200)


def dam3d_polygon(l0=0.01, fluid=(0.6, 0.6, 0.3), tank=(1.61, 0.6, 0.6), mode="inc",
                  jitter=0.0, seed=SEED, dt=None, obstacle=None):
    """3D dam break inside a closed polygon box.  mode 'inc' follows input/InputDamINC.json
    (mps 2, pnd 0, grad 0 + correction, fs 1); mode 'wc' follows input/InputDamWC.json
    (mps 1, pnd 2 diffusive, grad 3, shifting 2) with c = 10 sqrt(2 g H)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(round(a / l0)) for a in fluid)
    pos = _lattice3(nx, ny, nz, l0, jitter, rng)
    tri = box_triangles(0.0, 0.0, 0.0, *tank)
    if obstacle is not None:
        (ox, oy, oz), (sx, sy, sz) = obstacle
        tri = np.vstack([tri, box_triangles(ox, oy, oz, ox + sx, oy + sy, oz + sz)])
    p = _base_params()
    p.update(wallType=1, dim=3.0, partDist=l0, domainMin=[0.0, 0.0, 0.0], domainMax=list(tank))
    if mode == "inc":
        p.update(mpsType=2, pndType=0, gradientType=0, gradientCorrection=1, shiftingType=0,
                 freeSurfType=1, relaxPND=0.01, alphaCompressibility=1e-6,
                 timeStep=dt if dt is not None else 2.5e-4)
        name = "dam3d_inc_polygon"
    elif mode == "wc":
        p.update(mpsType=1, pndType=2, gradientType=3, gradientCorrection=0, shiftingType=2,
                 freeSurfType=1, soundSpeed=10.0 * math.sqrt(2 * 9.81 * fluid[2]),
                 timeStep=dt if dt is not None else 1e-4)
        name = "dam3d_wc_polygon"
    else:
        raise ValueError(mode)
    return Case(name, p, np.full(len(pos), FLUID, dtype=np.int32), pos, tri)


def config(k, jitter=0.0, seed=SEED, scale=1.0):
    """The five workloads of the benchmark plan.  scale > 1 coarsens l0 (for quick tests)."""
    if k == 1:
        c = dam2d_particle_walls(l0=0.01 * scale, jitter=jitter, seed=seed)
        c.steps = 200
    elif k == 2:
        c = dam3d_polygon(l0=0.01 * scale, mode="wc", jitter=jitter, seed=seed)
        c.steps = 2000
    elif k == 3:
        c = dam3d_polygon(l0=0.005 * scale, mode="inc", jitter=jitter, seed=seed, dt=2.5e-4)
        c.steps = 1000
    elif k == 4:
        c = dam3d_polygon(l0=0.01 * scale, mode="inc", jitter=jitter, seed=seed, dt=2.5e-4)
        c.steps = 2000
    elif k == 5:
        c = dam3d_polygon(l0=0.004 * scale, fluid=(1.2, 1.0, 0.5), tank=(3.22, 1.0, 1.0),
                          mode="inc", jitter=jitter, seed=seed, dt=2.5e-4,
                          obstacle=((2.4, 0.42, 0.0), (0.16, 0.16, 0.4)))
        c.params.update(shiftingType=2)
        c.steps = 500
    else:
        raise ValueError(k)
    c.name = "cfg%d_" % k + c.name
    return c
