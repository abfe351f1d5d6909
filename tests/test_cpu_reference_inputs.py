"""The reference's own example inputs through the drop-in reader (CPU, no GPU).

Every input/*.json of the reference (the schema of MpsInputOutput::readInputFile,
src/MpsInputOutput.cpp:58-641) is read by the C++ host driver (`mps_gb300 --check-input`)
with its .grid file replaced by a small stub lattice (the reference's .grid files are not
distributed) and its .stl taken from the reference's input/stl.  Checked:

* every value present in the JSON reaches the matching MpsParams field unchanged;
* every JSON key of the table below occurs in at least one of the reference's files (the
  table's key names are the reference's, not this reader's);
* the status: switches outside the implemented path (non-Newtonian rheology, deformable
  or forced meshes, periodic domains) give MPSGPU_ERR_UNSUPPORTED with a message naming the switch; the
  reference's own input check (incompressible MPS with pnd type 1 or 2,
  src/MpsInputOutput.cpp:531-544) gives MPSGPU_ERR_ARG; every other file is accepted.

The files are read where the reference lies (POLYMPS_REFERENCE, default /root/reference);
the test is skipped where it is absent.
"""
import glob
import json
import os
import subprocess

import numpy as np
import pytest

from polymps_gb300 import abi

REF = os.environ.get("POLYMPS_REFERENCE", "/root/reference")
FILES = sorted(glob.glob(os.path.join(REF, "input", "*.json")))

# JSON path -> MpsParams field (k: component of a 3-vector)
KEYS = [
    (("flags", "wall_type"), "wallType"), (("flags", "fem_MESH"), "femOn"), (("flags", "forced_MESH"), "forcedOn"),
    (("domain", "min", "x"), ("domainMin", 0)), (("domain", "min", "y"), ("domainMin", 1)),
    (("domain", "min", "z"), ("domainMin", 2)), (("domain", "max", "x"), ("domainMax", 0)),
    (("domain", "max", "y"), ("domainMax", 1)), (("domain", "max", "z"), ("domainMax", 2)),
    (("domain", "boundary", "type"), "domainTypeBC"), (("domain", "boundary", "limit"), "limitTypeBC"),
    (("physical", "fluid_density"), "densityFluid"), (("physical", "wall_density"), "densityWall"),
    (("physical", "kinematic_visc"), "KNM_VS1"), (("physical", "fluid_type"), "fluidType"),
    (("physical", "gravity", "x"), ("gravity", 0)), (("physical", "gravity", "y"), ("gravity", 1)),
    (("physical", "gravity", "z"), ("gravity", 2)),
    (("physical", "rheological", "kinematic_visc_phase_2"), "KNM_VS2"),
    (("physical", "rheological", "fluid_density_phase_1"), "DNS_FL1"),
    (("physical", "rheological", "fluid_density_phase_2"), "DNS_FL2"),
    (("numerical", "dimension"), "dim"), (("numerical", "particle_dist"), "partDist"),
    (("numerical", "time_step"), "timeStep"), (("numerical", "final_time"), "timeSimulation"),
    (("numerical", "iter_output"), "iterOutput"), (("numerical", "CFL_number"), "cflNumber"),
    (("numerical", "weight_type"), "weightType"), (("numerical", "slip_condition"), "slipCondition"),
    (("numerical", "effective_radius", "small"), "reS"), (("numerical", "effective_radius", "large"), "reL"),
    (("numerical", "gradient", "type"), "gradientType"), (("numerical", "gradient", "correction"), "gradientCorrection"),
    (("numerical", "gradient", "relax_fact"), "relaxPress"), (("numerical", "mps_type"), "mpsType"),
    (("numerical", "explicit_mps", "equation_state", "speed_sound"), "soundSpeed"),
    (("numerical", "explicit_mps", "equation_state", "gamma"), "gamma"),
    (("numerical", "semi_implicit_mps", "solver_type"), "solverType"),
    (("numerical", "semi_implicit_mps", "weak_compressibility", "alpha"), "alphaCompressibility"),
    (("numerical", "semi_implicit_mps", "source_term", "relax_pnd"), "relaxPND"),
    (("numerical", "particle_shifting", "type"), "shiftingType"), (("numerical", "particle_shifting", "DRI"), "dri"),
    (("numerical", "particle_shifting", "coef_A"), "coefA"),
    (("numerical", "particle_shifting", "mach_number"), "machNumber"),
    (("numerical", "pnd", "type"), "pndType"), (("numerical", "pnd", "diffusive_coeff"), "diffusiveCoef"),
    (("numerical", "wall_repulsive_force", "type"), "repulsiveForceType"),
    (("numerical", "wall_repulsive_force", "re"), "reRepulsiveForce"),
    (("numerical", "wall_repulsive_force", "maxVel"), "expectMaxVelocity"),
    (("numerical", "wall_repulsive_force", "coefficient", "Mitsume"), "repForceCoefMitsume"),
    (("numerical", "wall_repulsive_force", "coefficient", "Lennard-Jones"), "repForceCoefLennardJones"),
    (("numerical", "wall_repulsive_force", "coefficient", "Monaghan-Kajtar"), "repForceCoefMonaghanKajtar"),
    (("numerical", "wall_repulsive_force", "eps_re"), "EPS_RE"),
    (("numerical", "free_surface_threshold", "type"), "freeSurfType"),
    (("numerical", "free_surface_threshold", "pnd"), "pndThreshold"),
    (("numerical", "free_surface_threshold", "neigh"), "neighThreshold"),
    (("numerical", "free_surface_threshold", "NPCD"), "npcdThreshold"),
    (("numerical", "free_surface_threshold", "ARC"), "thetaThreshold"),
    (("numerical", "free_surface_threshold", "normal"), "normThreshold"),
    (("numerical", "particle_collision", "type"), "collisionType"),
    (("numerical", "particle_collision", "ratio"), "collisionRatio"),
    (("numerical", "particle_collision", "dist_limit_ratio"), "distLimitRatio"),
    (("numerical", "particle_collision", "lambda"), "lambdaCollision"),
    (("numerical", "particle_type", "ghost"), "ghost"), (("numerical", "particle_type", "fluid"), "fluid"),
    (("numerical", "particle_type", "wall"), "wall"), (("numerical", "particle_type", "dummyWall"), "dummyWall"),
    (("numerical", "boundary_type", "free_surface"), "surface"), (("numerical", "boundary_type", "inner"), "inner"),
    (("numerical", "boundary_type", "other"), "other"),
]


def _strip_comments(t):
    """Drop // and /* */ comments outside strings (the reference parses with comments
    skipped, src/MpsInputOutput.cpp:126-129)."""
    out, i, instr = [], 0, False
    while i < len(t):
        c = t[i]
        if instr:
            out.append(c)
            if c == "\\" and i + 1 < len(t):
                out.append(t[i + 1]); i += 2; continue
            if c == '"':
                instr = False
            i += 1
        elif c == '"':
            instr = True; out.append(c); i += 1
        elif t.startswith("//", i):
            j = t.find("\n", i)
            i = len(t) if j < 0 else j
        elif t.startswith("/*", i):
            j = t.find("*/", i + 2)
            i = len(t) if j < 0 else j + 2
        else:
            out.append(c); i += 1
    return "".join(out)


def _load(path):
    with open(path) as f:
        return json.loads(_strip_comments(f.read()))


def _get(d, path):
    for k in path:
        if not isinstance(d, dict) or k not in d:
            return None
        d = d[k]
    return d


def _stub_grid(path, d):
    """A small lattice of fluid particles in the middle of the JSON's domain."""
    dim = int(_get(d, ("numerical", "dimension")) or 3)
    l0 = float(_get(d, ("numerical", "particle_dist")) or 0.01)
    lo = np.array([_get(d, ("domain", "min", k)) or 0.0 for k in "xyz"], dtype=float)
    hi = np.array([_get(d, ("domain", "max", k)) or 0.0 for k in "xyz"], dtype=float)
    c = 0.5 * (lo + hi)
    rng = range(-2, 3)
    pts = [(c[0] + i * l0, c[1] + j * l0, (c[2] + k * l0) if dim == 3 else 0.0)
           for i in rng for j in rng for k in (rng if dim == 3 else [0])]
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        f.write("0\n%d\n" % len(pts))
        for p in pts:
            f.write("0 %.17g %.17g %.17g 0 0 0 0 0\n" % p)
    return len(pts)


def _expected_status(d):
    fluid = int(_get(d, ("physical", "fluid_type")) or 0)
    fem = bool(_get(d, ("flags", "fem_MESH"))) or bool(_get(d, ("flags", "forced_MESH")))
    mps = int(_get(d, ("numerical", "mps_type")) if _get(d, ("numerical", "mps_type")) is not None else 1)
    pnd = int(_get(d, ("numerical", "pnd", "type")) or 0)
    if mps in (2, 3) and pnd in (1, 2):
        return abi.ERR_ARG, "pnd-type"
    if fem:
        return abi.ERR_UNSUPPORTED, "fem_MESH"
    if int(_get(d, ("domain", "boundary", "type")) or 0) != 0:
        return abi.ERR_UNSUPPORTED, "periodic"
    if fluid != 0:
        return abi.ERR_UNSUPPORTED, "fluid_type"
    return 0, "ok"


@pytest.fixture(scope="module")
def driver():
    from polymps_gb300 import build
    build.build()
    exe = os.path.join(os.path.dirname(abi.LIB_PATH), "mps_gb300")
    assert os.path.exists(exe)
    return exe


@pytest.mark.skipif(not FILES, reason="the reference's input/*.json are not present")
def test_table_keys_are_the_references():
    docs = [_load(f) for f in FILES]
    missing = [".".join(path) for path, _ in KEYS if all(_get(d, path) is None for d in docs)]
    assert not missing, "keys in no reference input: %s" % missing


@pytest.mark.skipif(not FILES, reason="the reference's input/*.json are not present")
@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_reference_input_reads(driver, tmp_path, path):
    d = _load(path)
    grid = _get(d, ("pathNames", "particle_grid_file"))
    stl = _get(d, ("pathNames", "mesh_rigid_file"))
    n = _stub_grid(str(tmp_path / grid), d)
    if stl and os.path.exists(os.path.join(REF, stl)):
        os.makedirs(os.path.dirname(str(tmp_path / stl)), exist_ok=True)
        os.symlink(os.path.join(REF, stl), str(tmp_path / stl))
    out = str(tmp_path / "params.bin")
    r = subprocess.run([driver, path, "--check-input", out], capture_output=True, text=True, cwd=str(tmp_path),
                       timeout=120)
    status_line = [ln for ln in r.stdout.splitlines() if ln.startswith("check-input status")]
    assert status_line, r.stdout + r.stderr
    want, word = _expected_status(d)
    assert r.returncode == want, status_line[0]
    if want:
        assert word in status_line[0], status_line[0]
    else:
        assert "particles %d" % n in status_line[0]
    with open(out, "rb") as f:
        raw = f.read()
    assert len(raw) == C_SIZE
    p = abi.MpsParams.from_buffer_copy(raw)
    for jpath, field in KEYS:
        v = _get(d, jpath)
        if v is None or isinstance(v, (dict, list, str)):
            continue
        got = getattr(p, field[0])[field[1]] if isinstance(field, tuple) else getattr(p, field)
        assert float(got) == float(v), "%s: JSON %r, read %r" % (".".join(jpath), v, got)


C_SIZE = __import__("ctypes").sizeof(abi.MpsParams)
