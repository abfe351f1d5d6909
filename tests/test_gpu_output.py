"""Binary .vtu output formatted from the device buffers (`mpsgpu_write_vtu`) and the host
driver's ASCII and binary outputs (MpsInputOutput::writeVtuAscii, src/MpsInputOutput.cpp:
1313-1580: same arrays, names and types)."""
import os
import subprocess

import numpy as np
import pytest

from polymps_gb300 import abi, build, cases
from polymps_gb300.vtu import read_vtu

pytestmark = pytest.mark.gpu

ALL = abi.VTU_PND | abi.VTU_NEIGH | abi.VTU_DEVIATION | abi.VTU_CONCENTRATION | abi.VTU_AUXILIAR


def test_binary_vtu_matches_fields(mps_lib, tmp_path):
    from polymps_gb300 import mps
    c = cases.config(3, jitter=0.02, scale=5.0)
    g = mps.MpsGpu(c, precision=abi.PRECISION_DF32)
    g.initialize()
    g.run(3)
    path = tmp_path / "s.vtu"
    g.write_vtu(path, ALL)
    v = read_vtu(path)
    n = g.n
    f32 = lambda f: g.get(f).astype(np.float32)
    assert np.array_equal(v["Position"], f32(abi.F_POS))
    assert np.array_equal(v["Velocity"], f32(abi.F_VEL))
    assert np.array_equal(v["pressure"], f32(abi.F_PRESS))
    assert np.array_equal(v["BC"], g.get(abi.F_BC))
    assert np.array_equal(v["pnd"], f32(abi.F_PNDI))
    assert np.array_equal(v["pndSmall"], f32(abi.F_PNDSMALL))
    assert np.array_equal(v["nNeigh"], g.get(abi.F_NUMNEIGH))
    assert np.array_equal(v["npcdDeviation"], f32(abi.F_NPCD))
    assert np.array_equal(v["polygonNormal"], f32(abi.F_POLYNORMAL))
    assert np.array_equal(v["concentration"], f32(abi.F_CONC))
    assert np.array_equal(v["GradCi"], f32(abi.F_GRADC))
    assert np.array_equal(v["ParticleType"], g.get(abi.F_TYPE))
    assert np.array_equal(v["nearMeshType"], np.zeros(n, np.int32))
    assert np.array_equal(v["connectivity"], np.arange(n, dtype=np.int32))
    assert np.array_equal(v["offsets"], np.arange(1, n + 1, dtype=np.int32))
    assert np.array_equal(v["types"], np.ones(n, np.uint8))
    g.close()


def test_driver_ascii_and_binary_outputs(mps_lib, tmp_path):
    c = cases.config(3, jitter=0.02, scale=5.0)
    c.params.update(iterOutput=2)
    c.write_grid(str(tmp_path / "c.grid"))
    c.write_stl(str(tmp_path / "c.stl"))
    exe = os.path.join(build.OUT, "mps_gb300")
    out = {}
    for t in (0, 1):
        folder = str(tmp_path / ("out%d" % t))
        js = str(tmp_path / ("c%d.json" % t))
        c.write_json(js, str(tmp_path / "c.grid"), str(tmp_path / "c.stl"), folder, vtu_type=t)
        r = subprocess.run([exe, js, "--max-steps", "3"], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        out[t] = [read_vtu(os.path.join(folder, "output%05d.vtu" % k)) for k in (0, 1)]
    for a, b in zip(out[0], out[1]):
        assert set(a) == set(b)
        for name in a:
            if a[name].dtype.kind in "iu":
                assert np.array_equal(a[name], b[name]), name
            else:   # ASCII: six decimals
                assert np.allclose(a[name], b[name], rtol=1e-6, atol=1.01e-6), name
