"""The drop-in flow on the reference's own benchmark geometry: the cylinder of
src/geometries/Geometry.cpp, run through (a) the Python mirror of Parameters /
Propagation and (b) the C++ driver lbm-gb300-app, against golden readouts of
the reference's full app run (tests/golden/cylinder_*.npz, made by
tests/golden/make_golden.py from the reference itself).  Velocities within
1e-10 relative (F64X arithmetic), 1e-13 with exact FP64 arithmetic."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests._helpers import cylinder_cases, load_golden, rel_err

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def write_input(path, g, extra=""):
    path.write_text(f"simulationSize 2.0\npropPattern {int(g['propPattern'])}\npull {int(g['pull'])}\n"
                    f"unroll {int(g['unroll'])}\ndensityChange 0.01\nwritevtk 0\ntimesteps {int(g['steps'])}\n"
                    + extra)
    return path


@pytest.mark.parametrize("name", cylinder_cases())
@pytest.mark.parametrize("arithmetic,tol", [("f64x", 1e-10), ("f64", 1e-13)])
def test_reference_api_cylinder(gpu, tmp_path, name, arithmetic, tol):
    from lbmminiapp_gb300 import reference_api
    g = load_golden(name)
    lines = []
    inp = write_input(tmp_path / "in.txt", g, f"arithmetic {arithmetic}\n")
    prop = reference_api.main(str(inp), out=lines.append)
    assert "Simulation has 153216 fluid points" in lines
    assert "Passed baseline validation" in lines
    assert any(l.startswith("Total") and "MFLUPS" in l for l in lines)
    cx = int(g["centre_x"])
    u = prop.u[:, :, :, cx]
    fluid = np.isfinite(g["rho_plane"])
    assert np.array_equal(np.isfinite(prop.rho[:, :, cx]), fluid)
    assert rel_err(prop.rho[:, :, cx], g["rho_plane"], fluid) < tol
    assert rel_err(u, g["u_plane"], np.broadcast_to(fluid, u.shape)) < tol


@pytest.mark.parametrize("name", cylinder_cases())
def test_cpp_driver_cylinder(gpu, tmp_path, name):
    from lbmminiapp_gb300 import build
    app = build.build_app() if not build.APP.exists() else build.APP
    g = load_golden(name)
    inp = write_input(tmp_path / "in.txt", g)
    out = subprocess.run([str(app), str(inp)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    text = out.stdout
    assert "Simulation has 153216 fluid points" in text
    assert "Passed baseline validation" in text
    line = [l for l in text.splitlines() if l.startswith("Centre-line velocity")][0]
    vel = float(line.split()[2])
    dims = g["dims"]
    cj, ck = (int(dims[1]) - 1) // 2, (int(dims[2]) - 1) // 2
    ref_vel = float(g["u_plane"][0, ck, cj])
    assert abs(vel - ref_vel) <= 1e-10 * abs(ref_vel)


def _vtk_golden():
    import gzip
    text = gzip.open(ROOT / "tests" / "golden" / "cylinder_s1_aa_unroll_vtk.txt.gz", "rt").read().split("\n")
    return text


def _vtk_input(path, extra=""):
    path.write_text("simulationSize 1.0\npropPattern 1\npull 0\nunroll 1\ndensityChange 0.01\nwritevtk 1\n"
                    "timesteps 100\n" + extra)
    return path


def _check_vtk_against_reference(path):
    """Header, rho and velocity sections: the same text as the reference's
    outs.00000.vtk; ids: LAT_PT_WALL at the reference's walls (rho 0 there)."""
    golden = _vtk_golden()
    ours = Path(path).read_text().split("\n")
    i_id, i_vel, i_nodes = (ours.index(k) for k in ("SCALARS id int", "VECTORS velocity double",
                                                    "VECTORS nodes int"))
    assert ours[:i_id] + ours[i_vel:i_nodes] == golden[:-1]
    ids = np.array(ours[i_id + 2:i_vel], dtype=np.int64)
    rho = golden[10:i_id]
    walls = np.array([r == "0" for r in rho])
    assert np.array_equal(ids < 0, walls) and (ids[walls] == -10).all()
    assert np.array_equal(ids[~walls], np.arange((~walls).sum()))


def test_reference_api_writes_reference_vtk(gpu, tmp_path, monkeypatch):
    """writevtk 1 through the Python mirror, exact FP64 arithmetic: the VTK
    text equals the reference's own output of the same run."""
    from lbmminiapp_gb300 import reference_api
    inp = _vtk_input(tmp_path / "in.txt", "arithmetic f64\n")
    monkeypatch.chdir(tmp_path)
    reference_api.main(str(inp), out=lambda s: None)
    _check_vtk_against_reference(tmp_path / "outs.00000.vtk")


def test_cpp_driver_writes_reference_vtk(gpu, tmp_path):
    from lbmminiapp_gb300 import build
    app = build.build_app() if not build.APP.exists() else build.APP
    inp = _vtk_input(tmp_path / "in.txt", "arithmetic f64\n")
    out = subprocess.run([str(app), str(inp)], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert out.returncode == 0, out.stderr
    _check_vtk_against_reference(tmp_path / "outs.00000.vtk")
