"""VTK writer (no GPU): the reference's section layout and number format,
ASCII and BINARY round trips."""
import gzip
from pathlib import Path

import numpy as np

from lbmminiapp_gb300 import vtk

GOLDEN = Path(__file__).resolve().parent / "golden" / "cylinder_s1_aa_unroll_vtk.txt.gz"


def _case(seed=0, shape=(3, 4, 5)):
    rng = np.random.default_rng(seed)
    rho = 1.0 + 1e-3 * rng.standard_normal(shape)
    u = 1e-4 * rng.standard_normal((3,) + shape)
    solid = rng.random(shape) < 0.3
    rho[solid] = np.nan
    u[:, solid] = np.nan
    return rho, u, solid


def test_ascii_round_trip_and_layout(tmp_path):
    rho, u, solid = _case()
    p = tmp_path / "a.vtk"
    vtk.write_vtk(p, rho, u, solid)
    lines = p.read_text().split("\n")
    assert lines[:8] == ["# vtk DataFile Version 3.0", "Placeholder", "ASCII", "DATASET STRUCTURED_POINTS",
                         "DIMENSIONS 5 4 3", "ORIGIN 0 0 0", "SPACING 1 1 1", "POINT_DATA 60"]
    d = vtk.read_vtk(p)
    fluid = ~solid
    assert np.allclose(d["rho"][fluid], rho[fluid], rtol=1e-5) and (d["rho"][solid] == 0).all()
    assert np.allclose(d["velocity"][:, fluid], u[:, fluid], rtol=1e-5)
    assert (d["id"][solid] == vtk.LAT_PT_WALL).all()
    assert np.array_equal(d["id"][fluid], np.arange(fluid.sum()))
    assert np.array_equal(d["nodes"][0], np.broadcast_to(np.arange(5), (3, 4, 5)))
    assert np.array_equal(d["nodes"][2], np.broadcast_to(np.arange(3)[:, None, None], (3, 4, 5)))


def test_binary_round_trip_is_exact(tmp_path):
    rho, u, solid = _case(1, (4, 3, 6))
    p = tmp_path / "b.vtk"
    vtk.write_vtk(p, rho, u, solid, binary=True)
    d = vtk.read_vtk(p)
    r, ids, v, nodes = vtk.fields(rho, u, solid)
    assert np.array_equal(d["rho"], r) and np.array_equal(d["velocity"], v)
    assert np.array_equal(d["id"], ids) and np.array_equal(d["nodes"], nodes)


def test_number_format_matches_the_reference_file(tmp_path):
    """Values parsed from the reference's own VTK and written again give the
    same text (the C++ default stream format is %g)."""
    text = gzip.open(GOLDEN, "rt").read().split("\n")
    i_vel = text.index("VECTORS velocity double")
    nx, ny, nz = (int(t) for t in text[4].split()[1:])
    rho_txt = text[10:i_vel]
    vel_txt = text[i_vel + 1:i_vel + 1 + nx * ny * nz]
    rho = np.array(rho_txt, dtype=float).reshape(nz, ny, nx)
    vel = np.array([l.split() for l in vel_txt], dtype=float).T.reshape(3, nz, ny, nx)
    solid = np.array([t == "0" for t in rho_txt]).reshape(nz, ny, nx)
    p = tmp_path / "c.vtk"
    vtk.write_vtk(p, rho, vel, solid)
    d = vtk.read_vtk(p)
    assert d["text"]["rho"] == rho_txt
    assert d["text"]["velocity"] == vel_txt
    assert text[:8] == p.read_text().split("\n")[:8]
