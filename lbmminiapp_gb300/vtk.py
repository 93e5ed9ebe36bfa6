"""Legacy-VTK output of a state, in the layout of the reference's
``Propagation::writeVTK`` (src/propagation/Propagation.cpp:36-161):

    # vtk DataFile Version 3.0 / Placeholder / ASCII / DATASET STRUCTURED_POINTS
    DIMENSIONS nx ny nz, ORIGIN 0 0 0, SPACING 1 1 1, POINT_DATA nx*ny*nz
    SCALARS rho double   (0 at non-fluid points)
    SCALARS id int       (fluid points: a fluid index; others: LAT_PT_WALL = -10)
    VECTORS velocity double   (sum c f / rho, no F/2 shift; 0 0 0 at non-fluid points)
    VECTORS nodes int    (i j k)

points in x-fastest order, numbers formatted like a default C++ stream (%g,
6 significant digits), the file named ``outs.00000.vtk`` by the reference's
single rank.  The fluid index of the "id" section is the point's rank among
the fluid points in x-fastest order (the reference numbers them in its own
sorted order, GeometryAAAB.cpp:127-205, which the dense layout here does not
have).  ``binary=True`` writes the same sections as legacy-VTK BINARY
(big-endian), which large grids need.
"""
from __future__ import annotations

import numpy as np

LAT_PT_WALL = -10  # src/geometries/Geometry.hh:41


def _fmt(a) -> str:
    a = np.asarray(a).ravel()
    if a.dtype.kind in "iu":
        return "\n".join(map(str, a.tolist()))
    return "\n".join(format(v, "g") for v in a.tolist())


def _fmt3(a) -> str:
    """(3, N) -> "x y z" lines."""
    cols = [np.asarray(c).ravel() for c in a]
    if cols[0].dtype.kind in "iu":
        strs = [list(map(str, c.tolist())) for c in cols]
    else:
        strs = [[format(v, "g") for v in c.tolist()] for c in cols]
    return "\n".join(f"{x} {y} {z}" for x, y, z in zip(*strs))


def fields(rho, u, solid):
    """The four sections' arrays: rho (0 at solids), id, velocity (3, ...)
    (0 at solids), nodes (3, ...) int32."""
    rho = np.asarray(rho, dtype=np.float64)
    fluid = ~np.asarray(solid, bool)
    nz, ny, nx = rho.shape
    r = np.where(fluid, rho, 0.0)
    v = np.where(fluid[None], np.asarray(u, dtype=np.float64), 0.0)
    ids = np.full(rho.shape, LAT_PT_WALL, dtype=np.int32)
    ids[fluid] = np.arange(int(fluid.sum()), dtype=np.int32)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    nodes = np.stack([i, j, k]).astype(np.int32)
    return r, ids, v, nodes


def write_vtk(path, rho, u, solid, binary=False):
    """Write rho (nz, ny, nx), u (3, nz, ny, nx) and the solid mask (nz, ny,
    nx) as a legacy VTK file at ``path``."""
    r, ids, v, nodes = fields(rho, u, solid)
    nz, ny, nx = r.shape
    head = (f"# vtk DataFile Version 3.0\nPlaceholder\n{'BINARY' if binary else 'ASCII'}\n"
            f"DATASET STRUCTURED_POINTS\nDIMENSIONS {nx} {ny} {nz}\nORIGIN 0 0 0\nSPACING 1 1 1\n"
            f"POINT_DATA {nx * ny * nz}\n")
    sections = [("SCALARS rho double\nLOOKUP_TABLE default\n", r, False),
                ("SCALARS id int\nLOOKUP_TABLE default\n", ids, False),
                ("VECTORS velocity double\n", v, True),
                ("VECTORS nodes int\n", nodes, True)]
    with open(path, "wb") as f:
        f.write(head.encode())
        for title, a, vec in sections:
            f.write(title.encode())
            if binary:
                data = np.moveaxis(a, 0, -1) if vec else a
                be = ">f8" if a.dtype.kind == "f" else ">i4"
                f.write(np.ascontiguousarray(data).astype(be).tobytes())
                f.write(b"\n")
            else:
                f.write(((_fmt3(a) if vec else _fmt(a)) + "\n").encode())


def read_vtk(path):
    """Parse a file written by :func:`write_vtk` (or the reference) into
    {"dims": (nx, ny, nz), section name: array}; ASCII values keep their text
    in ``text[name]``."""
    raw = open(path, "rb").read()
    lines = raw.split(b"\n")
    binary = lines[2].strip() == b"BINARY"
    dims = tuple(int(t) for t in lines[4].split()[1:4])
    n = dims[0] * dims[1] * dims[2]
    out = {"dims": dims, "text": {}}
    if binary:
        pos = len(b"\n".join(lines[:8])) + 1
        while pos < len(raw):
            end = raw.index(b"\n", pos)
            words = raw[pos:end].split()
            kind, name, typ = words[0].decode(), words[1].decode(), words[2].decode()
            pos = end + 1
            if kind == "SCALARS":
                pos = raw.index(b"\n", pos) + 1  # LOOKUP_TABLE line
            comps = 3 if kind == "VECTORS" else 1
            dt = np.dtype(">f8" if typ == "double" else ">i4")
            cnt = n * comps
            a = np.frombuffer(raw, dtype=dt, count=cnt, offset=pos).astype(dt.newbyteorder("="))
            out[name] = a.reshape(n, comps).T.reshape((comps,) + dims[::-1]) if comps == 3 else a.reshape(dims[::-1])
            pos += cnt * dt.itemsize + 1
        return out
    i = 8
    text = [ln.decode() for ln in lines]
    while i < len(text) and text[i]:
        words = text[i].split()
        kind, name, typ = words[0], words[1], words[2]
        i += 2 if kind == "SCALARS" else 1
        block = text[i:i + n]
        out["text"][name] = block
        if kind == "VECTORS":
            a = np.array([ln.split() for ln in block], dtype=float if typ == "double" else np.int64)
            out[name] = a.T.reshape((3,) + dims[::-1])
        else:
            out[name] = np.array(block, dtype=float if typ == "double" else np.int64).reshape(dims[::-1])
        i += n
    return out
