"""Generate the golden fixtures in this directory from the reference itself.

Runs the UNMODIFIED lbmminiapp CPU kernels (compiled by oracle/build_ref.sh,
driven by oracle/ref_harness.cpp) on small seeded cases and stores inputs and
final raw population buffers as .npz files.  The reference sources are needed
only to regenerate; the fixtures themselves are committed so parity checks run
where the reference is absent.

    python tests/golden/make_golden.py          # small cases
    python tests/golden/make_golden.py --pins   # full-size C1 / C2 pins (about 25 min)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import core, ref  # noqa: E402
from lbmminiapp_gb300 import workloads  # noqa: E402

# name: (Q, variant, pattern, compat, (nx, ny, nz), periodic, walls, tau, gx, steps, U, noise)
CASES = {
    "q19_aa_base_tg_box": (19, ref.AA_BASE, core.AA, 0, (12, 10, 8), (1, 1, 1), False, 0.8, 0.0, 20, 0.05, 0.0),
    "q19_aa_unroll_channel_force": (19, ref.AA_UNROLL, core.AA, 1, (10, 9, 6), (1, 0, 1), True, 0.6, 1e-5, 15,
                                    0.02, 1e-3),
    "q19_ab_push_unroll_channel": (19, ref.AB_PUSH_UNROLL, core.AB_PUSH, 0, (9, 8, 7), (1, 0, 1), True, 0.7, 1e-5,
                                   11, 0.02, 1e-3),
    "q19_ab_pull_base_odd_box": (19, ref.AB_PULL_BASE, core.AB_PULL, 0, (17, 9, 5), (1, 1, 1), False, 0.55, 1e-6,
                                 9, 0.05, 1e-3),
    "q27_aa_base_tg_box": (27, ref.AA_BASE, core.AA, 0, (8, 8, 8), (1, 1, 1), False, 0.8, 0.0, 13, 0.05, 0.0),
    "q27_ab_push_channel_force": (27, ref.AB_PUSH_BASE, core.AB_PUSH, 0, (10, 8, 6), (1, 0, 1), True, 0.6, 1e-6,
                                  12, 0.0, 0.0),
    "q27_ab_pull_channel_force": (27, ref.AB_PULL_BASE, core.AB_PULL, 0, (10, 8, 6), (1, 0, 1), True, 0.6, 1e-6,
                                  12, 0.0, 0.0),
}


def case_inputs(Q, dims, walls, U, noise, seed=7):
    nx, ny, nz = dims
    u = workloads.taylor_green(nx, ny, nz, U=U, noise=noise, seed=seed)
    rho = 1.0 + workloads.uniform_noise((nz, ny, nx), seed, 3, 1e-3 if noise else 0.0)
    solid = workloads.channel_mask(nx, ny, nz) if walls else np.zeros((nz, ny, nx), np.uint8)
    if walls:
        u[:, solid.astype(bool)] = 0.0
    f0 = core.equilibrium(Q, rho, u)
    return f0, solid


# Reference app flow (src/Main.cpp) on the cylinder, size 2: keys of the
# reference's input files; only the centre x-plane of the readouts is kept.
CYLINDER_CASES = {
    "cylinder_s2_aa_unroll": dict(propPattern=1, pull=0, unroll=1),
    "cylinder_s2_ab_push_unroll": dict(propPattern=0, pull=0, unroll=1),
    "cylinder_s2_ab_pull_unroll": dict(propPattern=0, pull=1, unroll=1),
}
CYLINDER_STEPS = 100


def cylinder_input(path, propPattern, pull, unroll, steps=CYLINDER_STEPS, size=2.0):
    path.write_text(f"simulationSize {size}\npropPattern {propPattern}\npull {pull}\nunroll {unroll}\n"
                    f"densityChange 0.01\nwritevtk 0\ntimesteps {steps}\n")
    return path


def make_cylinder(tmpdir):
    for name, keys in CYLINDER_CASES.items():
        inp = cylinder_input(Path(tmpdir) / f"{name}.txt", **keys)
        out = ref.app_run(19, inp, omega=1.0, gx=1e-6)
        nx = out["dims"][0]
        cx = (nx - 1) // 2
        np.savez_compressed(HERE / f"{name}.npz", dims=np.array(out["dims"]), nfluid=out["nfluid"],
                            steps=out["steps"], centre_x=cx, rho_plane=out["rho"][:, :, cx],
                            u_plane=out["u"][:, :, :, cx], f_plane=out["f_raw"][:, :, :, cx], **keys)
        print(f"{name}: nfluid {out['nfluid']}")


# Compact-layout cases: the reference's own sorted fluid list, adjacency
# (GeometryAAAB::setupAdjacency) and final raw population buffer of a size-0.25
# cylinder (21 x 7 x 7, 672 fluid points) run through its app flow with the
# Base kernels (unroll 0).  The initial buffer is the rest state: every slot s
# holds w_s (checked here, so the tests rebuild it instead of storing it).
SPARSE_CASES = {
    "sparse_q19_aa_cylinder": dict(Q=19, propPattern=1, pull=0),
    "sparse_q19_ab_push_cylinder": dict(Q=19, propPattern=0, pull=0),
    "sparse_q19_ab_pull_cylinder": dict(Q=19, propPattern=0, pull=1),
    "sparse_q27_aa_cylinder": dict(Q=27, propPattern=1, pull=0),
}
SPARSE_SIZE, SPARSE_STEPS, SPARSE_OMEGA, SPARSE_GX = 0.25, 12, 1.0 / 0.7, 1e-4


def make_sparse(tmpdir):
    for name, keys in SPARSE_CASES.items():
        Q = keys["Q"]
        inp = cylinder_input(Path(tmpdir) / f"{name}.txt", keys["propPattern"], keys["pull"], 0,
                             steps=SPARSE_STEPS, size=SPARSE_SIZE)
        out = ref.app_run_compact(Q, inp, omega=SPARSE_OMEGA, gx=SPARSE_GX)
        _, _, w = core.stencil(Q)
        assert np.array_equal(out["raw_init"], np.repeat(w[:, None], out["nfluid"], axis=1))
        np.savez_compressed(HERE / f"{name}.npz", Q=Q, prop_pattern=keys["propPattern"], pull=keys["pull"],
                            dims=np.array(out["dims"]), steps=out["steps"], omega=SPARSE_OMEGA, gx=SPARSE_GX,
                            fluid_pts=out["fluid_pts"], adjacency=out["adjacency"], raw_final=out["raw_final"])
        print(f"{name}: nfluid {out['nfluid']}")


# The reference's VTK output (Propagation::writeVTK, src/propagation/
# Propagation.cpp:36-161) of a size-1 AA Unroll cylinder run: the header and
# the rho and velocity sections as the reference printed them (its "id"
# section numbers fluid points in the reference's own sorted order, and
# "nodes" is the index grid, so neither is kept).
VTK_CASE = "cylinder_s1_aa_unroll_vtk"
VTK_KEYS = dict(propPattern=1, pull=0, unroll=1)


def make_vtk(tmpdir):
    import gzip
    import os
    inp = cylinder_input(Path(tmpdir) / f"{VTK_CASE}.txt", **VTK_KEYS, size=1.0)
    inp.write_text(inp.read_text().replace("writevtk 0", "writevtk 1"))
    cwd = os.getcwd()
    os.chdir(tmpdir)
    try:
        ref.app_run(19, inp, omega=1.0, gx=1e-6)
    finally:
        os.chdir(cwd)
    lines = (Path(tmpdir) / "outs.00000.vtk").read_text().split("\n")
    i_id, i_vel, i_nodes = (lines.index(k) for k in ("SCALARS id int", "VECTORS velocity double",
                                                     "VECTORS nodes int"))
    keep = lines[:i_id] + lines[i_vel:i_nodes]
    with gzip.open(HERE / f"{VTK_CASE}.txt.gz", "wt") as f:
        f.write("\n".join(keep) + "\n")
    print(f"{VTK_CASE}: {len(keep)} lines")


# Reference pins of the full-size parity configurations.  The states are too
# large to commit (C1 40 MB, C2 906 MB per pattern), so each fixture keeps the
# SHA-256 of the reference's final populations over the fluid cells (the raw
# buffer in (q, z, y, x) order, little-endian float64) and a seeded sample of
# 1024 fluid cells.  The C1 initial state is rebuilt from 1-D tables of the
# Taylor-Green factors stored in the fixture (tests/_helpers.py:tg_box_init), so
# it does not depend on the host's libm.
#   c1_q19_aa_tg64      64^3 periodic, D3Q19 AA Base, tau 0.8, rho 1, TG U 0.05, 200 steps
#   c2_q27_ab_*_channel 256x128x128 channel (solid rows y = 0, 127), periodic x and z,
#                       D3Q27 AB Base push / pull, gx 1e-6, tau 0.6, rest start, 1000 steps
PIN_CASES = {
    "pin_c1_q19_aa_tg64": dict(Q=19, variant=ref.AA_BASE, pattern=core.AA, dims=(64, 64, 64), periodic=(1, 1, 1),
                               walls=False, tau=0.8, gx=0.0, steps=200, U=0.05),
    "pin_c2_q27_ab_push_channel": dict(Q=27, variant=ref.AB_PUSH_BASE, pattern=core.AB_PUSH, dims=(256, 128, 128),
                                       periodic=(1, 0, 1), walls=True, tau=0.6, gx=1e-6, steps=1000, U=0.0),
    "pin_c2_q27_ab_pull_channel": dict(Q=27, variant=ref.AB_PULL_BASE, pattern=core.AB_PULL, dims=(256, 128, 128),
                                       periodic=(1, 0, 1), walls=True, tau=0.6, gx=1e-6, steps=1000, U=0.0),
}


def make_pin(name):
    from tests._helpers import fluid_digest, pin_init, tg_tables
    c = PIN_CASES[name]
    nx, ny, nz = c["dims"]
    tables = tg_tables(nx, ny, nz) if c["U"] else {}
    fix = dict(Q=c["Q"], pattern=c["pattern"], variant=c["variant"], dims=np.array(c["dims"]),
               periodic=np.array(c["periodic"]), walls=int(c["walls"]), omega=1.0 / c["tau"], gx=c["gx"],
               steps=c["steps"], U=c["U"], **tables)
    f0, solid = pin_init(fix)
    raw, sec = ref.box_run(c["Q"], c["variant"], f0, c["steps"], 1.0 / c["tau"], c["gx"], c["periodic"], solid)
    fluid = ~solid.astype(bool)
    idx = np.flatnonzero(fluid.ravel())
    pick = np.sort(np.random.default_rng(11).choice(idx, 1024, replace=False))
    np.savez_compressed(HERE / f"{name}.npz", **fix, init_sha256=fluid_digest(f0, solid),
                        final_sha256=fluid_digest(raw, solid), sample_cells=pick,
                        sample_f=raw.reshape(c["Q"], -1)[:, pick], ref_seconds=sec)
    print(f"{name}: reference {sec:.1f} s, digest {fluid_digest(raw, solid)}", flush=True)


def main():
    if not ref.available():
        sys.exit("reference harness unavailable (oracle/build_ref.sh needs the reference sources)")
    if "--pins" in sys.argv:
        # one process per case (the reference kernels are serial)
        import multiprocessing as mp
        names = [a for a in sys.argv[1:] if a in PIN_CASES] or list(PIN_CASES)
        with mp.get_context("spawn").Pool(len(names)) as pool:
            pool.map(make_pin, names)
        return
    for name, (Q, variant, pattern, compat, dims, per, walls, tau, gx, steps, U, noise) in CASES.items():
        f0, solid = case_inputs(Q, dims, walls, U, noise)
        raw, _ = ref.box_run(Q, variant, f0, steps, 1.0 / tau, gx, per, solid)
        np.savez_compressed(HERE / f"{name}.npz", Q=Q, pattern=pattern, compat=compat, dims=np.array(dims),
                            periodic=np.array(per), solid=solid, omega=1.0 / tau, gx=gx, steps=steps,
                            f_init=f0, f_raw=raw, variant=variant)
        print(f"{name}: {raw.nbytes + f0.nbytes} bytes")
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        make_cylinder(tmp)
    with tempfile.TemporaryDirectory() as tmp:
        make_vtk(tmp)
    with tempfile.TemporaryDirectory() as tmp:
        make_sparse(tmp)


if __name__ == "__main__":
    main()
