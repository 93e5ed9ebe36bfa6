#!/usr/bin/env python
"""Benchmark of the GB300 collide-stream path (one JSON line on stdout).

Workload (the headline configuration): D3Q19 BGK + Guo, AA propagation, SOA,
512^3 fully periodic box, tau = 0.55, Taylor-Green vortex (peak 0.05) plus
seeded uniform +-1e-3 velocity noise, FP64 population storage.  One bench step
is one lattice time step over the whole box (one kernel launch); the state is
20.4 GB, far larger than the 129 MB L2, so no flush is needed between steps.

* value      MLUPS with the state resident in HBM, CUDA events on the launch
             stream, max over ranks (independent replicas when --gpus > 1);
* e2e        the same metric through the C ABI from pinned host memory: the
             whole workload -- the initial velocity field copied in, its 1000
             steps, rho/u copied back -- inside the timed region;
* roofline   HBM bound: algorithmic bytes 2*Q*8 = 304 B per fluid-cell update
             over the measured copy bandwidth (MEASURED_PEAKS.json);
* cpu_baseline  the oracle port (C restatement of the reference's CPU kernels,
             OpenMP on all host cores) on a bounded sample of the workload;
* parity     the end-to-end run's result (F64X arithmetic, 1000 steps) against
             the exact FP64 arithmetic on the same workload (the reference's
             operation order, bit-identical to its CPU build): max relative
             error of the populations, rho and u (bound 1e-10; one GPU only).

``--impl reference`` times that CPU implementation alone (each step one lattice
step of a 256^3 sample of the same workload) and prints the same line shape.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MLUPS (D3Q19 AA FP64, 512^3 Taylor-Green box)"
UNIT = "MLUPS"
TAU = 0.55
# The port's speed against the reference's own CPU kernels, both on one thread
# of the x86-64 build host (Xeon @ 2.70 GHz, 128^3 sample of this workload, 10
# steps, two runs; the reference sources are not on the benchmark machine):
# port 7.05 / 6.76 MLUPS, reference KernelAA_SOA_Unroll 6.33 / 6.93, Base 5.21 / 5.14.
PORT_VS_REFERENCE = ("per thread the port runs 0.98-1.11x the reference's own AA Unroll kernel "
                     "(KernelAA_SOA_Unroll.cpp, 6.3-6.9 MLUPS) and 1.3-1.4x its Base kernel on an x86-64 "
                     "Xeon @ 2.70 GHz (128^3 sample of this workload)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=512, help="box edge (cells)")
    ap.add_argument("--no-variants", action="store_true", help="skip the other storage formats")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=1000,
                    help="lattice steps of the end-to-end round trip (the workload's 1000 steps)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the F64X-vs-exact-FP64 comparison of the end-to-end run (about 2 min at 512^3)")
    ap.add_argument("--ref-n", type=int, default=256, help="box edge of the reference arm's sample")
    ap.add_argument("--storage", default="f64", choices=["f64", "f32", "bf16", "f16"],
                    help="population storage of the timed run (headline: f64)")
    ap.add_argument("--lattice", type=int, default=19, choices=[19, 27])
    ap.add_argument("--pattern", default="aa", choices=["aa", "ab_push", "ab_pull"])
    ap.add_argument("--accuracy", action="store_true",
                    help="print the mixed-precision error table (n^3, 1000 steps) instead of timing")
    ap.add_argument("--porous", action="store_true",
                    help="print the sphere-packing permeability / porosity-gradient study instead of timing")
    ap.add_argument("--porous-n", type=int, default=384)
    ap.add_argument("--reference-benchmark", action="store_true",
                    help="print only the reference's cylinder benchmark (compact and dense layouts)")
    ap.add_argument("--configs", action="store_true",
                    help="print only the rates of the other workloads (small box, channel, porous channel, spheres)")
    ap.add_argument("--spheres", type=int, default=0, metavar="N",
                    help="print only the N^3 sphere-packing step rates (D3Q27 AA FP16, compact and dense), "
                         "even and odd steps timed apart")
    ap.add_argument("--cylinder-size", type=float, default=8.0)
    ap.add_argument("--cylinder-steps", type=int, default=20)
    ap.add_argument("--porous-steps", type=int, default=2000)
    return ap.parse_args()


def run_porous(args, device):
    """D3Q27 AA sphere packing (radius 6-12, solid fraction 0.35, periodic),
    g_x = 1e-6, tau = 0.7: permeability in FP64 / FP32 / BF16 / FP16 storage
    and the mean-flux porosity gradient of the FP16 forward with the FP32
    adjoint (checkpoints every 100 steps, sub-checkpoints every 10) against
    the FP64-storage forward (F64X arithmetic, within 1e-10 of exact FP64)
    with the FP64 adjoint (nested checkpoints of stride 3^6 .. 3, which fit
    the FP64 states in device memory)."""
    from lbmminiapp_gb300 import porous, workloads
    n, steps, tau, gx = args.porous_n, args.porous_steps, 0.7, 1e-6
    t0 = time.perf_counter()
    solid, centres, radii = workloads.sphere_packing(n, 0.35, 6.0, 12.0, seed=2024)
    t_pack = time.perf_counter() - t0
    fluid = ~solid.astype(bool)
    fw = {}
    for st, ar in (("f64", "f64"), ("f64", "f64x"), ("f32", "auto"), ("bf16", "auto"), ("f16", "auto")):
        fw[f"{st}/{ar}"] = porous.forward(solid, tau, gx, steps, storage=st, arithmetic=ar, device=device)
    k64 = fw["f64/f64"]["permeability"]
    for v in fw.values():
        v["k_rel_err"] = abs(v["permeability"] - k64) / k64
    L16, g16, t16 = porous.flux_gradient(solid, tau, gx, steps, (100, 10), storage="f16", adjoint="f32",
                                         device=device)
    L64, g64, t64 = porous.flux_gradient(solid, tau, gx, steps, (729, 243, 81, 27, 9, 3), storage="f64",
                                         adjoint="f64", arithmetic="f64x", device=device)
    out = {"porous": "D3Q27 AA periodic sphere packing", "grid": [n] * 3, "spheres": int(len(radii)),
           "solid_fraction": float(solid.mean()), "radius": [6, 12], "seed": 2024, "tau": tau, "gx": gx,
           "steps": steps, "packing_seconds": round(t_pack, 1),
           "forward": {k: {kk: (round(vv, 3) if kk in ("seconds", "mflups") else vv) for kk, vv in v.items()}
                       for k, v in fw.items()},
           "gradient": {"loss_f16_f32adj": L16, "loss_f64": L64, "loss_rel_err": abs(L16 - L64) / abs(L64),
                        "seconds_f16_f32adj": round(t16, 1), "seconds_f64": round(t64, 1),
                        "checkpoints_f16": [100, 10], "checkpoints_f64": [729, 243, 81, 27, 9, 3],
                        "reference": "FP64 storage, F64X forward, FP64 adjoint",
                        **porous.gradient_errors(g16, g64, fluid)}}
    print(json.dumps(out), flush=True)
    return 0


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend)
        return dist, rank, world, local
    return None, rank, world, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons every 100 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload_velocity(n, seed=2024):
    from lbmminiapp_gb300 import workloads
    return workloads.taylor_green(n, n, n, U=0.05, noise=1e-3, seed=seed)


def cpu_port_mlups(n, target_seconds=10.0, nthreads=0):
    """Oracle port (C restatement, OpenMP) on an n^3 sample of the workload:
    returns (MLUPS, threads, steps, seconds)."""
    from oracle import core
    u = workload_velocity(n)
    f0 = core.equilibrium(19, np.ones((n, n, n)), u)
    del u
    runner = core.Runner(19, core.AA, f0, 1.0 / TAU, nthreads=nthreads)
    del f0
    runner.step(2)
    t = runner.step(2)
    steps = max(2, int(target_seconds / max(t / 2, 1e-6)) // 2 * 2)
    t = runner.step(steps)
    threads = nthreads if nthreads > 0 else core.max_threads()
    runner.close()
    return n ** 3 * steps / t / 1e6, threads, steps, t


def traffic_per_launch():
    """DRAM bytes per step launch from the committed ncu summary, scaled to a
    512^3 launch (null when no capture is committed)."""
    p = ROOT / "profiles" / "aa_step_f64x_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    return d.get("bytes_per_launch_512")


def config_benchmarks(device, steps=20):
    """MLUPS (fluid cells) of the other workloads' shapes, each timed over
    `steps` steps after 2 warm-up steps with CUDA events:
    D3Q19 AA FP64 64^3 periodic Taylor-Green (tau 0.8);
    D3Q27 AB push / pull FP64 256x128x128 channel, gx 1e-6 (tau 0.6);
    D3Q19 AA FP32 128x64x64 channel with the smoothed porosity field, gx 1e-5 (tau 0.7);
    D3Q27 AA FP16 384^3 sphere packing (solid fraction 0.35), gx 1e-6 (tau 0.7), in the compact
    fluid-only storage and on the dense grid."""
    import torch
    import lbmminiapp_gb300 as lbm
    from lbmminiapp_gb300 import workloads

    def timed(sim, n):
        sim.step(2)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        sim.step(n)
        b.record()
        b.synchronize()
        return round(sim.nfluid * n / (a.elapsed_time(b) * 1e-3) / 1e6, 1)

    out = {}
    u = workloads.taylor_green(64, 64, 64, 0.05)
    with lbm.Simulation(64, 64, 64, lattice=19, pattern="aa", omega=1 / 0.8, force=(0, 0, 0), device=device) as sim:
        sim.init_equilibrium(None, u)
        out["q19 aa f64x 64^3 periodic"] = timed(sim, 200)
    solid = workloads.channel_mask(256, 128, 128)
    for pattern in ("ab_push", "ab_pull"):
        with lbm.Simulation(256, 128, 128, lattice=27, pattern=pattern, omega=1 / 0.6, force=(1e-6, 0, 0),
                            periodic=(1, 0, 1), device=device) as sim:
            sim.set_solid(solid)
            sim.init_equilibrium()
            out[f"q27 {pattern} f64x 256x128x128 channel"] = timed(sim, steps)
    solid = workloads.channel_mask(128, 64, 64)
    with lbm.Simulation(128, 64, 64, lattice=19, pattern="aa", omega=1 / 0.7, force=(1e-5, 0, 0), periodic=(1, 0, 1),
                        storage="f32", device=device) as sim:
        sim.set_solid(solid)
        sim.set_porosity(workloads.smoothed_porosity((64, 64, 128), sigma=3.0, seed=7))
        sim.init_equilibrium()
        out["q19 aa f32 128x64x64 channel + porosity"] = timed(sim, 100)
    solid, _, _ = workloads.sphere_packing(384, 0.35, 6.0, 12.0, seed=2024)
    for compact in (True, False):
        with lbm.Simulation(384, 384, 384, lattice=27, pattern="aa", omega=1 / 0.7, force=(1e-6, 0, 0),
                            storage="f16", device=device, compact=compact) as sim:
            sim.set_solid(solid)
            sim.init_equilibrium()
            name = "compact fluid-only storage" if compact else "dense grid"
            out[f"q27 aa f16 384^3 spheres, {name}"] = timed(sim, steps)
    return out


def spheres_benchmark(device, n, steps=10):
    """D3Q27 AA FP16 on the n^3 periodic sphere packing (radius 6-12, solid
    fraction 0.35, seed 2024), gx 1e-6, tau 0.7: per step kind, the mean time
    of `steps` launches (CUDA events around each) after 2 warm-up steps, as
    fluid-cell GLUPS and GB/s of algorithmic traffic (108 B per fluid-cell
    update), for the compact fluid-only storage and the dense grid."""
    import torch
    import lbmminiapp_gb300 as lbm
    from lbmminiapp_gb300 import workloads
    solid, _, _ = workloads.sphere_packing(n, 0.35, 6.0, 12.0, seed=2024)
    out = {"workload": f"D3Q27 AA FP16 {n}^3 sphere packing, solid fraction {solid.mean():.3f}"}
    for compact in (True, False):
        with lbm.Simulation(n, n, n, lattice=27, pattern="aa", omega=1 / 0.7, force=(1e-6, 0, 0), storage="f16",
                            device=device, compact=compact) as sim:
            sim.set_solid(solid)
            sim.init_equilibrium()
            sim.step(2)
            times = {0: [], 1: []}
            for k in range(2 * steps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                sim.step(1)
                b.record()
                b.synchronize()
                times[k % 2].append(a.elapsed_time(b))
            nf = sim.nfluid
            res = {}
            for kind, name in ((0, "even"), (1, "odd")):
                ms = statistics.mean(times[kind])
                res[name] = {"ms": round(ms, 4), "GLUPS": round(nf / (ms * 1e-3) / 1e9, 2),
                             "GB/s": round(nf * 108 / (ms * 1e-3) / 1e9, 1)}
            ms = statistics.mean(times[0] + times[1])
            res["mean"] = {"ms": round(ms, 4), "GLUPS": round(nf / (ms * 1e-3) / 1e9, 2),
                           "GB/s": round(nf * 108 / (ms * 1e-3) / 1e9, 1)}
            out["compact" if compact else "dense"] = res
            out["nfluid"] = nf
    return out


def cylinder_benchmark(device, size=8.0, steps=20):
    """The reference's own published benchmark workload: the size-8 cylinder
    (8,913,408 fluid points, src/geometries/Geometry.cpp:59-71,112-140),
    D3Q19, FP64, gravity-driven flow from rest, x periodic.  MLUPS per fluid
    point for AA, AB push and AB pull, through the compact fluid-only layout
    (the reference's own buffers and adjacency list) and the dense layout
    (link words), both with F64X arithmetic; CUDA events around `steps`
    steps after 2 warm-up steps.  The reference publishes 457-1017 MLUPS for
    this workload on one Intel Xe-HP tile."""
    import torch
    import lbmminiapp_gb300 as lbm
    from lbmminiapp_gb300 import sparse
    dims, solid = lbm.cylinder(size)
    nx, ny, nz = dims
    out = {"workload": f"cylinder size {size:g}, {nx}x{ny}x{nz}, D3Q19 FP64 (F64X), omega 1, gx 1e-6",
           "steps": steps}
    nfluid = int((solid == 0).sum())
    out["nfluid"] = nfluid
    w = np.array([1 / 18] * 6 + [1 / 36] * 12 + [1 / 3])

    def timed(run):
        run(2)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        run(steps)
        b.record()
        b.synchronize()
        return round(nfluid * steps / (a.elapsed_time(b) * 1e-3) / 1e6, 1)

    for pattern in ("aa", "ab_push", "ab_pull"):
        _, adj = sparse.build_adjacency(solid, (1, 0, 0), pattern, 19)
        f0 = torch.tensor(np.repeat(w[:, None], nfluid, axis=1), dtype=torch.float64, device="cuda")
        bufs = [f0] if pattern == "aa" else [f0, f0.clone()]
        with sparse.SparseKernels(adj, lattice=19, pattern=pattern, omega=1.0, force=(1e-6, 0, 0),
                                  device=device) as k:
            k.set_stream(torch.cuda.current_stream())

            def run(n):   # n even: AA parity and the AB buffer roles are unchanged
                k.run(bufs, n)
            out[f"compact/{pattern}"] = timed(run)
        del bufs, f0
        with lbm.Simulation(nx, ny, nz, lattice=19, pattern=pattern, omega=1.0, force=(1e-6, 0, 0),
                            periodic=(1, 0, 0), device=device) as sim:
            sim.set_solid(solid)
            sim.init_equilibrium(None, None)
            out[f"dense/{pattern}"] = timed(sim.step)
    return out


def state_copy(sim):
    """The handle's population buffer, copied into a new device tensor."""
    import ctypes
    import torch
    t = torch.empty(int(sim.info.buffer_bytes), dtype=torch.uint8, device="cuda")
    sim.synchronize()
    torch.cuda.synchronize()
    st = sim.lib.lbm_copy_state(sim.h, ctypes.c_void_p(t.data_ptr()), 0)
    if st:
        raise RuntimeError(f"lbm_copy_state failed ({st})")
    sim.synchronize()
    return t


def parity_vs_exact(n, u0, steps, state_x, rho_x, u_x, device):
    """The end-to-end run's F64X result against the exact FP64 arithmetic (the
    reference's operation order, bit-identical to its CPU build) on the same
    workload: max |a - b| / max |b| of the raw populations, rho and u."""
    import torch
    import lbmminiapp_gb300 as lbm
    t0 = time.perf_counter()
    with lbm.Simulation(n, n, n, lattice=19, pattern="aa", omega=1.0 / TAU, force=(0, 0, 0), storage="f64",
                        arithmetic="f64", device=device) as sim:
        sim.init_equilibrium(None, u0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        sim.step(steps)
        sim.synchronize()
        exact_s = time.perf_counter() - t1
        rho_e, u_e = sim.macros()
        state_e = state_copy(sim)
        plane = int(sim.info.plane_stride)
    ncell = n ** 3
    a = state_x.view(torch.float64).view(19, plane)[:, :ncell]
    b = state_e.view(torch.float64).view(19, plane)[:, :ncell]
    dmax = max(float((a[q] - b[q]).abs().max()) for q in range(19))
    bmax = max(float(b[q].abs().max()) for q in range(19))
    del a, b, state_e
    return {"workload": f"D3Q19 AA {n}^3, tau {TAU}, Taylor-Green U 0.05 + 1e-3 noise, {steps} steps",
            "compared": "F64X (the timed arithmetic) vs exact FP64 (reference operation order) on the GPU",
            "pop_rel_max": dmax / bmax,
            "rho_rel_max": float(np.abs(rho_x - rho_e).max() / np.abs(rho_e).max()),
            "u_rel_max": float(np.abs(u_x - u_e).max() / np.abs(u_e).max()),
            "tolerance": 1e-10, "exact_f64_mlups": round(ncell * steps / exact_s / 1e6, 1),
            "seconds": round(time.perf_counter() - t0, 1)}


def max_over_ranks(dist, value: float, device) -> float:
    """The largest `value` over all ranks (every rank gets it); `value` itself
    without a process group."""
    if not dist:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference_arm(args, dist, rank, world):
    if rank != 0:
        return 0
    from oracle import core
    n = args.ref_n
    u = workload_velocity(n)
    f0 = core.equilibrium(19, np.ones((n, n, n)), u)
    del u
    runner = core.Runner(19, core.AA, f0, 1.0 / TAU)
    del f0
    threads = core.max_threads()
    for _ in range(args.warmup):
        runner.step(1)
    times = [runner.step(1) for _ in range(args.steps)]
    runner.close()
    total = sum(times)
    mlups = n ** 3 * args.steps / total / 1e6
    line = {
        "metric": METRIC, "value": round(mlups, 3), "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Taylor-Green + SplitMix64 noise)",
        "config": {"workload": "D3Q19 AA FP64 Taylor-Green periodic box, tau=0.55; each step one lattice "
                               f"step of a {n}^3 sample of the 512^3 box", "lattice": "D3Q19",
                   "propagation": "AA", "grid": [n, n, n], "storage": "f64"},
        "cpu_baseline": {"value": round(mlups, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n}^3 box, {args.steps} timed lattice steps; oracle/lbm_oracle.c "
                                   "(C restatement of the reference's AA kernels, int32 adjacency, OpenMP); "
                                   f"{PORT_VS_REFERENCE}"},
        "e2e": {"value": round(mlups, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    dist, rank, world, local = dist_setup(args)
    if args.impl == "reference":
        return run_reference_arm(args, dist, rank, world)

    import torch
    import lbmminiapp_gb300 as lbm

    if args.accuracy:
        from lbmminiapp_gb300.accuracy import error_table
        t0 = time.perf_counter()
        table = error_table(n=args.n, steps=1000, tau=TAU, device=local)
        print(json.dumps({"accuracy": table, "grid": [args.n] * 3, "steps": 1000, "tau": TAU,
                          "workload": "D3Q19 AA Taylor-Green U=0.05 + 1e-3 noise, errors vs FP64 storage",
                          "seconds": round(time.perf_counter() - t0, 1)}), flush=True)
        return 0

    torch.cuda.set_device(local)
    if args.porous:
        return run_porous(args, local)
    if args.reference_benchmark:
        print(json.dumps(cylinder_benchmark(local, args.cylinder_size, args.cylinder_steps)), flush=True)
        return 0
    if args.configs:
        print(json.dumps(config_benchmarks(local)), flush=True)
        return 0
    if args.spheres:
        print(json.dumps(spheres_benchmark(local, args.spheres)), flush=True)
        return 0
    n = args.n
    ncell = n ** 3
    Q = args.lattice
    u = workload_velocity(n)
    arith = "f64x" if args.storage == "f64" else "auto"
    sim = lbm.Simulation(n, n, n, lattice=Q, pattern=args.pattern, omega=1.0 / TAU, force=(0, 0, 0),
                         storage=args.storage, arithmetic=arith, device=local)
    bpu = int(sim.info.bytes_per_update)
    headline = (args.storage, Q, args.pattern, n) == ("f64", 19, "aa", 512)
    sim.init_equilibrium(None, u)
    for _ in range(max(args.warmup, 3)):
        sim.step(1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev[0].record()
        for k in range(args.steps):
            sim.step(1)
            ev[k + 1].record()
        ev[-1].synchronize()
    torch.cuda.synchronize()
    per_launch_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    if dist:
        total_ms = max_over_ranks(dist, total_ms, "cuda")
        dist.barrier()
    value = world * ncell * args.steps / (total_ms * 1e-3) / 1e6
    mass = float(sim.conserved()[0]) / ncell
    launches = args.steps

    peak, peak_kind = measured_peaks()
    avg_launch_s = statistics.mean(per_launch_ms) * 1e-3
    achieved = ncell * bpu / avg_launch_s / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic_per_launch() if headline else None,
                "peak_kind": f"{peak_kind} copy bandwidth",
                "kernel": (f"step_async_kernel<{Q},{args.pattern}> (F64X, persistent warps, cp.async-prefetched "
                           f"tiles of 32 cells; one launch per step)"
                           if arith == "f64x" and n % 32 == 0 else
                           f"step_kernel<{Q},{args.storage},{arith},{args.pattern}> (one launch per step)"),
                "algorithmic_bytes_per_launch": ncell * bpu}

    # end to end through the C ABI, pinned host buffers
    e2e = None
    if not args.no_e2e:
        steps_e2e = args.e2e_steps
        u_host = torch.empty((3, n, n, n), dtype=torch.float64, pin_memory=True)
        u_host.numpy()[...] = u
        rho_out = torch.empty((n, n, n), dtype=torch.float64, pin_memory=True)
        u_out = torch.empty((3, n, n, n), dtype=torch.float64, pin_memory=True)
        times = []
        for nsteps in (10, steps_e2e):   # a short warm-up round trip, then the timed one
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sim.init_equilibrium(None, u_host.numpy())
            sim.step(nsteps)
            sim.macros(out=(rho_out.numpy(), u_out.numpy()))
            times.append(time.perf_counter() - t0)
        launches_e2e = steps_e2e + 2
        e2e = {"value": round(ncell * steps_e2e / times[-1] / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": 3 * 8 * ncell, "d2h_bytes_per_step": 4 * 8 * ncell,
               "step": f"init_equilibrium(u from pinned host) + {steps_e2e} lattice steps + get_macros "
                       "(rho, u to pinned host)",
               "gpu_launches_per_step": launches_e2e}
        del u_host
    parity = None
    if e2e is not None and arith == "f64x" and Q == 19 and args.pattern == "aa" and world == 1 \
            and not args.no_parity:
        state_x = state_copy(sim)
        sim.close()
        parity = parity_vs_exact(n, u, args.e2e_steps, state_x, rho_out.numpy(), u_out.numpy(), local)
        del state_x
    if e2e is not None:
        del rho_out, u_out
    sim.close()
    del u

    variants = {}
    if not args.no_variants and headline:
        uv = workload_velocity(n)
        for storage, v_arith, steps in [("f16", "auto", 12), ("bf16", "auto", 12), ("f32", "auto", 12),
                                        ("f64", "f64", 3)]:
            s2 = lbm.Simulation(n, n, n, lattice=Q, pattern="aa", omega=1.0 / TAU, force=(0, 0, 0),
                                storage=storage, arithmetic=v_arith, device=local)
            s2.init_equilibrium(None, uv)
            s2.step(2)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            s2.step(steps)
            b.record()
            b.synchronize()
            ms = a.elapsed_time(b) / steps
            bytes_u = s2.info.bytes_per_update
            variants[f"{storage}/{v_arith}"] = {"MLUPS": round(ncell / (ms * 1e-3) / 1e6, 1),
                                              "GB/s": round(ncell * bytes_u / (ms * 1e-3) / 1e9, 1),
                                              "bytes_per_update": bytes_u}
            s2.close()
        del uv

    cylinder, configs = {}, {}
    if not args.no_variants and headline:
        cylinder = cylinder_benchmark(local)
        configs = config_benchmarks(local)

    cpu = None
    if not args.no_cpu and rank == 0:
        sample_n = 128
        mlups_cpu, threads, csteps, csec = cpu_port_mlups(sample_n)
        cpu = {"value": round(mlups_cpu, 3), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{sample_n}^3 box of the same workload, {csteps} lattice steps in {csec:.1f} s; "
                         "oracle/lbm_oracle.c (C restatement of the reference AA kernels, int32 adjacency, "
                         f"OpenMP); {PORT_VS_REFERENCE}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(total_ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 storage, df64 (FP32-pair) arithmetic" if arith == "f64x" else
                     f"{args.storage} storage (f - w), f32 arithmetic",
            "data": "synthetic (seeded Taylor-Green + SplitMix64 noise)",
            "config": {"workload": f"D3Q{Q} BGK {args.pattern.upper()}, {n}^3 periodic box, tau=0.55, "
                                   f"Taylor-Green U=0.05 + uniform 1e-3 noise, {args.storage.upper()} storage",
                       "lattice": f"D3Q{Q}", "propagation": args.pattern, "grid": [n, n, n], "tau": TAU,
                       "storage": args.storage,
                       "arithmetic": "F64X (within 1e-10 of the reference)" if arith == "f64x" else "FP32 on f - w",
                       "l2": f"state {ncell * bpu / 2 / 1e9:.1f} GB >> 129 MB L2 (no flush needed)",
                       "parallelism": "independent replica per GPU" if world > 1 else "1 GPU"},
            "gpu_launches": launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "parity": parity,
            "variants": variants,
            "reference_benchmark": cylinder,
            "configs": configs,
            "mass_per_cell_after": mass,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
