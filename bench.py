#!/usr/bin/env python3
"""Benchmark of the GB300 SPH pipeline: particle-steps/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

Workloads (seeded synthetic scenes; sph/scenes.py):
  wcsph-1m   1,048,576-particle WCSPH slab (128 x 64 x 128 lattice, spacing
             0.005 m, h = 0.01 m, +-5e-5 m jitter) in a [0,1]^3 box, dt = 2e-5 s: the
             plain single-scene drop-in path, one CUDA-graph substep per step
             (default)
  dam-8k     8,000-particle WCSPH dam break (20^3 at 0.01 m, h = 0.02 m) in
             [0,0.4]^3, dt = 1e-4 s
  beam-4k    4,000-particle corotational beam (10x10x40), E = 1e5 Pa,
             nu = 0.3, two clamped layers, dt = 5e-5 s

One JSON line on rank 0.  `value` is device throughput over the K timed
substeps (CUDA events on the store's stream, the L2 flushed by a 256 MB
write between substeps, outside the timed events); `e2e` repeats the
measurement through the C ABI with host buffers (a per-step upload of the
scene parameters and download of all positions into the pinned host
store); `roofline` times each phase of the substep live
(sph_profile_substep) and sets the dominant kernel's algorithmic bytes
against the measured HBM peak; `cpu_baseline` times the CPU oracle on a
bounded sample.  With --impl reference the reference's own kernels
(oracle/_ref, the reference's kernels/*.cl compiled for the host CPU with
OpenMP) -- or, where they were not built, the C restatement -- run the same
workload on all host cores.  N > 1 GPUs run independent replicas (no
collective; the path does not shard), aggregated over ranks.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "opencl-sph_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s on 1 GB300: batched+served vs plain at FP64 err; p50/p99 lat"
UNIT = "particle-steps/s"

# Algorithmic bytes per phase (the reference's FP32 field set, each field
# read or written once per kernel, atomics as 8-byte read-modify-writes):
# (bytes per particle, bytes per cell).  WCSPH total 188 B/particle + 36 B/cell.
PHASE_BYTES = {
    "bin_count": (28, 4),             # find_particle_bins 16 + count 12; zero 4/cell
    "scan": (0, 16),                  # prefix_sum 8 + copy_celloffset_to_backup 8 per cell
    "insert": (16, 0),                # insert_particles_in_bin_array
    "gather": (0, 0),                 # no reference counterpart
    "density": (24, 8),               # compute_density + one stencil pass over the tables
    "forces_fluids+step": (120, 8),   # compute_forces_fluids 44 + step_forward 76
    "rotations_and_strains": (168, 16),
    "deformations": (64, 8),
    "stresses": (48, 0),
    "forces_solids": (160, 8),
    "step_forward": (76, 0),
}


def workload(name, seed):
    from sph import scenes
    if name == "wcsph-1m":
        # 1,048,576 particles (the configuration's count; a 128^3 lattice
        # would hold 2,097,152) as a 128 x 64 x 128 slab, 64 layers high.
        # The reference's fluid force omits the neighbour mass
        # (fluids.cl:43-56), so stiffness and viscosity act per unit particle
        # mass: at 1/8 of the dam break's particle mass they are scaled by
        # 1/8 to keep its sound speed and viscous time (unscaled, the slab
        # blows up within ten substeps).
        return scenes.wcsph_block(128, 64, 128, spacing=0.005, h=0.01, box=(0.0, 1.0), jitter=5e-5, seed=seed,
                                  dt=2e-5, walls=True, stiffness=0.375, viscosity=0.025, name="wcsph-1m"), \
            ("1,048,576-particle WCSPH slab, 128x64x128 at 0.005 m, h=0.01 m, [0,1]^3 box, dt=2e-5 s, "
             "stiffness 0.375, viscosity 0.025 (the dam break's 3 and 0.2 scaled by the 1/8 particle mass)")
    if name == "dam-8k":
        return scenes.wcsph_block(20, 20, 20, seed=seed, name="dam-8k"), \
            "8,000-particle WCSPH dam break, 20^3 at 0.01 m, h=0.02 m, [0,0.4]^3 box, dt=1e-4 s"
    if name == "beam-4k":
        return scenes.solid_lattice(10, 10, 40, material="corot", seed=seed, name="beam-4k"), \
            "4,000-particle corotational beam 10x10x40 at 0.01 m, E=1e5 Pa, nu=0.3, 2 clamped layers, dt=5e-5 s"
    raise SystemExit("unknown workload " + name)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


class Clocks(object):
    """nvidia-smi sampling during the timed region (every 200 ms)."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def setup_store(scene):
    ps = scene.system()
    if scene.material in ("corot", "svk"):
        ps.setup()
    return ps


def _solid_setup(ps):
    ps.call_for_all_particles("init_original_position")
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_original_density")


def run_ours(args, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    from sph import bindings as bnd
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    scene, desc = workload(args.workload, args.seed + rank)
    ps = scene.system()
    if scene.material in ("corot", "svk"):
        _solid_setup(ps)
    n = scene.n
    cells = int(np.prod(ps.get_fields("gridres")[0]))
    ext = torch.cuda.ExternalStream(bnd.sph_stream(ps.psdata_opencl))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # warm-up (also captures the CUDA graph)
    ps.update_fused(max(args.warmup, 1))
    ps.synchronize()
    kernels_per_step = bnd.sph_graph_kernel_count(ps.psdata_opencl)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = Clocks(torch.cuda.current_device())
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    with torch.cuda.stream(ext):
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(ext)
            ps.update_fused(1)
            ends[k].record(ext)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([total_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    status = ps.status()

    # live per-phase device times of the same kernels (roofline)
    maxp = 16
    ms = (ctypes.c_float * maxp)()
    names = (ctypes.c_char_p * maxp)()
    np_ = bnd.sph_profile_substep(ps.psdata_opencl, max(3, min(args.steps, 10)), ms, names, maxp)
    phases = {names[i].decode(): float(ms[i]) for i in range(np_)}

    # end to end through the C ABI with host buffers (pinned host store)
    e2e = run_e2e(ps, scene, args.steps, torch)

    line = None
    if rank == 0:
        peak, peak_kind = measured_peak_gbs()
        dom = max(phases, key=phases.get)
        bp, bc = PHASE_BYTES.get(dom, (0, 0))
        alg_bytes = bp * n + bc * cells
        achieved = alg_bytes / (phases[dom] * 1e-3) / 1e9
        step_alg = 0
        for ph in phases:
            b = PHASE_BYTES.get(ph, (0, 0))
            step_alg += b[0] * n + b[1] * cells
        value = n * args.steps * world / total_s
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": total_s * 1e3 / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded lattice scene, seed %d)" % args.seed,
            "config": {"workload": args.workload + ": " + desc, "particles": n, "cells": cells,
                       "path": "plain single scene, one CUDA-graph substep per step (sph_update)",
                       "l2": "flushed between timed steps (256 MB write, outside the timed events)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "clocks": clk,
            "e2e": e2e,
            "gpu_launches": kernels_per_step * args.steps,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback", "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "step_algorithmic_gbs": step_alg / (sum(phases.values()) * 1e-3) / 1e9,
                         "phase_ms": phases},
            "wall_s": wall,
            "status_word": status,
        }
    ps.close()
    return line


def run_e2e(ps, scene, steps, torch):
    """Per step: upload gravity+timestep from the host store, one substep,
    download every position into the host store (pinned for the run)."""
    from sph import bindings as bnd
    size = bnd.psdata_data_size(ps.psdata)
    cudart = torch.cuda.cudart()
    try:
        registered = int(cudart.cudaHostRegister(ps.psdata.data, size, 0)) == 0
    except Exception:
        registered = False
    names_in = ("gravity", "timestep")
    t0 = time.perf_counter()
    for _ in range(steps):
        ps.sync_fields_host_to_device(*names_in)
        ps.update_fused(1)
        ps.sync_fields_device_to_host("position")
    el = time.perf_counter() - t0
    if registered:
        cudart.cudaHostUnregister(ps.psdata.data)
    return {"value": scene.n * steps / el, "unit": UNIT, "h2d_bytes_per_step": 12 + 4,
            "d2h_bytes_per_step": 12 * scene.n, "host_memory": "pinned" if registered else "pageable"}


def cpu_sample(scene, material, steps, nthreads, reference):
    """Times the CPU oracle (or the reference's own kernels) on `steps`
    substeps of the scene; returns particle-steps/s."""
    from sph import bindings as bnd
    from sph import init_data_cpu, free_data_cpu
    ps = init_data_cpu(scene.spec)
    v = bnd.store_views(ps)
    for k, val in scene.init.items():
        v[k][...] = val
    kind = "port"
    if reference:
        from oracle import ref
        if ref.available():
            kind = "reference"
    if kind == "reference":
        from oracle import ref
        rs = ref.RefStore(scene.spec)
        for k in scene.init:
            rs.view(k)[...] = v[k]
        prog = {"fluid": "fluid", "corot": "corot", "svk": "svk"}[material]
        rec = {"fluid": ["compute_density", "compute_forces_fluids"],
               "corot": ["compute_density", "compute_rotations_and_strains", "compute_stresses",
                         "compute_forces_solids"],
               "svk": ["compute_density", "compute_deformations", "compute_stresses", "compute_forces_solids"]}[
            material]

        def one():
            rs.call(prog, "f32", "compute_particle_bins", scene.n, nthreads)
            for k in rec:
                rs.call(prog, "f32", k, scene.n, nthreads)
            rs.call(prog, "f32", "step_forward", scene.n, nthreads)
        if material != "fluid":
            for k in ("init_original_position", "compute_particle_bins", "compute_original_density"):
                rs.call(prog, "f32", k, scene.n, nthreads)
    else:
        from oracle.oracle import OracleScene
        orc = OracleScene(v, "f32", nthreads=nthreads)
        if material != "fluid":
            orc.setup_solid()

        def one():
            orc.substep(material)
    one()  # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    el = time.perf_counter() - t0
    free_data_cpu(ps)
    return scene.n * steps / el, kind, el


def run_reference(args, rank, world):
    if rank != 0:
        return None
    scene, desc = workload(args.workload, args.seed)
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        pass
    value, kind, el = cpu_sample(scene, scene.material, args.steps, nthreads, reference=True)
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded lattice scene, seed %d)" % args.seed,
        "config": {"workload": args.workload + ": " + desc, "particles": scene.n},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": kind,
                         "sample": "%d full substeps of the workload" % args.steps},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="wcsph-1m")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-steps", type=int, default=3, help="substeps in the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return 0
    line = run_ours(args, rank, world, local_rank)
    if line is not None:
        if world == 1 and not args.no_cpu_baseline:
            scene, _ = workload(args.workload, args.seed)
            nthreads = os.cpu_count() or 1
            v, kind, el = cpu_sample(scene, scene.material, args.cpu_steps, nthreads, reference=False)
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nthreads, "kind": kind,
                                    "sample": "%d substeps of the full workload on the C oracle (%.1f s)"
                                              % (args.cpu_steps, el)}
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
