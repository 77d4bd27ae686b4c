#!/usr/bin/env python3
"""Benchmark of the GB300 SPH pipeline: particle-steps/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

Workloads (seeded synthetic scenes; sph/scenes.py):
  batched-256  256 independent scenes (60% WCSPH, 25% corotational, 15% SVK,
               1,000-65,536 particles each, log-uniform) advanced together,
               one CUDA graph per substep (default: the headline metric is
               the batched/served form against the plain per-scene loop)
  large-scene  one interacting scene: 1,048,576 WCSPH particles, a 32^3
               SVK cube resting on them and a rigid ball dropped beside it
               (the mixed fluid-solid extension), through the drop-in
  wcsph-1m     1,048,576-particle WCSPH slab (128 x 64 x 128 at 0.005 m,
               h = 0.01 m) in [0,1]^3: the plain single-scene drop-in path
  dam-8k       8,000-particle WCSPH dam break (20^3 at 0.01 m, h = 0.02 m)
  beam-4k      4,000-particle corotational beam (10x10x40), E = 1e5 Pa

One JSON line on rank 0.  `value` is device throughput over the K timed
substeps (CUDA events on the work's stream; plain scenes flush the L2 with a
256 MB write between substeps, outside the events; the batched working set
exceeds the L2).  `e2e` repeats the measurement through the public API with
host buffers (per step: the step's inputs -- time step and gravity -- written
from the host stores, the substep, then every scene's positions read into
its host store).  `roofline` sets the dominant phase's algorithmic bytes
against the measured HBM peak (phase times from live CUDA events).
`cpu_baseline` times the CPU oracle on a bounded sample.  The default run
also reports the batch after 500 more substeps, the plain per-scene loop,
the stated SVK stiffness mix, the error against the FP64 oracle (small
scenes, the dam break, the beam and the 1M slab after 1,000 substeps), the
served stream (60 s of 50 requests/s, p50/p99) beside the plain loop
measured one request at a time, the plain 1M slab and the large interacting
scene.  With --impl reference the reference's own kernels (oracle/_ref, the
reference's kernels/*.cl compiled for the host CPU with OpenMP, in stores the
reference's own builder made) run the same workload on all host cores; that
arm loads neither the sph package nor the CUDA library.  N > 1 GPUs run
independent replicas (no collective; scenes do not shard), aggregated over
ranks.
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
    # fused solid phases: the first pass also applies the stress law, the
    # force pass also steps (separate stress and step phases only for
    # scenes with symmetry planes)
    "rotations_and_strains": (216, 16),  # 168 + compute_stresses 48
    "deformations": (124, 8),            # 64 + compute_stresses 60
    "stresses": (48, 0),
    "forces_solids+step": (236, 8),      # compute_forces_solids 160 + step_forward 76
    "step_forward": (76, 0),
    # batched-form phases (bench_batched): the same figures per material
    "fluid forces+step": (120, 8),
    "corotational rotations": (216, 16),
    "corotational stresses": (48, 0),
    "corotational forces+step": (236, 8),
    "corotational step (planes)": (76, 0),
    "svk deformations": (124, 8),
    "svk stresses": (60, 0),
    "svk forces+step": (200, 8),         # 124 + 76
    "svk step (planes)": (76, 0),
    "corotational density (planes)": (24, 8),
    "svk density (planes)": (24, 8),
}

# DRAM traffic per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
# the dominant phase's kernel, from one ncu capture of that kernel alone
# (one launch after two warm-up substeps, `bench.py --quick --steps 2
# --warmup 3` of the same workload), taken with the register caps and
# kernels of this source: k_rotations_and_strains at 64 registers (its
# spills add DRAM traffic), k_deformations uncapped (80), the solid force
# passes at 80, the fluid force pass at 64; the density and fluid force passes with their sums blocked per cell
# row; distance tests and the fluid pair term in packed FP32x2 instructions.
MEASURED_TRAFFIC = {
    ("wcsph-1m", "density"): 45.20e6,                           # k_density<false>
    ("wcsph-1m", "forces_fluids+step"): 116.82e6,               # k_forces_fluids_masked<false>
    ("batched-256", "density"): 262.97e6,                       # k_density<false> (masks, pressure, 1/density too)
    ("batched-256", "fluid forces+step"): 365.65e6,             # k_forces_fluids_masked<false>
    ("batched-256", "corotational rotations"): 285.09e6,        # k_rotations_and_strains (with the stress law)
    ("batched-256", "corotational forces+step"): 241.63e6,      # k_forces_solids<1, 1> (with the step)
    ("batched-256", "svk deformations"): 105.53e6,              # k_deformations (with the stress law)
    ("batched-256", "svk forces+step"): 161.73e6,               # k_forces_solids<0, 1> (with the step)
}

# Warp instructions per launch of the same kernels (ncu
# smsp__inst_executed.sum, same captures as the traffic above): with the
# live phase time they give the issue rate, against 4 warp instructions per
# SM per clock.
MEASURED_INST = {
    ("wcsph-1m", "density"): 169.65e6,
    ("wcsph-1m", "forces_fluids+step"): 141.36e6,
    ("batched-256", "density"): 430.89e6,
    ("batched-256", "fluid forces+step"): 363.75e6,
    ("batched-256", "corotational rotations"): 454.02e6,
    ("batched-256", "corotational forces+step"): 260.60e6,
    ("batched-256", "svk deformations"): 347.92e6,
    ("batched-256", "svk forces+step"): 259.39e6,
}


def scenes_module(standalone=False):
    """The scene builders.  `standalone`: sph/scenes.py loaded on its own,
    without the sph package, whose import loads the CUDA library -- the
    reference arm builds the same scenes while mapping only the reference's
    own CPU libraries."""
    if not standalone:
        from sph import scenes
        return scenes
    import importlib.util
    name = "sph_scenes_standalone"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, os.path.join(PKG, "sph", "scenes.py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def workload(name, seed, standalone=False):
    scenes = scenes_module(standalone)
    if name == "wcsph-1m":
        return scenes.wcsph_slab_1m(seed), \
            ("1,048,576-particle WCSPH slab, 128x64x128 at 0.005 m, h=0.01 m, [0,1]^3 box, dt=2e-5 s, "
             "stiffness 0.375, viscosity 0.025 (the dam break's 3 and 0.2 scaled by the 1/8 particle mass)")
    if name == "dam-8k":
        return scenes.wcsph_block(20, 20, 20, seed=seed, name="dam-8k"), \
            "8,000-particle WCSPH dam break, 20^3 at 0.01 m, h=0.02 m, [0,0.4]^3 box, dt=1e-4 s"
    if name == "batched-256":
        raise SystemExit("batched-256 has no single scene")
    if name == "large-scene":
        return scenes.large_fluid_solid_scene(seed), \
            ("large interacting scene: 1,048,576 WCSPH particles (128x64x128 at 0.005 m, h=0.01 m, [0,1]^3, "
             "dt=2e-5 s, stiffness 0.375, viscosity 0.025), a 32^3 SVK cube (E=5e4 Pa, nu=0.35) resting on the "
             "fluid and a rigid ball of radius 0.05 m (4,169 particles, body_dynamic 2) dropped beside it, all "
             "in one store (mixed fluid-solid extension)")
    if name == "beam-4k":
        return scenes.solid_lattice(10, 10, 40, material="corot", seed=seed, name="beam-4k"), \
            "4,000-particle corotational beam 10x10x40 at 0.01 m, E=1e5 Pa, nu=0.3, 2 clamped layers, dt=5e-5 s"
    raise SystemExit("unknown workload " + name)


def aggregate_replicas(n_local, steps, seconds_local, world, device="cpu"):
    """Whole-job throughput of independent replicas: every rank's particles
    times the substeps, over the slowest rank's time.  Returns (value,
    max_seconds); needs an initialised process group when world > 1."""
    if world <= 1:
        return n_local * steps / seconds_local, seconds_local
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds_local], dtype=torch.float64, device=device)
    n = torch.tensor([float(n_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(n.item()) * steps / float(t.item()), float(t.item())


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


class Clocks(object):
    """nvidia-smi sampling during the timed region (every 50 ms; start()
    returns once the first sample is in, so the sampler is live when the
    timed region begins)."""
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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.005)

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


def _solid_setup(ps):
    ps.call_for_all_particles("init_original_position")
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_original_density")


def _issue_roofline(phases, workload, clocks):
    """The instruction-issue limit of each captured phase kernel: its warp
    instructions per launch over its live time, against 4 warp instructions
    per SM per clock at the SM clock sampled under load."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not mhz:
        return None
    peak = 4.0 * sms * mhz * 1e6 / 1e12
    per = {}
    for ph, ms in phases.items():
        inst = MEASURED_INST.get((workload, ph))
        if inst and ms:
            a = inst / (ms * 1e-3) / 1e12
            per[ph] = {"achieved": a, "frac": a / peak, "warp_instructions_per_launch": inst}
    return {"unit": "T warp-instructions/s", "peak": peak, "sm_mhz": mhz, "sms": sms, "phases": per,
            "source": "instruction counts from ncu captures of the same kernels, times live"}


def _phase_roofline(phases, n, cells, peak, peak_kind, counts=None, workload=None, clocks=None):
    """Roofline of the phase that takes longest: its algorithmic bytes (for
    the particles and cells it processes) over its measured time; traffic is
    the measured DRAM bytes of that phase's kernel where captured.  `issue`
    sets the pair kernels against the instruction-issue limit that binds
    them."""
    dom = max(phases, key=phases.get)
    bp, bc = PHASE_BYTES.get(dom, (0, 0))
    pn, pc = (counts or {}).get(dom, (n, cells))
    alg = bp * pn + bc * pc
    achieved = alg / (phases[dom] * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "traffic": MEASURED_TRAFFIC.get((workload, dom)),
            "algorithmic_bytes_per_launch": alg, "phase_ms": phases,
            "issue": _issue_roofline(phases, workload, clocks)}


def bench_plain(args, scene, torch, world):
    """The drop-in path on one scene: K CUDA-graph substeps (sph_update)."""
    from sph import bindings as bnd
    ps = scene.system()
    if scene.material != "fluid":
        _solid_setup(ps)
    n = scene.n
    cells = int(np.prod(ps.get_fields("gridres")[0]))
    ext = torch.cuda.ExternalStream(bnd.sph_stream(ps.psdata_opencl))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
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
    with torch.cuda.stream(ext):
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(ext)
            ps.update_fused(1)
            ends[k].record(ext)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    total_s = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / 1e3
    maxp = 16
    ms = (ctypes.c_float * maxp)()
    names = (ctypes.c_char_p * maxp)()
    k = bnd.sph_profile_substep(ps.psdata_opencl, max(3, min(args.steps, 10)), ms, names, maxp)
    phases = {names[i].decode(): float(ms[i]) for i in range(k)}
    e2e = run_e2e(ps, scene, args.steps, torch)
    status = ps.status()
    pairs = pair_counts(ps)
    ps.close()
    return {"n": n, "cells": cells, "total_s": total_s, "clocks": clk, "phases": phases, "e2e": e2e,
            "status": status, "kernels_per_step": kernels_per_step, "pairs": pairs}


# The reference drivers' update recipes (scripts/sph/systems.py:113-189),
# kernel by kernel through call_for_all_particles after
# compute_particle_bins.
NAMED_RECIPES = {
    "fluid": ("compute_density", "compute_forces_fluids", "step_forward"),
    "corot": ("compute_density", "compute_rotations_and_strains", "compute_stresses", "compute_forces_solids",
              "step_forward"),
    "svk": ("compute_density", "compute_deformations", "compute_stresses", "compute_forces_solids",
            "step_forward"),
    # the mixed-scene extension's recipe (the solids' elastic passes, then
    # the fluid force pass, which adds the fluid pair terms)
    "mixed": ("compute_density", "compute_deformations", "compute_stresses", "compute_forces_solids",
              "compute_forces_fluids", "step_forward"),
}


def bench_named(args, scene, torch):
    """The drop-in's named path, the one an unmodified reference driver
    takes: per substep compute_particle_bins and the material's kernels by
    name (each pair call re-gathers the sorted copies from the fields and
    scans the stencil; no masks), on the same scene as the fused substep.
    Device time with CUDA events on the store's stream, L2 flushed between
    substeps as for the fused line."""
    from sph import bindings as bnd
    ps = scene.system()
    if scene.material != "fluid":
        _solid_setup(ps)
    recipe = NAMED_RECIPES[scene.material]

    def substep():
        ps.compute_particle_bins()
        for k in recipe:
            ps.call_for_all_particles(k)

    ext = torch.cuda.ExternalStream(bnd.sph_stream(ps.psdata_opencl))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(args.warmup, 1)):
        substep()
    ps.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    with torch.cuda.stream(ext):
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(ext)
            substep()
            ends[k].record(ext)
    torch.cuda.synchronize()
    total_s = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / 1e3
    status = ps.status()
    ps.close()
    return {"value": scene.n * args.steps / total_s, "unit": UNIT, "ms_per_step": total_s * 1e3 / args.steps,
            "status": status, "recipe": ["compute_particle_bins"] + list(recipe),
            "how": "the reference driver's update() recipe by name (call_for_all_particles per kernel), "
                   "CUDA events on the store's stream, L2 flushed between substeps"}


def pair_counts(ps):
    """Pair evaluations of one substep of the store's current state: stencil
    candidates (every particle against the 27 cells around its own, from
    the cell counts) and neighbours within h (num_neighbours, self
    included)."""
    ps.sync_device_to_host()
    res = [int(x) for x in np.ravel(ps.get_fields("gridres")[0])]
    cnt = np.asarray(ps.get_fields("gridcount")[0], dtype=np.int64).reshape(res[2], res[1], res[0])
    box = np.pad(cnt, 1)
    acc = np.zeros_like(cnt)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                acc += box[dz:dz + res[2], dy:dy + res[1], dx:dx + res[0]]
    n = int(np.ravel(ps.get_fields("n")[0])[0])
    return {"candidates": int((cnt * acc).sum()),
            "neighbours": int(np.asarray(ps.get_fields("num_neighbours")[0][:n], dtype=np.int64).sum())}


def run_e2e(ps, scene, steps, torch):
    """Per step, through the store's public API: upload gravity+timestep from
    the host store, one substep, and a read of every position into the host
    store (pinned for the run).  Transfers are pipelined: each step's read
    runs on the copy engines while the next substep computes, and the host
    waits for it one step later; the last read is waited for inside the
    timed region."""
    ps.pin()
    t0 = time.perf_counter()
    prev = None
    for _ in range(steps):
        ps.write_fields_async("gravity", "timestep")
        ps.update_fused(1)
        t = ps.read_fields_async("position")
        if prev is not None:
            ps.wait_read(prev)
        prev = t
    ps.wait_read(prev)
    el = time.perf_counter() - t0
    ps.unpin()
    return {"value": scene.n * steps / el, "unit": UNIT, "h2d_bytes_per_step": 12 + 4,
            "d2h_bytes_per_step": 12 * scene.n, "host_memory": "pinned", "transfers": "pipelined"}


def batched_scenes(seed, workload="batched-256", standalone=False):
    return scenes_module(standalone).batch_mix(256, seed=seed)


BATCHED_WORKLOADS = ("batched-256",)


def bench_batched(args, torch, world):
    """256 uneven scenes (60% WCSPH, 25% corotational, 15% SVK) advanced
    together: one CUDA graph per substep over all scenes."""
    from sph.batch import Batch
    from sph import autotune
    scs = batched_scenes(args.seed, args.workload)
    tuned = None
    if not args.quick and args.workload == "batched-256":
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        cands = [(b_, p_, c_) for b_ in (128, 256) for p_ in (64, 128, 256) for c_ in (0, 4 * sms, 8 * sms)]
        best, best_s, table = autotune.tune(scs, steps=3, cands=cands)
        default_s = dict(table).get((256, 128, 0))
        tuned = {"block": best[0], "pair_block": best[1], "grid_cap": best[2], "candidates": len(table),
                 "best_ms_per_step": best_s * 1e3,
                 "default_ms_per_step": default_s * 1e3 if default_s else None}
    b = Batch()
    if tuned:
        b.tune(tuned["block"], tuned["pair_block"], tuned["grid_cap"])
    ids = [b.add(s) for s in scs]
    n = sum(s.n for s in scs)
    ext = torch.cuda.ExternalStream(b.stream)
    b.step(max(args.warmup, 1))
    b.synchronize()
    kernels_per_step = b.kernels_per_step
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = Clocks(torch.cuda.current_device())
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    with torch.cuda.stream(ext):
        for k in range(args.steps):
            starts[k].record(ext)
            b.step(1)
            ends[k].record(ext)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    total_s = sum(a.elapsed_time(e) for a, e in zip(starts, ends)) / 1e3
    phases = b.profile(reps=max(3, min(args.steps, 10)))
    # end to end: per step, one batched substep and every scene's positions
    # written into its host store.  The stores are pinned through the batch;
    # each step's positions are snapshot on the device and written to the
    # host while the next substep runs, and the loop waits for step s - 1's
    # positions to be on the host before it enqueues step s + 1.
    for sid in ids:
        b.pin(sid)
    b.wait_read(b.read_fields_async(ids, "position"))  # allocates the read buffers
    b.write_fields_async(ids, "timestep", "gravity")
    b.synchronize()
    h2d = sum(16 + 16 for _ in ids) + (2 * len(ids) * 24 + 255) // 256 * 256  # fields + segment table
    t0 = time.perf_counter()
    prev = None
    for _ in range(args.steps):
        # each step's inputs: every scene's time step and gravity from its
        # host store (one staged copy, scattered on the device)
        b.write_fields_async(ids, "timestep", "gravity")
        b.step(1)
        t = b.read_fields_async(ids, "position")
        if prev is not None:
            b.wait_read(prev)
        prev = t
    b.wait_read(prev)
    e2e_s = time.perf_counter() - t0
    for sid in ids:
        b.unpin(sid)
    # away from the lattice start: the same batch after 500 more substeps
    late = None
    if not args.quick:
        b.step(500)
        b.synchronize()
        ls = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        with torch.cuda.stream(ext):
            ls[0].record(ext)
            b.step(args.steps)
            ls[1].record(ext)
        torch.cuda.synchronize()
        late_s = ls[0].elapsed_time(ls[1]) / 1e3
        late = {"value": n * args.steps / late_s, "ms_per_step": late_s * 1e3 / args.steps,
                "substeps_before": max(args.warmup, 1) + 2 * args.steps + 500 + 1,
                "scenes_with_bad_status": sum(1 for sid in ids if b.status(sid) != 0),
                "how": "the headline batch timed again (CUDA events) after 500 further substeps"}
    status = sum(1 for sid in ids if b.status(sid) != 0)
    cells = 0
    by_mat = {"fluid": [0, 0], "corot": [0, 0], "svk": [0, 0]}
    for sid in ids:
        c = int(np.prod(b.scenes[sid].views["gridres"]))
        cells += c
        m = b.scenes[sid].scene.material
        by_mat[m][0] += b.scenes[sid].scene.n
        by_mat[m][1] += c
    # the density pass covers the fluid scenes (a plane-free solid's first
    # pass sums its own density)
    counts = {"fluid forces+step": tuple(by_mat["fluid"]), "density": tuple(by_mat["fluid"])}
    for ph in ("rotations", "stresses", "forces+step", "step (planes)"):
        counts["corotational " + ph] = tuple(by_mat["corot"])
    for ph in ("deformations", "stresses", "forces+step", "step (planes)"):
        counts["svk " + ph] = tuple(by_mat["svk"])
    b.close()
    return {"scenes": scs, "n": n, "cells": cells, "counts": counts, "total_s": total_s, "clocks": clk,
            "phases": phases, "tuned": tuned, "late": late,
            "kernels_per_step": kernels_per_step, "status_scenes": status,
            "e2e": {"value": n * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 12 * n,
                    "host_memory": "pinned (sph_batch_pin_host; a page-locked staging buffer for the writes)",
                    "writes": "per step: every scene's time step and gravity from its host store, staged in "
                              "page-locked memory and scattered into the scenes by one kernel that reads it "
                              "(sph_batch_write_fields_many_async)",
                    "reads": "per step: device snapshot of every scene's positions, written to the host stores "
                             "beside the next substep (sph_batch_read_field_many_async); step s - 1's positions "
                             "are on the host before step s + 1 is enqueued"}}


def bench_plain_loop(scs, steps):
    """The plain per-scene loop: the scenes one after another through the
    drop-in path.  Two forms: `synced` runs one sph_update substep at a time
    and waits for it (the reference's blocking calls); `graph` runs each
    scene's substeps as one sph_update call and waits once per scene."""
    systems = []
    for s in scs:
        ps = s.system()
        if s.material in ("corot", "svk"):
            _solid_setup(ps)
        ps.update_fused(1)
        ps.synchronize()
        systems.append(ps)
    t0 = time.perf_counter()
    for _ in range(steps):
        for ps in systems:
            ps.update_fused(1)
            ps.synchronize()
    synced = time.perf_counter() - t0
    t0 = time.perf_counter()
    for ps in systems:
        ps.update_fused(steps)
        ps.synchronize()
    graph = time.perf_counter() - t0
    for ps in systems:
        ps.close()
    n = sum(s.n for s in scs)
    return {"synced": n * steps / synced, "graph": n * steps / graph}


def sequential_plain(requests):
    """The plain per-scene loop on requests, one at a time through the
    drop-in path as a reference driver would serve them: build the store
    (device lattice scenes on the host), set up solids, sph_update for the
    request's substeps, read the positions back, free.  Returns each
    request's measured service time (seconds)."""
    import torch  # noqa: F401  (the CUDA context is up already)
    out = []
    for r in requests:
        t0 = time.perf_counter()
        ps = r.scene.system()
        if r.scene.material != "fluid":
            _solid_setup(ps)
        ps.update_fused(r.steps)
        ps.sync_fields_device_to_host("position")
        ps.close()
        out.append(time.perf_counter() - t0)
    return out


def _chunk_profile(log):
    """Chunks binned by resident particles: particle-steps/s in each bin."""
    bins = {}
    for resident, scenes, chunk, advanced, dt in log:
        key = "%dM" % min(8, int(resident / 1e6))
        b = bins.setdefault(key, [0, 0.0, 0.0, 0])
        b[0] += 1
        b[1] += advanced
        b[2] += dt
        b[3] += scenes
    return {k: {"chunks": v[0], "particle_steps_per_s": v[1] / v[2] if v[2] else 0.0,
                "mean_scenes": v[3] / v[0]} for k, v in sorted(bins.items())}


def bench_served(args):
    """Poisson arrivals at 50 requests/s for `served_seconds`; each request a
    scene of the batched mix with 2,000-262,144 particles (log-uniform) and
    100-2,000 substeps (uniform); continuous batching under a 150 GB budget.
    Beside it, the plain per-scene loop measured one request at a time on a
    seeded 5% subsample of the same requests."""
    import math  # noqa: F401
    from sph import scenes
    from sph.serving import Server, poisson_requests, release, sequential_fifo

    def make(rng, i):
        # built on the device at admission (sph_batch_add_lattice)
        return scenes.mixed_scene(rng, i, n_range=(2000, 262144), prefix="q", jitter_hash=True)
    reqs = poisson_requests(rate=50.0, duration=args.served_seconds, make_scene=make, steps_range=(100, 2000),
                            seed=args.seed)
    srv = Server(budget_bytes=150e9, max_chunk=args.served_chunk, max_particles=8 << 20, keep_results=False)
    srv.prepare(reqs)
    st = srv.run(reqs, realtime=True)
    demand = sum(r.work for r in reqs) / args.served_seconds
    release(reqs)
    # the sequential plain loop, measured: every 20th request (seeded start)
    rng = np.random.default_rng(args.seed + 1)
    first = int(rng.integers(20))
    sub = [r for r in reqs if r.id % 20 == first]
    service = sequential_plain(sub)
    seq_work = float(sum(r.work for r in sub))
    seq_tput = seq_work / float(sum(service))
    svc = dict(zip([r.id for r in sub], service))
    # the subsample's own arrivals served one at a time with the measured times
    seq_sub = sequential_fifo(sub, lambda r: svc[r.id])
    return {"requests": st["requests"], "arrival_rate_per_s": 50.0, "window_s": args.served_seconds,
            "throughput": st["throughput"], "p50_s": st["p50_s"], "p99_s": st["p99_s"],
            "makespan_s": st["makespan_s"], "peak_resident": st["peak_resident"],
            "peak_particles": st["peak_particles"], "chunks": st["chunks"], "gpu_busy_s": st["gpu_busy_s"],
            "busy_throughput": st["busy_throughput"], "chunk_profile": _chunk_profile(st["chunk_log"]),
            "requests_with_bad_status": st["status_failed"],
            "offered_load": demand, "saturated": bool(demand > st["throughput"]),
            "policy": "FIFO admission by 150 GB HBM budget and 8M resident particles; scenes built on the "
                      "device at admission; device-side substep quotas; chunks of up to %d substeps"
                      % args.served_chunk,
            "sequential_plain": {
                "throughput": seq_tput, "requests_measured": len(sub),
                "particle_steps_measured": seq_work, "seconds_measured": float(sum(service)),
                "served_vs_sequential": st["throughput"] / seq_tput,
                "subsample_fifo": {"p50_s": seq_sub["p50_s"], "p99_s": seq_sub["p99_s"],
                                   "makespan_s": seq_sub["makespan_s"]},
                "how": "every 20th request of the same stream (seeded), served one at a time through the "
                       "drop-in path (store built, solids set up, sph_update for the request's substeps, "
                       "positions read back, store freed), each timed on the host; throughput = their "
                       "particle-steps over the summed service times; subsample_fifo = the subsample's own "
                       "arrivals (2.5 requests/s) served one at a time with the measured times"}}


def fp64_error_sample(scs, steps):
    """Relative L2 position error of batched FP32 results against the
    all-FP64 oracle run, on the smallest scene of each material."""
    from sph.batch import Batch
    from sph import bindings as bnd
    from oracle.oracle import OracleScene
    picks = {}
    for s in sorted(scs, key=lambda s: s.n):
        picks.setdefault(s.material, s)
    out = {}
    b = Batch()
    ids = {m: b.add(s) for m, s in picks.items()}
    b.step(steps)
    for m, s in picks.items():
        host = Batch.host_store(s)
        o = OracleScene(bnd.store_views(host), "f64", nthreads=os.cpu_count() or 1)
        if m != "fluid":
            o.setup_solid()
        o.run(m, steps)
        p = b.read(ids[m])["position"][: s.n].astype(np.float64)
        q = o.a["position"][: s.n]
        out[m] = {"scene": s.name, "particles": s.n, "rel_l2": float(np.linalg.norm(p - q) / np.linalg.norm(q))}
        from sph import free_data_cpu
        free_data_cpu(host)
    b.close()
    return {"substeps": steps, "per_material": out}


def fp64_error_configs():
    """The plain drop-in (FP32, fused CUDA-graph substeps) against the
    all-FP64 oracle run of the same scene, on the two configurations the
    accuracy target is stated for: the 8,000-particle dam break after 1,000
    substeps and the 4,000-particle corotational beam after 2,000."""
    from sph import bindings as bnd
    from sph import free_data_cpu
    from oracle.oracle import OracleScene
    out = {}
    for name, steps in (("dam-8k", 1000), ("beam-4k", 2000)):
        sc, _ = workload(name, 0)
        ps = sc.system()
        o = OracleScene(bnd.store_views(ps.psdata), "f64", nthreads=os.cpu_count() or 1)
        if sc.material != "fluid":
            _solid_setup(ps)
            o.setup_solid()
        ps.update_fused(steps)
        o.run(sc.material, steps)
        ps.sync_device_to_host()
        p = np.asarray(ps.get_fields("position")[0][: sc.n], dtype=np.float64)
        q = o.a["position"][: sc.n]
        out[name] = {"substeps": steps, "particles": sc.n,
                     "rel_l2": float(np.linalg.norm(p - q) / np.linalg.norm(q)),
                     "max_abs_m": float(np.max(np.abs(p - q)))}
        ps.close()
    return out


def exact_mix(args, torch):
    """The batched configuration's mix as stated -- SVK stiffness log-uniform
    over the whole [1e4, 1e6] Pa -- advanced 500 substeps, then timed over
    `steps` more (CUDA events); reports the scenes whose status word is set
    (non-finite positions: the reference's SVK formulation diverges above
    about 1e5 Pa)."""
    from sph import scenes
    from sph.batch import Batch
    scs = scenes.batch_mix(256, seed=args.seed, svk_e_range=(1e4, 1e6))
    b = Batch()
    ids = [b.add(x) for x in scs]
    n = sum(x.n for x in scs)
    b.step(500)
    b.synchronize()
    ext = torch.cuda.ExternalStream(b.stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    with torch.cuda.stream(ext):
        ev[0].record(ext)
        b.step(args.steps)
        ev[1].record(ext)
    torch.cuda.synchronize()
    sec = ev[0].elapsed_time(ev[1]) / 1e3
    bad = [x.name for x, sid in zip(scs, ids) if b.status(sid) != 0]
    svk = [x for x in scs if x.material == "svk"]
    b.close()
    return {"value": n * args.steps / sec, "unit": UNIT, "ms_per_step": sec * 1e3 / args.steps,
            "substeps_before": 500, "svk_e_range_pa": [1e4, 1e6], "svk_scenes": len(svk),
            "scenes_with_bad_status": len(bad), "bad_scenes": bad[:20],
            "how": "the 256-scene mix of the headline with SVK stiffness drawn from the stated [1e4, 1e6] Pa"}


def fp64_error_1m(seed):
    """The plain 1,048,576-particle WCSPH slab through the drop-in (FP32,
    fused CUDA-graph substeps) after 1,000 substeps, against the FP64
    oracle run of the same scene on all host cores."""
    from sph import bindings as bnd
    from oracle.oracle import OracleScene
    sc, _ = workload("wcsph-1m", seed)
    ps = sc.system()
    o = OracleScene(bnd.store_views(ps.psdata), "f64", nthreads=os.cpu_count() or 1)
    ps.update_fused(1000)
    t0 = time.perf_counter()
    o.run("fluid", 1000)
    oracle_s = time.perf_counter() - t0
    ps.sync_device_to_host()
    p = np.asarray(ps.get_fields("position")[0][: sc.n], dtype=np.float64)
    q = o.a["position"][: sc.n]
    out = {"substeps": 1000, "particles": sc.n, "rel_l2": float(np.linalg.norm(p - q) / np.linalg.norm(q)),
           "max_abs_m": float(np.max(np.abs(p - q))), "status": int(ps.status()),
           "fp64_oracle_seconds": oracle_s, "target": 1e-4}
    ps.close()
    return out


def _fill(view, val):
    arr = np.asarray(val)
    if arr.size > 1:
        view[tuple(slice(None, d) for d in arr.shape)] = arr.reshape(arr.shape)
    else:
        view[...] = arr


def cpu_sample(scene, material, steps, nthreads, reference, warmup=1):
    """Times the CPU oracle (or, with `reference`, the reference's own
    kernels in a store the reference's own builder made) on `steps`
    substeps of the scene, after `warmup` untimed ones (at least one);
    returns (particle-steps, seconds, kind)."""
    kind = "port"
    if reference:
        from oracle import ref
        if ref.available():
            kind = "reference"
    if kind == "reference":
        from oracle import ref
        rs = ref.RefStore(scene.spec)
        for k, val in scene.init.items():
            _fill(rs.view(k), val)
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
        closer = rs.free
    else:
        from sph import bindings as bnd
        from sph import init_data_cpu, free_data_cpu
        from oracle.oracle import OracleScene
        ps = init_data_cpu(scene.spec)
        v = bnd.store_views(ps)
        for k, val in scene.init.items():
            _fill(v[k], val)
        orc = OracleScene(v, "f32", nthreads=nthreads)
        if material != "fluid":
            orc.setup_solid()

        def one():
            orc.substep(material)

        def closer():
            free_data_cpu(ps)
    for _ in range(max(1, warmup)):
        one()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    el = time.perf_counter() - t0
    closer()
    return scene.n * steps, el, kind


def cpu_workload(name, seed, standalone=False):
    if name in BATCHED_WORKLOADS:
        return batched_scenes(seed, name, standalone)
    return [workload(name, seed, standalone)[0]]


BATCHED_DESC = ("256 independent scenes, 60% WCSPH / 25% corotational / 15% SVK, particle counts log-uniform in "
                "[1,000, 65,536], E log-uniform [1e4, 1e6] Pa (SVK [1e4, 1e5]: the reference's SVK diverges "
                "within 2,000 substeps above; the stated range is the exact_mix extra), Poisson uniform "
                "[0.25, 0.45], 0.01 m spacing, h=0.02 m, seeded jitter")


def workload_config(name, seed, standalone=False):
    """The line's `config`, the same in both arms: the workload, its size
    and how the L2 is kept out of the timing."""
    if name in BATCHED_WORKLOADS:
        scs = batched_scenes(seed, name, standalone)
        n = sum(x.n for x in scs)
        return {"workload": name + ": " + BATCHED_DESC, "particles": n, "scenes": len(scs),
                "l2": "working set %.2f GB > L2 (129 MB); no flush needed" % (n * 300e-9)}
    sc, desc = workload(name, seed, standalone)
    return {"workload": name + ": " + desc, "particles": sc.n, "scenes": 1,
            "l2": "flushed between timed steps (256 MB write, outside the timed events)"}


def _plain_extra(args, name, torch, peak, peak_kind, named=False):
    sc, desc = workload(name, args.seed)
    p = bench_plain(args, sc, torch, 1)
    out = {"workload": name + ": " + desc, "value": p["n"] * args.steps / p["total_s"],
           "ms_per_step": p["total_s"] * 1e3 / args.steps, "clocks": p["clocks"], "status": p["status"],
           "kernels_per_step": p["kernels_per_step"], "phase_ms": p["phases"],
           "roofline": _phase_roofline(p["phases"], p["n"], p["cells"], peak, peak_kind, workload=name,
                                       clocks=p["clocks"]),
           "e2e": p["e2e"]}
    if named:
        out["plain_named"] = bench_named(args, sc, torch)
    return out


def run_ours(args, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    peak, peak_kind = measured_peak_gbs()
    peak_kind = "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback"
    extra = {}
    config = workload_config(args.workload, args.seed + (0 if args.workload in BATCHED_WORKLOADS else rank))
    if args.workload in BATCHED_WORKLOADS:
        r = bench_batched(args, torch, world)
        t = r.get("tuned")
        extra["path"] = ("batched form (sph_batch_step), one CUDA graph per substep over all scenes; launch shape "
                         "chosen by sph.autotune: block %d, pair block %d, grid cap %d"
                         % (t["block"], t["pair_block"], t["grid_cap"]) if t else
                         "batched form (sph_batch_step), one CUDA graph per substep over all scenes; launch "
                         "shape: block 256, pair block 128, no grid cap")
        if t:
            extra["autotune"] = t
        if r.get("late"):
            extra["late_state"] = r["late"]
        if rank == 0 and not args.quick:
            pl = bench_plain_loop(r["scenes"], max(3, args.steps // 2))
            batched = r["n"] * args.steps / r["total_s"]
            extra["plain_per_scene"] = {
                "value": pl["graph"], "unit": UNIT, "synced_value": pl["synced"],
                "how": "the same 256 scenes through the drop-in path one after another: value = each scene's "
                       "substeps as one sph_update call (graph launches back to back, one wait per scene); "
                       "synced_value = one substep per call, waiting for each (the reference's blocking calls)"}
            extra["batched_vs_plain"] = batched / pl["graph"]
            extra["batched_vs_plain_synced"] = batched / pl["synced"]
            extra["exact_mix"] = exact_mix(args, torch)
            extra["fp64_error"] = fp64_error_sample(r["scenes"], 100)
            extra["fp64_error_configs"] = fp64_error_configs()
            extra["served"] = bench_served(args)
            extra["plain_1m"] = _plain_extra(args, "wcsph-1m", torch, peak, peak_kind, named=True)
            extra["large_scene"] = _plain_extra(args, "large-scene", torch, peak, peak_kind)
            extra["fp64_error_1m"] = fp64_error_1m(args.seed)
    else:
        scene, _ = workload(args.workload, args.seed + rank)
        r = bench_plain(args, scene, torch, world)
        extra["path"] = "plain single scene, one CUDA-graph substep per step (sph_update)"
        if rank == 0 and scene.material in NAMED_RECIPES:
            extra["plain_named"] = bench_named(args, scene, torch)
    extra["cells"] = r["cells"]
    extra["parallelism"] = "replicas (no collective)" if world > 1 else "single GPU"
    if "pairs" in r and r["phases"]:
        ph = r["phases"]
        step_s = r["total_s"] / args.steps
        c, nb = r["pairs"]["candidates"], r["pairs"]["neighbours"]
        dens = ph.get("density")
        forces = ph.get("forces_fluids+step")
        extra["compute"] = {
            "candidates_per_step": c, "neighbours_per_step": nb,
            "pair_evals_per_s": (c + nb) / step_s,
            "density_candidate_evals_per_s": c / (dens * 1e-3) if dens else None,
            "force_pair_evals_per_s": nb / (forces * 1e-3) if forces else None,
            "how": "density tests every stencil candidate (27 cells); the fused force pass evaluates only the "
                   "neighbours within h from the density pass's masks"}
    value, total_s = aggregate_replicas(r["n"], args.steps, r["total_s"], world, device="cuda")
    if rank != 0:
        return None
    n = r["n"]
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
        "data": "synthetic (seeded lattice scenes, seed %d)" % args.seed,
        "config": config,
        "clocks": r["clocks"],
        "e2e": r["e2e"],
        "gpu_launches": r["kernels_per_step"] * args.steps,
        "roofline": _phase_roofline(r["phases"], n, r["cells"], peak, peak_kind, r.get("counts"),
                                    workload=args.workload, clocks=r["clocks"]),
    }
    line.update(extra)
    return line


def run_reference(args, rank, world):
    """The reference's own kernels (kernels/*.cl compiled for the host CPU
    into oracle/_ref, run by OpenMP over all host cores) in stores its own
    builder made, on the same workload: `warmup` untimed substeps, then
    `steps` timed ones, of every scene.  Neither the sph package nor the
    CUDA library is loaded."""
    if rank != 0:
        return None
    scs = cpu_workload(args.workload, args.seed, standalone=True)
    nthreads = os.cpu_count() or 1
    work = 0
    el = 0.0
    kinds = set()
    for x in scs:
        w, e, kind = cpu_sample(x, x.material, args.steps, nthreads, reference=True, warmup=args.warmup)
        work += w
        el += e
        kinds.add(kind)
    value = work / el
    kind = "reference" if kinds == {"reference"} else "port"
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
        "data": "synthetic (seeded lattice scenes, seed %d)" % args.seed,
        "config": workload_config(args.workload, args.seed, standalone=True),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": kind,
                         "sample": "%d full substeps of every scene of the workload (the reference's kernels in "
                                   "stores its own builder made)" % args.steps},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100,
                    help="timed substeps (100 by default: the clock sampler, every 50 ms, sees several "
                         "samples)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="batched-256",
                    choices=["batched-256", "large-scene", "wcsph-1m", "dam-8k", "beam-4k"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-steps", type=int, default=3, help="substeps in the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="skip the late-state, plain loop, exact mix, served, FP64, 1M and large-scene extras")
    ap.add_argument("--served-seconds", type=float, default=60.0, help="arrival window of the served stream")
    ap.add_argument("--served-chunk", type=int, default=25, help="substeps per serving chunk")
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
            nthreads = os.cpu_count() or 1
            scs = cpu_workload(args.workload, args.seed)
            work, el = 0, 0.0
            for s in scs:
                w, e, kind = cpu_sample(s, s.material, args.cpu_steps, nthreads, reference=False)
                work += w
                el += e
            line["cpu_baseline"] = {"value": work / el, "unit": UNIT, "cores": nthreads, "kind": "port",
                                    "sample": "%d substeps of every scene of the workload on the C oracle "
                                              "(%.1f s)" % (args.cpu_steps, el)}
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
