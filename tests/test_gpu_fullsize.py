"""GPU parity at the benchmark's full sizes.

The oracle runs single passes at these sizes in about a second (C, all
host cores), so the cell tables and the neighbour counts of the
1,048,576-particle slab are compared with it bit for bit and its densities
within the usual 1e-5.  Whole trajectories at full size are checked through
properties that hold at any size:
  - the WCSPH pair term is antisymmetric, so the internal forces of the
    slab sum to zero (to float rounding of the per-particle sums);
  - each of the 256 scenes of the batched workload advanced inside the full
    batch equals itself advanced alone (bit for bit), and none raises a
    status bit;
  - the rigid ball of the large scene keeps its shape;
  - the interacting large scene (1M fluid, 32^3 SVK cube, rigid ball in one
    store) gives the same bits through the named recipe (scans) and the
    fused substeps (mask walks), and its ball stays rigid.
"""
import os

import numpy as np
import pytest

from helpers import max_rel, oracle_of
from sph import scenes
from sph.batch import Batch

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def slab(**kw):
    """The 1,048,576-particle WCSPH slab of the 1M workload (128 x 64 x 128
    at 0.005 m, h = 0.01 m, in [0, 1]^3)."""
    args = dict(spacing=0.005, h=0.01, box=(0.0, 1.0), jitter=5e-5, seed=0, dt=2e-5, walls=True, stiffness=0.375,
                viscosity=0.025, name="slab-1m")
    args.update(kw)
    return scenes.wcsph_block(128, 64, 128, **args)


def test_1m_cell_tables_and_density_match_oracle():
    sc = slab()
    assert sc.n == 1 << 20
    ps = sc.system()
    ps.update_fused(5)  # a few substeps first, so that particles have left their lattice cells
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_density")
    ps.sync_device_to_host()
    orc = oracle_of(ps, nthreads=THREADS)
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    n = sc.n
    cell, count, off, parts, nn, rho = ps.get_fields("gridcell", "gridcount", "celloffset", "cellparticles",
                                                    "num_neighbours", "density")
    assert np.array_equal(cell[:n], orc.a["gridcell"][:n])
    assert np.array_equal(count.ravel(), orc.a["gridcount"])
    assert np.array_equal(off.ravel(), orc.a["celloffset"])
    assert np.array_equal(parts[:n], orc.a["cellparticles"][:n])
    assert np.array_equal(nn[:n], orc.a["num_neighbours"][:n])
    assert max_rel(rho[:n], orc.a["density"][:n]) <= 1e-5
    ps.close()


def test_1m_internal_forces_sum_to_zero():
    """No gravity and no walls: the forces are the pair terms alone, each
    pair's two terms exact negatives of each other."""
    sc = slab(walls=False, gravity=(0.0, 0.0, 0.0))
    ps = sc.system()
    rng = np.random.default_rng(3)
    ps.set_fields(velocity=rng.normal(0.0, 0.05, size=(sc.n, 3)).astype(np.float32))
    ps.compute_particle_bins()
    for k in ("compute_density", "compute_forces_fluids"):
        ps.call_for_all_particles(k)
    ps.sync_device_to_host()
    f = ps.get_fields("force")[0][: sc.n].astype(np.float64)
    scale = np.abs(f).sum(axis=0)
    assert np.all(scale > 0)
    assert np.all(np.abs(f.sum(axis=0)) <= 1e-6 * scale)
    assert ps.status() == 0
    ps.close()


def test_batched_256_each_scene_equals_alone():
    scs = scenes.batch_mix(256, seed=0)
    b = Batch()
    ids = [b.add(s) for s in scs]
    steps = 3
    b.step(steps)
    assert all(b.status(i) == 0 for i in ids)
    # the largest and the smallest scene of each material
    picks = {}
    for s, i in sorted(zip(scs, ids), key=lambda t: t[0].n):
        picks.setdefault((s.material, "small"), (s, i))
        picks[(s.material, "large")] = (s, i)
    for (mat, _), (s, i) in picks.items():
        alone = s.system()
        if mat != "fluid":
            alone.call_for_all_particles("init_original_position")
            alone.compute_particle_bins()
            alone.call_for_all_particles("compute_original_density")
        alone.update_fused(steps)
        alone.sync_device_to_host()
        v = b.read(i)
        assert np.array_equal(v["position"][: s.n], alone.get_fields("position")[0][: s.n]), s.name
        assert np.array_equal(v["velocity"][: s.n], alone.get_fields("velocity")[0][: s.n]), s.name
        alone.close()
    b.close()


def test_large_scene_ball_stays_rigid():
    fluid = scenes.large_scene(seed=0)[0]
    ps = fluid.system()
    ps.update_fused(20)
    ps.sync_device_to_host()
    body = np.asarray(fluid.init["body_number"]) == 1
    x0 = np.asarray(fluid.init["position"], dtype=np.float64)[body]
    x1 = ps.get_fields("position")[0][: fluid.n][body].astype(np.float64)
    sub = np.random.default_rng(0).choice(len(x0), size=min(600, len(x0)), replace=False)

    def dists(x):
        d = x[sub][:, None, :] - x[sub][None, :, :]
        return np.sqrt((d * d).sum(-1))
    assert np.max(np.abs(dists(x1) - dists(x0))) <= 2e-6  # float positions, FP64 body state
    assert np.max(np.abs(x1 - x0)) > 1e-7  # it moved
    assert ps.status() == 0
    ps.close()


def test_large_interacting_scene_named_equals_fused():
    sc = scenes.large_fluid_solid_scene(seed=0)
    a, b = sc.system(), sc.system()
    for ps in (a, b):
        ps.call_for_all_particles("init_original_position")
        ps.compute_particle_bins()
        ps.call_for_all_particles("compute_original_density")
    steps = 5
    a.update_fused(steps)
    for _ in range(steps):
        b.compute_particle_bins()
        for k in ("compute_density", "compute_deformations", "compute_stresses", "compute_forces_solids",
                  "compute_forces_fluids", "step_forward"):
            b.call_for_all_particles(k)
    a.sync_device_to_host()
    b.sync_device_to_host()
    n = sc.n
    for f in ("position", "velocity", "force", "deformation", "density"):
        assert np.array_equal(a.get_fields(f)[0][:n], b.get_fields(f)[0][:n]), f
    body = np.asarray(sc.init["body_number"])[:n] == 1
    x0 = np.asarray(sc.init["position"], dtype=np.float64)[:n][body]
    x1 = a.get_fields("position")[0][:n][body].astype(np.float64)
    sub = np.random.default_rng(1).choice(len(x0), size=min(600, len(x0)), replace=False)
    d0 = np.sqrt((((x0[sub][:, None] - x0[sub][None]) ** 2).sum(-1)))
    d1 = np.sqrt((((x1[sub][:, None] - x1[sub][None]) ** 2).sum(-1)))
    assert np.max(np.abs(d1 - d0)) <= 2e-6
    assert a.status() == 0 and b.status() == 0
    a.close()
    b.close()
