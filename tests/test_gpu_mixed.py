"""Fluid and elastic solid in one interacting scene (the mixed-scene
extension): a WCSPH block, a St. Venant-Kirchhoff cube and a rigid ball.

The reference runs one program per store, so it has no counterpart; the
oracle restates the extension's rules (oracle/sph_oracle_impl.h, `phase`):
solid particles take the SVK law over their solid neighbours, every pair
with a fluid particle takes the fluid pair term of fluids.cl with both
pressures clamped at 0 when one of the two is solid.

- GPU (fused CUDA-graph substeps) against the oracle: positions within
  1e-5 relative L2 after 40 substeps, the cube hitting the fluid.
- The named kernels (the recipe a driver issues by name) equal the fused
  substeps bit for bit.
- With gravity and walls off and no solid viscosity (every remaining pair
  term is antisymmetric), the total momentum of fluid, cube and ball stays
  within 1e-5 of the sum of |momentum| over 200 substeps, on the GPU and in
  the FP64 oracle, while the cube and the ball exchange more than half
  their initial momentum with the fluid.
"""
import os

import numpy as np
import pytest

from helpers import oracle_of, rel_err
from sph import scenes

THREADS = os.cpu_count() or 4


def impact_scene(**kw):
    args = dict(fluid=(12, 8, 12), cube=(5, 5, 5), cube_origin=(0.035, 0.09, 0.035), cube_velocity=(0.0, -0.1, 0.0),
                ball=(0.025, (0.15, 0.04, 0.06), (-0.2, 0.0, 0.0)), seed=4)
    args.update(kw)
    return scenes.fluid_solid_scene(**args)


def free_scene():
    # no gravity, no walls, no solid viscosity: every pair term antisymmetric
    return impact_scene(gravity=(0.0, 0.0, 0.0), walls=False, solid_viscosity=0.0,
                        gridbounds=(-0.2, 0.6, -0.2, 0.6, -0.2, 0.6))


def setup(ps):
    ps.call_for_all_particles("init_original_position")
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_original_density")


def named_substep(ps):
    ps.compute_particle_bins()
    for k in ("compute_density", "compute_deformations", "compute_stresses", "compute_forces_solids",
              "compute_forces_fluids", "step_forward"):
        ps.call_for_all_particles(k)


def momentum(vel, mass, n):
    v = np.asarray(vel[:n], np.float64)
    return mass * v.sum(axis=0), mass * np.abs(v).sum()


def test_mixed_scene_momentum_oracle_fp64():
    sc = free_scene()
    from helpers import host_store
    _, v = host_store(sc)
    o = oracle_of(v, "f64", nthreads=THREADS)
    o.setup_solid()
    m, n = float(v["mass"][0]), sc.n
    cube = np.asarray(v["phase"][:n]) == 1
    P0, S0 = momentum(o.a["velocity"], m, n)
    pc0 = m * o.a["velocity"][:n][cube].sum(axis=0)
    o.run("mixed", 200)
    P, _ = momentum(o.a["velocity"], m, n)
    pc = m * o.a["velocity"][:n][cube].sum(axis=0)
    assert np.all(np.isfinite(o.a["position"][:n]))
    assert np.max(np.abs(P - P0)) <= 1e-9 * S0
    assert abs(pc[1] - pc0[1]) > 0.5 * abs(pc0[1])  # momentum went between the cube and the fluid


@pytest.mark.gpu
def test_mixed_scene_matches_oracle():
    sc = impact_scene()
    ps = sc.system()
    orc = oracle_of(ps, "f32", nthreads=THREADS)
    setup(ps)
    orc.setup_solid()
    ps.update_fused(40)
    orc.run("mixed", 40)
    ps.sync_device_to_host()
    n = sc.n
    err = rel_err(ps.get_fields("position")[0][:n], orc.a["position"][:n])
    print("mixed scene, 40 substeps: relative L2 position error %.2e against the oracle" % err)
    assert err <= 1e-5, err
    assert ps.status() == 0
    ps.close()


@pytest.mark.gpu
def test_mixed_named_kernels_equal_fused():
    sc = impact_scene(seed=5)
    a, b = sc.system(), sc.system()
    setup(a)
    setup(b)
    a.update_fused(15)
    for _ in range(15):
        named_substep(b)
    a.sync_device_to_host()
    b.sync_device_to_host()
    n = sc.n
    for f in ("position", "velocity", "force", "stress", "density"):
        assert np.array_equal(a.get_fields(f)[0][:n], b.get_fields(f)[0][:n]), f
    a.close()
    b.close()


@pytest.mark.gpu
def test_mixed_scene_conserves_momentum():
    sc = free_scene()
    ps = sc.system()
    setup(ps)
    n = sc.n
    m = float(ps.get_fields("mass")[0][0])
    cube = np.asarray(ps.get_fields("phase")[0][:n]) == 1
    ball = np.asarray(ps.get_fields("body_number")[0][:n]) == 1
    ps.sync_device_to_host()
    vel = ps.get_fields("velocity")[0]
    P0, S0 = momentum(vel, m, n)
    pc0 = m * np.asarray(vel[:n][cube], np.float64).sum(axis=0)
    pb0 = m * np.asarray(vel[:n][ball], np.float64).sum(axis=0)
    ps.update_fused(200)
    ps.sync_device_to_host()
    P, _ = momentum(vel, m, n)
    pc = m * np.asarray(vel[:n][cube], np.float64).sum(axis=0)
    pb = m * np.asarray(vel[:n][ball], np.float64).sum(axis=0)
    print("momentum drift %.2e of sum |p|; cube p_y %.4f -> %.4f, ball p_x %.4f -> %.4f"
          % (np.max(np.abs(P - P0)) / S0, pc0[1], pc[1], pb0[0], pb[0]))
    assert np.max(np.abs(P - P0)) <= 1e-5 * S0
    assert abs(pc[1] - pc0[1]) > 0.5 * abs(pc0[1]) and abs(pb[0] - pb0[0]) > 0.5 * abs(pb0[0])
    assert ps.status() == 0
    ps.close()
