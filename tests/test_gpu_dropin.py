"""GPU: the drop-in's scene builders, the corotational polar factor against
an exact FP64 one, and the store shape that uploads may not change.

- populate_position_cuboid / rotate_particles (common.cl:533-604) against
  the reference's own kernels (tests/golden/kernels_scene_builders.npz):
  positions and n bit for bit after populate_position_cuboid (every
  operation rounded as in the source), positions within 1e-6 of their
  magnitude after each rotate_particles (cosf/sinf may differ from the host
  libm's in the last bit; the products are rounded as in the source); the
  same against the oracle on seeded random cuboids and angles.
- compute_rotations_and_strains: R of every soft particle within 1e-7 of
  the exact polar factor U V^T of the particle's own Apq (apq_temp, from
  an FP64 SVD), on a rotated and stretched lattice; body particles keep
  the pose set_body_rotation gives them, within 5e-7 of the FP64 oracle's.
- gridres and pnum size the device tables: an upload that changes them is
  rejected, and the store keeps working.
"""
import os

import numpy as np
import pytest

from helpers import max_rel, oracle_of
from sph import bindings as bnd
from sph import scenes
from sph.systems import ParticleSystem

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_scene_builders_match_reference():
    g = dict(np.load(os.path.join(GOLD, "kernels_scene_builders.npz")))
    spec = str(g["spec"])
    for c, row in enumerate(g["cuboids"]):
        ps = ParticleSystem(spec=spec, kernel_files=scenes.FLUID_KERNELS)
        ps.set_fields(n=0)
        c1, c2, size = row[0:3], row[3:6], row[6:9].astype(int)
        bnd.populate_position_cuboid_device_opencl(ps.psdata_opencl, *[float(x) for x in c1],
                                                   *[float(x) for x in c2], *[int(x) for x in size])
        ps.sync_device_to_host()
        pre = "f32/cuboid%d/" % c
        assert int(ps.get_fields("n")[0][0]) == int(g[pre + "n"][0])
        assert np.array_equal(ps.get_fields("position")[0], g[pre + "position"]), "cuboid %d" % c
        for a, ang in enumerate(g["angles"]):
            bnd.rotate_particles_device_opencl(ps.psdata_opencl, *[float(x) for x in ang])
            ps.sync_device_to_host()
            got = ps.get_fields("position")[0]
            assert max_rel(got, g[pre + "rotate%d/position" % a]) <= 1e-6, (c, a)
            # and the reference's FP64 run of the same calls
            assert max_rel(got, g["f64/cuboid%d/rotate%d/position" % (c, a)]) <= 1e-6, (c, a)
        ps.close()


def test_scene_builders_random_against_oracle():
    """Seeded random cuboids (8 to 216 points against pnum 120, corners in
    any order) and angles: the GPU's populate_position_cuboid equals the
    oracle's bit for bit (positions and n), and each rotate_particles stays
    within 1e-6 of it."""
    sc = scenes.wcsph_block(6, 5, 4, jitter=0.0, seed=0, walls=False)
    rng = np.random.default_rng(61)
    for case in range(10):
        ps = ParticleSystem(spec=sc.spec, kernel_files=scenes.FLUID_KERNELS)
        ps.set_fields(n=0)
        orc = oracle_of(ps, "f32", guards=0)
        c1, c2 = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
        size = [int(x) for x in rng.integers(2, 7, 3)]
        c1f, c2f = c1.astype(np.float32), c2.astype(np.float32)
        bnd.populate_position_cuboid_device_opencl(ps.psdata_opencl, *[float(x) for x in c1f],
                                                   *[float(x) for x in c2f], *size)
        orc.populate_position_cuboid(c1f, c2f, size)
        ps.sync_device_to_host()
        assert int(ps.get_fields("n")[0][0]) == orc.n, case
        assert np.array_equal(ps.get_fields("position")[0], orc.a["position"]), case
        for _ in range(2):
            ang = rng.uniform(-4, 4, 3).astype(np.float32)
            bnd.rotate_particles_device_opencl(ps.psdata_opencl, *[float(x) for x in ang])
            orc.rotate_particles(*ang)
            ps.sync_device_to_host()
            assert max_rel(ps.get_fields("position")[0], orc.a["position"]) <= 1e-6, case
        ps.close()


def _rotation(axis, angle):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def test_polar_factor_against_fp64():
    sc = scenes.solid_lattice(8, 7, 10, spacing=0.01, h=0.02, material="corot", youngs_modulus=2e4, jitter=2e-4,
                              clamp_layers=1, seed=5, gravity=(0.0, 0.0, 0.0))
    ps = sc.system()
    n = sc.n
    ps.call_for_all_particles("init_original_position")
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_original_density")
    ps.sync_device_to_host()
    # a large rotation times a stretch, plus per-particle noise
    x0 = np.asarray(ps.get_fields("originalpos")[0][:n], np.float64)
    F = _rotation((0.3, -0.5, 0.8), 0.9) @ (np.eye(3) + np.array([[0.04, 0.01, 0.0], [0.01, -0.03, 0.02],
                                                                   [0.0, 0.02, 0.05]]))
    c = x0.mean(axis=0)
    x = (x0 - c) @ F.T + c + np.random.default_rng(7).normal(0, 3e-4, x0.shape)
    ps.set_fields(position=x.astype(np.float32))
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_density")
    ps.call_for_all_particles("compute_rotations_and_strains")
    ps.sync_device_to_host()
    soft = ps.get_fields("body_number")[0][:n] == 0
    apq = np.asarray(ps.get_fields("apq_temp")[0][:n][soft], np.float64)
    R = np.asarray(ps.get_fields("rotation")[0][:n][soft], np.float64)
    U, _, Vt = np.linalg.svd(apq)
    exact = U @ Vt
    err = float(np.max(np.abs(R - exact)))
    print("soft particles: %d, max |R - polar(Apq)| = %.2e" % (int(soft.sum()), err))
    assert err <= 1e-7, err
    # body particles: the kinematic pose, against the FP64 oracle
    o64 = oracle_of(ps, "f64")
    euler = np.array([[0.4, -0.3, 0.25]], np.float32)
    ps.set_fields(body_euler_rotation=euler)
    o64.a["body_euler_rotation"][:1] = euler
    ps.set_body_rotation(0, np.array([0.1, 0.2, 0.3], np.float32))
    o64.set_body_rotation(0, np.array([0.1, 0.2, 0.3]))
    ps.sync_device_to_host()
    body = ~soft
    Rb = np.asarray(ps.get_fields("rotation")[0][:n][body], np.float64)
    assert body.any()
    berr = float(np.max(np.abs(Rb - o64.a["rotation"][:n][body])))
    print("body particles: %d, max |R - R_fp64| = %.2e" % (int(body.sum()), berr))
    assert berr <= 5e-7, berr
    ps.close()


def test_upload_may_not_change_store_shape():
    ps = scenes.wcsph_block(6, 5, 4, seed=1).system()
    res = ps.get_fields("gridres")[0]
    res[0] += 1
    with pytest.raises(bnd.SphError, match="gridres"):
        ps.sync_fields_host_to_device("gridres")
    with pytest.raises(bnd.SphError, match="gridres"):
        ps.sync_host_to_device()
    res[0] -= 1
    ps.sync_host_to_device()
    ps.update_fused(2)
    ps.synchronize()
    assert ps.status() == 0
    ps.close()
