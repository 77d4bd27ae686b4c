"""GPU parity: corotational and St. Venant-Kirchhoff solids, symmetry
planes, plane constraints and kinematic bodies.

Kernels are compared one at a time on identical inputs (the oracle's
fields are uploaded first), then whole trajectories.  Tolerances, relative
to the largest magnitude of the compared field (measured errors on a
GB300 are 2-5x below them):
  - rotation R (GPU: Newton's polar iteration in FP32 finished by one
    FP64 step; oracle: the reference's FP32 Jacobi getR), deformation,
    stress, forces: 2e-5 (R against an exact FP64 polar factor is pinned
    separately, at 2e-7);
  - strain (a small difference of nearly equal neighbour sums): 5e-5;
  - positions after N substeps: relative L2 error 1e-5.
Neighbour counts stay bit-exact.
"""
import numpy as np
import pytest

from helpers import max_rel, oracle_of, rel_err
from sph import scenes

pytestmark = pytest.mark.gpu

MATERIAL = {
    "corot": ("compute_rotations_and_strains", "compute_stresses_corot", "compute_forces_solids_corot"),
    "svk": ("compute_deformations", "compute_stresses_svk", "compute_forces_solids_svk"),
}


def _solid(material, planes, seed=3, jitter=2e-4):
    sc = scenes.solid_lattice(7, 6, 9, spacing=0.01, h=0.02, material=material, youngs_modulus=2e4,
                              poisson=0.3, jitter=jitter, clamp_layers=1, seed=seed, gravity=(0.0, -9.8, 0.0))
    if planes:
        sc.entries = [("symmetry_planes", "3, 2, 3", "float", None) if e[0] == "symmetry_planes" else e
                      for e in sc.entries]
    ps = sc.system()
    if planes:
        sp = np.zeros((3, 2, 3), np.float32)
        for k in range(3):
            sp[k, 1, k] = 1.0
        ps.set_fields(symmetry_planes=sp)
    rng = np.random.default_rng(seed)
    ps.set_fields(velocity=rng.normal(0, 0.01, (sc.n, 3)).astype(np.float32))
    return sc, ps


def _setup_both(ps, orc):
    ps.call_for_all_particles("init_original_position")
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_original_density")
    orc.setup_solid()


FIELDS = ["position", "velocity", "originalpos", "density", "density0", "rotation", "stress", "strain",
          "deformation"]


def _upload(ps, orc):
    vals = {}
    for k in FIELDS:
        try:
            ps.get_fields(k)
        except Exception:
            continue
        vals[k] = orc.a[k]
    ps.set_fields(**vals)


@pytest.mark.parametrize("material", ["corot", "svk"])
@pytest.mark.parametrize("planes", [False, True])
def test_solid_kernels(material, planes):
    sc, ps = _solid(material, planes)
    orc = oracle_of(ps)
    n = sc.n
    _setup_both(ps, orc)
    ps.sync_device_to_host()
    assert max_rel(ps.get_fields("density0")[0][:n], orc.a["density0"][:n]) <= 1e-5
    # deform the lattice, then compare each kernel on the oracle's inputs
    rng = np.random.default_rng(1)
    orc.a["position"][:n] += rng.normal(0, 5e-4, (n, 3)).astype(np.float32)
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    _upload(ps, orc)
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_density")
    ps.sync_device_to_host()
    assert np.array_equal(ps.get_fields("num_neighbours")[0][:n], orc.a["num_neighbours"][:n])
    k1, k2, k3 = MATERIAL[material]
    ps.call_for_all_particles(k1.replace("_corot", "").replace("_svk", ""))
    orc.call(k1)
    ps.sync_device_to_host()
    if material == "corot":
        soft = ps.get_fields("body_number")[0][:n] == 0
        assert max_rel(ps.get_fields("rotation")[0][:n][soft], orc.a["rotation"][:n][soft]) <= 2e-5
        assert max_rel(ps.get_fields("strain")[0][:n][soft], orc.a["strain"][:n][soft]) <= 5e-5
    else:
        assert max_rel(ps.get_fields("deformation")[0][:n], orc.a["deformation"][:n]) <= 2e-5
    _upload(ps, orc)
    ps.call_for_all_particles("compute_stresses")
    orc.call(k2)
    ps.sync_device_to_host()
    assert max_rel(ps.get_fields("stress")[0][:n], orc.a["stress"][:n]) <= 2e-5
    _upload(ps, orc)
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_forces_solids")
    orc.call(k3)
    ps.sync_device_to_host()
    for f in ["force", "force_elastic", "force_viscous", "cutoff_force"]:
        assert max_rel(ps.get_fields(f)[0][:n], orc.a[f][:n]) <= 2e-5, f
    ps.close()


@pytest.mark.parametrize("planes", [False, True])
@pytest.mark.parametrize("material", ["corot", "svk"])
def test_solid_trajectory(material, planes):
    """The named recipe and the fused substep (first pass with the density
    and the stresses, forces with the step; separate stress and step passes
    for scenes with planes) agree bit for bit, and with the oracle."""
    sc, ps = _solid(material, planes, jitter=1e-4)
    _, ps2 = _solid(material, planes, jitter=1e-4)
    orc = oracle_of(ps)
    _setup_both(ps, orc)
    ps2.call_for_all_particles("init_original_position")
    ps2.compute_particle_bins()
    ps2.call_for_all_particles("compute_original_density")
    steps = 30
    recipe = ["compute_density", "compute_rotations_and_strains" if material == "corot" else "compute_deformations",
              "compute_stresses", "compute_forces_solids", "step_forward"]
    for _ in range(steps):
        ps.compute_particle_bins()
        for k in recipe:
            ps.call_for_all_particles(k)
    ps2.update_fused(steps)
    orc.run(material, steps)
    ps.sync_device_to_host()
    ps2.sync_device_to_host()
    n = sc.n
    pa = ps.get_fields("position")[0][:n]
    assert np.array_equal(pa, ps2.get_fields("position")[0][:n])
    assert rel_err(pa, orc.a["position"][:n]) <= 1e-5
    ps.close()
    ps2.close()


@pytest.mark.parametrize("planes", [False, True])
@pytest.mark.parametrize("material", ["corot", "svk"])
def test_named_solid_forces_walk_masks_only_in_the_recipe_chain(material, planes):
    """compute_forces_solids called right after compute_stresses, itself
    right after the first solid pass (the reference drivers' order), walks
    the first pass's masks over the sorted copies; with any call in between
    it scans the fields.  Both give the same bits."""
    sc, a = _solid(material, planes, seed=9, jitter=1e-4)
    _, b = _solid(material, planes, seed=9, jitter=1e-4)
    first = MATERIAL[material][0]
    for ps in (a, b):
        ps.call_for_all_particles("init_original_position")
        ps.compute_particle_bins()
        ps.call_for_all_particles("compute_original_density")
        ps.update_fused(3)  # a deformed state
        ps.compute_particle_bins()
        ps.call_for_all_particles("compute_density")
        ps.call_for_all_particles(first)
        ps.call_for_all_particles("compute_stresses")
    a.call_for_all_particles("compute_forces_solids")  # the masked walk
    assert b.status() == 0  # a call in between: the scan
    b.call_for_all_particles("compute_forces_solids")
    a.sync_device_to_host()
    b.sync_device_to_host()
    n = sc.n
    for f in ("force", "force_elastic", "force_viscous", "cutoff_force", "stress"):
        assert np.array_equal(a.get_fields(f)[0][:n], b.get_fields(f)[0][:n]), f
    a.close()
    b.close()


def test_plane_constraints():
    sc = scenes.solid_lattice(6, 6, 6, material="corot", jitter=1e-3, seed=2)
    sc.entries = [("plane_constraints", "3, 2, 4", "float", None) if e[0] == "plane_constraints" else e
                  for e in sc.entries]
    ps = sc.system()
    pc = np.zeros((4, 2, 3), np.float32)
    pc[0, 0, 0], pc[0, 1, 0] = 0.01, 1.0
    pc[1, 1] = np.array([0.6, 0.8, 0.0])
    pc[3, 0, 2], pc[3, 1, 2] = 0.03, 1.0
    rng = np.random.default_rng(0)
    mask = rng.integers(0, 16, sc.n).astype(np.uint32)
    ps.set_fields(plane_constraints=pc, plane_constraints_particles=mask,
                  velocity=rng.normal(0, 0.1, (sc.n, 3)).astype(np.float32))
    orc = oracle_of(ps)
    ps.call_for_all_particles("apply_plane_constraints")
    orc.call("apply_plane_constraints")
    ps.sync_device_to_host()
    assert max_rel(ps.get_fields("position")[0], orc.a["position"]) <= 1e-6
    assert max_rel(ps.get_fields("velocity")[0], orc.a["velocity"]) <= 1e-6
    ps.close()


def test_kinematic_bodies():
    sc = scenes.solid_lattice(6, 6, 8, material="corot", jitter=1e-3, seed=5, clamp_layers=2)
    ps = sc.system()
    ps.set_fields(body_position=np.array([[0.01, 0.02, 0.03]], np.float32),
                  body_euler_rotation=np.array([[0.1, 0.2, 0.3]], np.float32))
    orc = oracle_of(ps)
    ps.set_body_position(0, np.array([0.02, 0.0, 0.05]))
    orc.set_body_position(0, np.array([0.02, 0.0, 0.05]))
    ps.set_body_rotation(0, np.array([0.3, -0.2, 0.1]))
    orc.set_body_rotation(0, np.array([0.3, -0.2, 0.1]))
    ps.sync_device_to_host()
    for f in ["position", "velocity", "rotation", "body_position", "body_euler_rotation"]:
        assert max_rel(ps.get_fields(f)[0], orc.a[f].reshape(ps.get_fields(f)[0].shape)) <= 1e-5, f
    ps.close()
