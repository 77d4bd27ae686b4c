"""The CPU oracle (oracle/sph_oracle.c) against the reference's own kernels.

Golden files (tests/golden/kernels_*.npz) hold each kernel's inputs and
outputs from the reference's kernels/*.cl compiled for the CPU
(tests/golden/make_golden.py).  The restatement must reproduce them:
integer fields exactly, float fields to 1e-6 of their magnitude (the two
are bit-identical on the machine that made the files; the margin covers a
different libm).  Also: physical sanity properties of the oracle, and a
live comparison with oracle/_ref where it is built."""
import os

import numpy as np
import pytest

from helpers import host_store, max_rel
from oracle.oracle import OracleScene
from sph import bindings as bnd
from sph import free_data_cpu, init_data_cpu, scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["fluid", "corot", "corot_planes", "svk", "svk_planes"]
KERNEL = {
    ("fluid", "compute_forces_fluids"): "compute_forces_fluids",
    ("corot", "compute_rotations_and_strains"): "compute_rotations_and_strains",
    ("corot", "compute_stresses"): "compute_stresses_corot",
    ("corot", "compute_forces_solids"): "compute_forces_solids_corot",
    ("svk", "compute_deformations"): "compute_deformations",
    ("svk", "compute_stresses"): "compute_stresses_svk",
    ("svk", "compute_forces_solids"): "compute_forces_solids_svk",
}
RECIPES = {"fluid": ["compute_density", "compute_forces_fluids"],
           "corot": ["compute_density", "compute_rotations_and_strains", "compute_stresses", "compute_forces_solids"],
           "svk": ["compute_density", "compute_deformations", "compute_stresses", "compute_forces_solids"]}


def load(case):
    return dict(np.load(os.path.join(GOLD, "kernels_%s.npz" % case)))


def fields_of(g, prec, stage, spec):
    ps = init_data_cpu(spec)
    v = bnd.store_views(ps)
    pre = "%s/%s/" % (prec, stage)
    out = {}
    for k, arr in v.items():
        out[k] = np.array(arr)
    for key, val in g.items():
        if key.startswith(pre):
            out[key[len(pre):]] = val
    free_data_cpu(ps)
    return out


def check(got, want, name):
    if want.dtype.kind in "ui":
        assert np.array_equal(got.reshape(want.shape), want), name
    else:
        assert max_rel(got.reshape(want.shape), want) <= 1e-6, name


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_reproduces_reference_kernels(case, prec):
    g = load(case)
    mat = str(g["material"])
    spec = str(g["spec"])
    if prec == "f64":
        spec = spec.replace("| float", "| double")
    solid = mat != "fluid"
    orc = OracleScene(fields_of(g, prec, "init", spec), prec, guards=0)
    n = orc.n
    if solid:
        orc.setup_solid()
        for k in ("originalpos", "density0"):
            check(orc.a[k][:n], g["%s/setup/%s" % (prec, k)][:n], "setup " + k)
        orc.a["position"][:] = g["%s/deformed/position" % prec]
    orc.call("compute_particle_bins")
    for k in ("gridcell", "cellparticles"):
        check(orc.a[k][:n], g["%s/s1/compute_particle_bins/%s" % (prec, k)][:n], "bins " + k)
    for k in ("gridcount", "celloffset"):
        check(orc.a[k], g["%s/s1/compute_particle_bins/%s" % (prec, k)].ravel(), "bins " + k)
    for kern in RECIPES[mat] + ["step_forward"]:
        orc.call(KERNEL.get((mat, kern), kern))
        pre = "%s/s1/%s/" % (prec, kern)
        for key in g:
            if key.startswith(pre):
                f = key[len(pre):]
                check(orc.a[f][:n], g[key][:n], kern + " " + f)
    for _ in range(int(g["steps"]) - 1):
        orc.substep(mat)
    for f in ("position", "velocity", "density", "num_neighbours"):
        check(orc.a[f][:n], g["%s/final/%s" % (prec, f)][:n], "final " + f)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_bodies_and_constraints(prec):
    g = load("corot")
    spec = str(g["spec"])
    if prec == "f64":
        spec = spec.replace("| float", "| double")
    orc = OracleScene(fields_of(g, prec, "body_init", spec), prec, guards=0)
    orc.set_body_position(0, [0.02, 0.0, 0.05])
    for f in ("position", "velocity", "body_position"):
        check(orc.a[f], g["%s/set_body_position/%s" % (prec, f)].reshape(orc.a[f].shape), "set_body_position " + f)
    orc.set_body_rotation(0, [0.3, -0.2, 0.1])
    for f in ("position", "rotation", "body_euler_rotation"):
        check(orc.a[f], g["%s/set_body_rotation/%s" % (prec, f)].reshape(orc.a[f].shape), "set_body_rotation " + f)
    orc2 = OracleScene(fields_of(g, prec, "constraints_init", spec), prec)
    orc2.call("apply_plane_constraints")
    for f in ("position", "velocity"):
        check(orc2.a[f], g["%s/apply_plane_constraints/%s" % (prec, f)], "constraints " + f)


def test_single_particle_density_is_self_weight():
    sc = scenes.wcsph_block(1, 1, 1, jitter=0.0, walls=False)
    ps, v = host_store(sc)
    orc = OracleScene(v, "f64")
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    h = float(v["smoothingradius"][0])
    pi = float(np.float32(3.1415926535))
    assert orc.a["density"][0] == pytest.approx(float(v["mass"][0]) * 315 / (64 * pi * h ** 3), rel=1e-12)
    assert orc.a["num_neighbours"][0] == 1
    free_data_cpu(ps)


def test_pair_forces_are_equal_and_opposite():
    """Interior WCSPH forces are antisymmetric pair terms: their sum
    vanishes (no cube band inside [-1.8, 1.8]^3)."""
    sc = scenes.wcsph_block(6, 6, 6, jitter=1e-3, seed=5, walls=False)
    ps, v = host_store(sc, velocity=np.random.default_rng(0).normal(0, 0.1, (sc.n, 3)))
    orc = OracleScene(v, "f64")
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    orc.call("compute_forces_fluids")
    f = orc.a["force"][: sc.n]
    assert np.abs(f.sum(axis=0)).max() <= 1e-10 * np.abs(f).max() * sc.n
    free_data_cpu(ps)


def test_empty_scene():
    sc = scenes.wcsph_block(4, 4, 4, walls=False)
    ps, v = host_store(sc, n=0)
    orc = OracleScene(v, "f32")
    orc.run("fluid", 2)
    assert orc.a["gridcount"].sum() == 0 and np.all(orc.a["celloffset"] == 0)
    free_data_cpu(ps)


def test_jacobi_guard_defines_the_diagonal_case():
    """An already-diagonal matrix with equal entries: the reference's
    Givens angle is atan(0/0) = NaN; the guard gives the identity."""
    from oracle.oracle import lib
    import ctypes
    apq = np.diag([2.0, 2.0, 2.0]).astype(np.float32)
    r = np.zeros(9, np.float32)
    P = ctypes.POINTER(ctypes.c_float)
    lib().oracle_get_r_f32(apq.ctypes.data_as(P), r.ctypes.data_as(P), 1)
    assert np.allclose(r.reshape(3, 3), np.eye(3), atol=1e-6)
    lib().oracle_get_r_f32(apq.ctypes.data_as(P), r.ctypes.data_as(P), 0)
    assert np.isnan(r).any()


def test_oracle_matches_compiled_reference_live():
    from oracle import ref
    if not ref.available():
        pytest.skip("oracle/_ref not built on this machine")
    sc = scenes.wcsph_block(9, 8, 7, jitter=3e-3, seed=21, walls=False)
    ps, v = host_store(sc)
    orc = OracleScene(v, "f32", guards=0)
    rs = ref.RefStore(sc.spec)
    for k in ("position", "n"):
        rs.view(k)[...] = v[k]
    for _ in range(3):
        orc.substep("fluid")
        rs.call("fluid", "f32", "compute_particle_bins", sc.n)
        for k in ("compute_density", "compute_forces_fluids", "step_forward"):
            rs.call("fluid", "f32", k, sc.n)
    for k in ("position", "velocity", "density", "num_neighbours", "cellparticles"):
        assert np.array_equal(rs.view(k)[: sc.n], orc.a[k][: sc.n].reshape(rs.view(k)[: sc.n].shape)), k
    rs.free()
    free_data_cpu(ps)


def test_zero_distance_guard():
    sc = scenes.wcsph_block(5, 5, 5, jitter=1e-4, seed=2, walls=False)
    pos = sc.init["position"].copy()
    pos[10] = pos[11]
    ps, v = host_store(sc, position=pos)
    for guards, finite in ((3, True), (0, False)):
        orc = OracleScene(v, "f32", guards=guards)
        orc.call("compute_particle_bins")
        orc.call("compute_density")
        orc.call("compute_forces_fluids")
        assert np.isfinite(orc.a["force"][: sc.n]).all() == finite
    free_data_cpu(ps)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_reproduces_reference_scene_builders(prec):
    """populate_position_cuboid and rotate_particles (common.cl:533-604)
    against the reference's own kernels: positions and n bit for bit."""
    g = dict(np.load(os.path.join(GOLD, "kernels_scene_builders.npz")))
    spec = str(g["spec"])
    if prec == "f64":
        spec = spec.replace("| float", "| double")
    for c, row in enumerate(g["cuboids"]):
        ps = init_data_cpu(spec)
        v = bnd.store_views(ps)
        orc = OracleScene({k: np.array(a) for k, a in v.items()}, prec)
        free_data_cpu(ps)
        orc.state.n = 0
        orc.populate_position_cuboid(row[0:3], row[3:6], row[6:9].astype(int))
        pre = "%s/cuboid%d/" % (prec, c)
        assert orc.n == int(g[pre + "n"][0])
        assert np.array_equal(orc.a["position"], g[pre + "position"])
        for a, ang in enumerate(g["angles"]):
            orc.rotate_particles(*ang)
            assert np.array_equal(orc.a["position"], g[pre + "rotate%d/position" % a]), (c, a)


SOLID_OUT = {"corot": ["rotation", "strain", "stress", "apq_temp"], "svk": ["deformation", "stress"]}


@pytest.mark.parametrize("mat", ["corot", "svk"])
@pytest.mark.parametrize("with_planes", [False, True])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_matches_compiled_reference_live_solids(mat, with_planes, prec):
    """Seeded solid lattices of random shape, stiffness and jitter, deformed
    after their set-up, three substeps in the oracle (guards off) and in
    the reference's compiled kernels: in FP32 every field equal bit for
    bit; in FP64 the integer fields equal and the others as the golden
    files are checked (the reference's double build keeps its float
    literals, e.g. PI = 3.1415926535f, common.cl:15, in the kernel
    normalisations, so density0 differs by 3e-8 relative)."""
    from oracle import ref
    if not ref.available():
        pytest.skip("oracle/_ref not built on this machine")
    rng = np.random.default_rng({"corot": 11, "svk": 12}[mat] + 2 * with_planes + (prec == "f64"))
    for case in range(2):
        dims = [int(x) for x in rng.integers(3, 7, 3)]
        sc = scenes.solid_lattice(*dims, material=mat, youngs_modulus=float(rng.uniform(1e4, 1e5)),
                                  poisson=float(rng.uniform(0.2, 0.45)), jitter=float(rng.uniform(0, 1e-3)),
                                  clamp_layers=int(rng.integers(1, 3)), seed=int(rng.integers(1000)))
        if with_planes:
            sc.entries = [("symmetry_planes", "3, 2, 2", "float", None) if e[0] == "symmetry_planes" else e
                          for e in sc.entries]
        if prec == "f64":
            sc = sc.to_double()
        vel = rng.normal(0, 0.01, (sc.n, 3))
        ps, v = host_store(sc, velocity=vel)
        if with_planes:
            planes = np.zeros((2, 2, 3))
            planes[0, 1, 0] = 1.0                       # x = 0, normal +x
            planes[1, 0, 1], planes[1, 1, 1] = 0.01, 1.0  # y = 0.01, normal +y
            v["symmetry_planes"][...] = planes
        orc = OracleScene(v, prec, guards=0)
        rs = ref.RefStore(sc.spec)
        for k in list(sc.init) + ["velocity"] + (["symmetry_planes"] if with_planes else []):
            rs.view(k)[...] = v[k]
        n = sc.n
        orc.setup_solid()
        for k in ("init_original_position", "compute_particle_bins", "compute_original_density"):
            rs.call(mat, prec, k, n)
        kick = rng.normal(0, 5e-4, (n, 3)).astype(orc.T)
        orc.a["position"][:n] += kick
        rs.view("position")[:n] += kick
        recipe = ["compute_density", "compute_rotations_and_strains" if mat == "corot" else "compute_deformations",
                  "compute_stresses", "compute_forces_solids", "step_forward"]
        for _ in range(3):
            orc.substep(mat)
            rs.call(mat, prec, "compute_particle_bins", n)
            for k in recipe:
                rs.call(mat, prec, k, n)
        for k in ["position", "velocity", "density", "density0", "force", "num_neighbours", "cellparticles",
                  "gridcell"] + SOLID_OUT[mat]:
            want = rs.view(k)[:n]
            if prec == "f32" or want.dtype.kind in "ui":
                assert np.array_equal(orc.a[k][:n].reshape(want.shape), want), (k, case)
            else:
                check(orc.a[k][:n], want, k)
        rs.free()
        free_data_cpu(ps)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_bodies_and_constraints_live(prec):
    """set_body_position, set_body_rotation (rigidbody.cl) and
    apply_plane_constraints (constraints.cl) on seeded random scenes --
    three kinematic bodies with random members (particle 0 in a body or
    not), poses, moves and rotations; two random constraint planes with
    random particle masks -- in the oracle (guards off) and in the
    reference's compiled kernels: equal bit for bit in FP32, as the golden
    files are checked in FP64."""
    from oracle import ref
    if not ref.available():
        pytest.skip("oracle/_ref not built on this machine")
    rng = np.random.default_rng(31 + (prec == "f64"))
    for case in range(4):
        sc = scenes.solid_lattice(*[int(x) for x in rng.integers(3, 6, 3)], material="corot", clamp_layers=0,
                                  seed=int(rng.integers(1000)), jitter=1e-3)
        sc.entries = [("body_count", "1", "unsigned int", 3) if e[0] == "body_count" else
                      (("plane_constraints", "3, 2, 2", "float", None) if e[0] == "plane_constraints" else e)
                      for e in sc.entries]
        if prec == "f64":
            sc = sc.to_double()
        n = sc.n
        members = rng.integers(0, 4, n).astype(np.uint32)
        members[0] = int(rng.integers(0, 4))
        pc = np.zeros((2, 2, 3))
        pc[:, 0] = rng.uniform(0.0, 0.03, (2, 3))
        nrm = rng.normal(size=(2, 3))
        pc[:, 1] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
        values = {"body_number": members, "body_dynamic": np.zeros(3, np.uint32),
                  "velocity": rng.normal(0, 0.1, (n, 3)), "plane_constraints": pc,
                  "plane_constraints_particles": rng.integers(0, 4, n).astype(np.uint32),
                  "body_position": rng.uniform(0, 0.05, (3, 3)),
                  "body_euler_rotation": rng.uniform(-1, 1, (3, 3)),
                  "rotation": np.tile(np.eye(3), (n, 1, 1))}
        ps, v = host_store(sc, **values)
        orc = OracleScene(v, prec, guards=0)
        rs = ref.RefStore(sc.spec)
        for k in list(sc.init) + list(values):
            rs.view(k)[...] = v[k]
        for step in range(3):
            body = int(rng.integers(0, 3))
            move = rng.uniform(-0.02, 0.02, 3)
            orc.set_body_position(body, move)
            rs.call("corot", prec, "set_body_position", n, body=body, vec=tuple(move.astype(orc.T)))
            euler = rng.uniform(-np.pi, np.pi, 3)
            orc.set_body_rotation(body, euler)
            rs.call("corot", prec, "set_body_rotation", n, body=body, vec=tuple(euler.astype(orc.T)))
            orc.call("apply_plane_constraints")
            rs.call("corot", prec, "apply_plane_constraints", n)
            for k in ("position", "velocity", "rotation", "body_position", "body_euler_rotation"):
                want = rs.view(k)
                got = orc.a[k][: want.shape[0]].reshape(want.shape)
                if prec == "f32":
                    assert np.array_equal(got, want), (k, case, step)
                else:
                    check(got, want, k)
        rs.free()
        free_data_cpu(ps)


def test_oracle_matches_compiled_reference_live_fluid_edges():
    """Seeded fluid scenes with the cases the neighbour search must get
    right: a dense cluster (stencil rows of more than 64 candidates),
    particles past the grid's upper bounds (clamped into edge cells) and
    n < pnum (the tail ignored); three substeps in the oracle (guards off)
    and in the reference's compiled kernels, FP32, equal bit for bit."""
    from oracle import ref
    if not ref.available():
        pytest.skip("oracle/_ref not built on this machine")
    rng = np.random.default_rng(41)
    for case in range(3):
        sc = scenes.wcsph_block(10, 6, 5, jitter=0.0, seed=0, walls=False)  # pnum 300, grid [0, 0.4]^3, h 0.02
        P = sc.n
        pos = np.empty((P, 3))
        pos[:200] = rng.uniform(0.05, 0.2, (200, 3))
        centre = rng.uniform(0.08, 0.15, 3)
        d = rng.normal(size=(80, 3))
        pos[200:280] = centre + 0.012 * d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(0.1, 1, (80, 1))
        pos[280:] = rng.uniform(0.38, 0.47, (20, 3))
        n = P - int(rng.integers(0, 15))
        # the cluster's particles start with more than 64 neighbours each
        r = np.linalg.norm(pos[200:280, None] - pos[None, 200:280], axis=2)
        assert (r < 0.02).sum(axis=1).min() > 64
        ps, v = host_store(sc, position=pos, n=n, velocity=rng.normal(0, 0.05, (P, 3)))
        orc = OracleScene(v, "f32", guards=0)
        rs = ref.RefStore(sc.spec)
        for k in ("position", "n", "velocity"):
            rs.view(k)[...] = v[k]
        for _ in range(3):
            orc.substep("fluid")
            rs.call("fluid", "f32", "compute_particle_bins", P)
            for k in ("compute_density", "compute_forces_fluids", "step_forward"):
                rs.call("fluid", "f32", k, P)
        for k in ("position", "velocity", "density", "force", "num_neighbours", "gridcell", "cellparticles"):
            want = rs.view(k)[:n]
            assert np.array_equal(orc.a[k][:n].reshape(want.shape), want), (k, case)
        for k in ("gridcount", "celloffset"):
            assert np.array_equal(orc.a[k], rs.view(k).reshape(-1)), (k, case)
        rs.free()
        free_data_cpu(ps)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_oracle_scene_builders_live(prec):
    """populate_position_cuboid and rotate_particles (common.cl:533-604) on
    seeded random cuboids (8 to 216 points against pnum 120, so below and
    above it; corners in any order) and angles, in the oracle and in the
    reference's compiled kernels: positions and n equal bit for bit."""
    from oracle import ref
    if not ref.available():
        pytest.skip("oracle/_ref not built on this machine")
    rng = np.random.default_rng(51 + (prec == "f64"))
    sc = scenes.wcsph_block(6, 5, 4, jitter=0.0, seed=0, walls=False)  # pnum 120
    if prec == "f64":
        sc = sc.to_double()
    for case in range(12):
        ps, v = host_store(sc)
        orc = OracleScene({k: np.array(a) for k, a in v.items()}, prec)
        rs = ref.RefStore(sc.spec)
        rs.view("position")[...] = v["position"]
        free_data_cpu(ps)
        orc.state.n = 0
        rs.view("n")[...] = 0
        c1 = rng.uniform(-1, 1, 3)
        c2 = rng.uniform(-1, 1, 3)
        # at least 2 points per axis: with 1 the reference divides 0 by 0
        size = [int(x) for x in rng.integers(2, 7, 3)]
        orc.populate_position_cuboid(c1, c2, size)
        rs.populate_cuboid("fluid", prec, tuple(c1), tuple(c2), tuple(size))
        assert orc.n == int(np.ravel(rs.view("n"))[0]), case
        assert np.array_equal(orc.a["position"], rs.view("position")), case
        for _ in range(2):
            ang = rng.uniform(-4, 4, 3)
            orc.rotate_particles(*ang)
            rs.rotate("fluid", prec, tuple(ang), sc.n)
            assert np.array_equal(orc.a["position"], rs.view("position")), case
        rs.free()
