"""Seeded synthetic scenes in the reference's store format.

Each builder returns a :class:`Scene`: the $psdata_specification text, the
$opencl_kernel_files list, and initial field values.  The scenes are the
workloads of the benchmark (all synthetic; no dataset is involved):

* :func:`wcsph_block` -- WCSPH fluid lattice in the corner of a box (the
  8,000-particle dam break at 20^3, and the 1,048,576-particle 128^3 block);
* :func:`solid_lattice` -- corotational or St. Venant-Kirchhoff solid
  lattice with clamped layers (the 10x10x40 beam);
* :func:`batch_mix` -- many uneven scenes, 60% fluid / 25% corotational /
  15% SVK, particle counts log-uniform;
* :func:`rigid_body_scene` -- a rigid ball (the rigid-body extension),
  alone or dropped into a fluid block.

Lattices are x-fastest, so particle order follows the grid's cell order.
"""
import math

import numpy as np

FLUID_KERNELS = "common, fluids"
COROT_KERNELS = "common, solids, solid_corotation, constraints, rigidbody"
SVK_KERNELS = "common, solids, solid_svk, constraints, rigidbody"


def _fmt(v):
    if isinstance(v, (list, tuple, np.ndarray)):
        return ", ".join(_fmt(x) for x in np.ravel(v))
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return repr(float(v))


class Scene(object):
    """A store specification plus initial values.  `gen`, for a lattice
    scene jittered by the counter-based generator, holds the lattice
    parameters with which sph_batch_add_lattice builds the same particle
    fields on the device."""

    def __init__(self, name, material, kernel_files, entries, init, n, gen=None):
        self.name = name
        self.material = material          # 'fluid' | 'corot' | 'svk'
        self.kernel_files = kernel_files
        self.entries = entries            # (name, dims, type, value or None)
        self.init = init                  # field -> array (set after build)
        self.n = n
        self.gen = gen

    @property
    def spec(self):
        lines = []
        for name, dims, typ, val in self.entries:
            line = "%s | %s | %s" % (name, dims, typ)
            if val is not None:
                line += " | " + _fmt(val)
            lines.append(line)
        return "\n".join(lines) + "\n"

    def param(self, name):
        for n, _, _, v in self.entries:
            if n == name:
                return v
        raise KeyError(name)

    def to_double(self):
        """The same scene with every float field declared double (the FP64
        run that errors are reported against)."""
        ents = [(n, d, "double" if t == "float" else t, v) for n, d, t, v in self.entries]
        return Scene(self.name + "-fp64", self.material, self.kernel_files, ents, self.init, self.n)

    def system(self):
        """A ParticleSystem on the device with the initial values uploaded."""
        from .systems import ParticleSystem
        ps = ParticleSystem(spec=self.spec, kernel_files=self.kernel_files)
        ps.set_fields(True, **self.init)
        ps.sync_host_to_device()
        return ps


def splitmix64(x):
    """splitmix64 (Steele, Lea and Flood, 2014) of a uint64 array."""
    x = np.asarray(x, dtype=np.uint64)
    z = x + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def hash_jitter(count, seed, jitter):
    """(count, 3) offsets jitter * (2u - 1), u the top 53 bits of
    splitmix64(seed * 2^32 + 3p + axis) over 2^53, in IEEE double: the
    device lattice builder (sph_batch_add_lattice) computes the same."""
    ctr = np.uint64(seed) * np.uint64(1 << 32) + np.arange(3 * count, dtype=np.uint64)
    u = (splitmix64(ctr) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return (float(jitter) * (2.0 * u - 1.0)).reshape(count, 3)


def lattice(nx, ny, nz, spacing, origin=(0.0, 0.0, 0.0), jitter=0.0, rng=None, hash_seed=None):
    """x-fastest (nx*ny*nz, 3) lattice at `spacing` from `origin`, each
    coordinate jittered uniformly in [-jitter, jitter]: from `rng`, or with
    `hash_seed` from the counter-based generator of hash_jitter (the
    device builder's)."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([i.T.ravel(), j.T.ravel(), k.T.ravel()], axis=1).astype(np.float64) * spacing
    p += np.asarray(origin, dtype=np.float64)
    if hash_seed is not None:
        if jitter:
            p += hash_jitter(p.shape[0], hash_seed, jitter)
    elif jitter:
        rng = rng if rng is not None else np.random.default_rng(0)
        p += rng.uniform(-jitter, jitter, size=p.shape)
    return p.astype(np.float32)


def _gen(nx, ny, nz, spacing, origin, jitter, seed, clamp_layers=0, identity_rotation=0):
    return {"nx": int(nx), "ny": int(ny), "nz": int(nz), "spacing": float(spacing),
            "origin": tuple(float(o) for o in origin), "jitter": float(jitter), "seed": int(seed),
            "clamp_layers": int(clamp_layers), "identity_rotation": int(identity_rotation)}


def _common_entries(pnum, mass, dt, h, gravity, gridbounds, nplanes=0, body_count=1):
    return [
        ("pnum", "1", "unsigned int", pnum),
        ("n", "1", "unsigned int", None),
        ("mass", "1", "float", mass),
        ("timestep", "1", "float", dt),
        ("smoothingradius", "1", "float", h),
        ("gravity", "3", "float", list(gravity)),
        ("position", "3, pnum", "float", None),
        ("posnext", "3, pnum", "float", None),
        ("velocity", "3, pnum", "float", None),
        ("veleval", "3, pnum", "float", None),
        ("acceleration", "3, pnum", "float", None),
        ("force", "3, pnum", "float", None),
        ("density", "pnum", "float", None),
        ("num_neighbours", "pnum", "unsigned int", None),
        ("gridbounds", "2, 3", "float", list(gridbounds)),
        ("symmetry_planes", "3, 2, %d" % nplanes, "float", None),
        ("body_number", "pnum", "unsigned int", None),
        ("body_count", "1", "unsigned int", body_count),
        ("body_dynamic", "body_count", "unsigned int", None),
    ]


def wcsph_block(nx=20, ny=20, nz=20, spacing=0.01, h=0.02, box=(0.0, 0.4), jitter=1e-4, seed=0,
                restdens=1000.0, stiffness=3.0, viscosity=0.2, gravity=(0.0, -9.8, 0.0), dt=1e-4,
                mass=None, walls=True, pnum=None, name=None, jitter_hash=False):
    """WCSPH fluid lattice in the low corner of the cube box^3 (the dam
    break).  `walls` adds the reflective-box extension at the box faces.
    `jitter_hash`: the counter-based jitter, so that the device builder
    (Batch.add_lattice) can make the scene without the host arrays."""
    rng = np.random.default_rng(seed)
    origin = (box[0] + spacing / 2,) * 3
    pos = lattice(nx, ny, nz, spacing, origin=origin, jitter=jitter, rng=rng,
                  hash_seed=seed if jitter_hash else None)
    n = pos.shape[0]
    pnum = pnum or n
    if mass is None:
        mass = restdens * spacing ** 3
    gb = [box[0], box[1]] * 3
    entries = _common_entries(pnum, mass, dt, h, gravity, gb)
    entries += [("restdens", "1", "float", restdens), ("stiffness", "1", "float", stiffness),
                ("viscosity", "1", "float", viscosity)]
    if walls:
        entries.append(("wallbounds", "6", "float", gb))
    gen = _gen(nx, ny, nz, spacing, origin, jitter, seed) if jitter_hash else None
    return Scene(name or "wcsph-%d" % n, "fluid", FLUID_KERNELS, entries, {"position": pos, "n": n}, n, gen)


def wcsph_slab_1m(seed=0):
    """The 1,048,576-particle WCSPH slab: 128 x 64 x 128 at 0.005 m (the
    configuration's count; a 128^3 lattice would hold 2,097,152), h = 0.01
    m, +-5e-5 m jitter, on the floor of a [0,1]^3 box with reflective
    walls, dt = 2e-5 s.  The reference's fluid force omits the neighbour
    mass (fluids.cl:43-56), so stiffness and viscosity act per unit
    particle mass: at 1/8 of the dam break's particle mass its 3 and 0.2
    are scaled to 0.375 and 0.025 (unscaled, the slab blows up within ten
    substeps)."""
    return wcsph_block(128, 64, 128, spacing=0.005, h=0.01, box=(0.0, 1.0), jitter=5e-5, seed=seed, dt=2e-5,
                       walls=True, stiffness=0.375, viscosity=0.025, name="wcsph-1m")


def ball_points(radius, spacing, center):
    """Lattice points within `radius` of `center` (x-fastest order)."""
    k = int(math.floor(radius / spacing))
    g = np.arange(-k, k + 1) * spacing
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    p = p[np.sum(p * p, axis=1) <= radius * radius * (1 + 1e-9)]
    return (p + np.asarray(center, dtype=np.float64)).astype(np.float32)


def rigid_body_scene(radius=0.05, spacing=0.01, h=0.02, center=(0.2, 0.2, 0.2), velocity=(0.0, 0.0, 0.0),
                     omega=(0.0, 0.0, 0.0), fluid=None, box=(0.0, 0.4), gravity=(0.0, -9.8, 0.0), dt=1e-4,
                     restdens=1000.0, stiffness=3.0, viscosity=0.2, jitter=1e-4, seed=0, walls=True, name=None,
                     balls=None):
    """Rigid balls (body_dynamic = 2: the rigid-body extension) of lattice
    particles, optionally in a WCSPH fluid block `fluid` = (nx, ny, nz)
    filling the low corner of the box.  One ball of `radius` at `center`
    with linear velocity `velocity` and angular velocity `omega` about its
    centre, or several: `balls` = [(radius, center, velocity, omega), ...],
    body 1, 2, ... in that order.  The balls' particles come after the
    fluid's; they carry the store's particle mass, so a ball is as dense as
    the fluid."""
    rng = np.random.default_rng(seed)
    parts, body, vels = [], [], []
    if fluid is not None:
        f = lattice(*fluid, spacing, origin=(box[0] + spacing / 2,) * 3, jitter=jitter, rng=rng)
        parts.append(f)
        body.append(np.zeros(len(f), np.uint32))
        vels.append(np.zeros((len(f), 3)))
    for k, (rad, cen, v0, w0) in enumerate(balls or [(radius, center, velocity, omega)]):
        b = ball_points(rad, spacing, cen)
        parts.append(b)
        body.append(np.full(len(b), k + 1, np.uint32))
        r = b.astype(np.float64) - np.asarray(cen, dtype=np.float64)
        vels.append(np.asarray(v0, dtype=np.float64) + np.cross(np.asarray(w0, dtype=np.float64), r))
    nb = len(balls or [0])
    pos = np.concatenate(parts).astype(np.float32)
    bn = np.concatenate(body)
    vel = np.concatenate(vels).astype(np.float32)
    n = len(pos)
    mass = restdens * spacing ** 3
    gb = [box[0], box[1]] * 3
    entries = _common_entries(n, mass, dt, h, gravity, gb, body_count=nb)
    entries += [("restdens", "1", "float", restdens), ("stiffness", "1", "float", stiffness),
                ("viscosity", "1", "float", viscosity), ("body_position", "3, body_count", "float", None)]
    if walls:
        entries.append(("wallbounds", "6", "float", gb))
    init = {"position": pos, "n": n, "velocity": vel, "body_number": bn,
            "body_dynamic": np.full(nb, 2, np.uint32)}
    return Scene(name or "rigid-%d" % n, "fluid", FLUID_KERNELS, entries, init, n)


def large_scene(seed=0):
    """The large single-scene configuration as two scenes: 1,048,576 WCSPH
    particles (128 x 64 x 128 at 0.005 m, h = 0.01 m, +-5e-5 m jitter, in
    [0,1]^3, dt = 2e-5 s) with a rigid ball of radius 0.05 m dropped into
    them (4,169 lattice particles, the rigid-body extension), and a 32^3 SVK
    cube (E = 5e4 Pa, nu = 0.35) at the same spacing.  Mixed materials
    within one store are not a reference feature, so the cube is its own
    scene.  The fluid's stiffness and viscosity are the dam break's scaled
    by the 1/8 particle mass (the reference's force omits the neighbour
    mass)."""
    fluid = rigid_body_scene(radius=0.05, spacing=0.005, h=0.01, center=(0.32, 0.45, 0.32), fluid=(128, 64, 128),
                             box=(0.0, 1.0), dt=2e-5, stiffness=0.375, viscosity=0.025, jitter=5e-5, seed=seed,
                             name="large-fluid+ball")
    cube = solid_lattice(32, 32, 32, spacing=0.005, h=0.01, material="svk", youngs_modulus=5e4, poisson=0.35,
                         dt=2e-5, clamp_layers=0, jitter=5e-5, seed=seed + 1, name="large-svk-cube")
    return [fluid, cube]


MIXED_KERNELS = "common, fluids, solids, solid_svk, rigidbody"


def fluid_solid_scene(fluid=(12, 8, 12), cube=(6, 6, 6), cube_origin=None, cube_velocity=(0.0, 0.0, 0.0),
                      ball=None, spacing=0.01, h=0.02, box=(0.0, 0.4), restdens=1000.0, stiffness=3.0,
                      viscosity=0.2, youngs_modulus=5e4, poisson=0.35, solid_viscosity=6e-5,
                      gravity=(0.0, -9.8, 0.0), dt=1e-4, jitter=1e-4, seed=0, walls=True, gridbounds=None,
                      name=None):
    """Fluid, an elastic St. Venant-Kirchhoff cube and optionally a rigid
    ball in one interacting scene (the mixed-scene extension: the store
    lists both fluids.cl and solid_svk.cl, and `phase` tells each particle's
    law -- 0 fluid, 1 solid).  The fluid block fills the low corner of the
    box; the cube (cube = lattice counts) sits at `cube_origin` (default:
    resting on the fluid's surface, centred over it) with an initial
    velocity; `ball` = (radius, center, velocity) adds a rigid body of
    fluid-phase particles (body_dynamic 2).  Every particle carries the
    store's mass (restdens spacing^3), so the cube and the ball are as
    dense as the fluid.  Particle order: fluid, cube, ball."""
    rng = np.random.default_rng(seed)
    origin = (box[0] + spacing / 2,) * 3
    f = lattice(*fluid, spacing, origin=origin, jitter=jitter, rng=rng)
    if cube_origin is None:
        top = origin[1] + (fluid[1] - 1) * spacing
        cube_origin = (origin[0] + 0.5 * (fluid[0] - cube[0]) * spacing, top + spacing,
                       origin[2] + 0.5 * (fluid[2] - cube[2]) * spacing)
    c = lattice(*cube, spacing, origin=cube_origin, jitter=jitter, rng=rng)
    parts, phase, body, vel = [f, c], [np.zeros(len(f), np.uint32), np.ones(len(c), np.uint32)], \
        [np.zeros(len(f), np.uint32), np.zeros(len(c), np.uint32)], \
        [np.zeros((len(f), 3)), np.tile(np.asarray(cube_velocity, np.float64), (len(c), 1))]
    nb = 0
    if ball is not None:
        radius, center, v0 = ball
        b = ball_points(radius, spacing, center)
        parts.append(b)
        phase.append(np.zeros(len(b), np.uint32))
        body.append(np.ones(len(b), np.uint32))
        vel.append(np.tile(np.asarray(v0, np.float64), (len(b), 1)))
        nb = 1
    pos = np.concatenate(parts).astype(np.float32)
    n = len(pos)
    gb = list(gridbounds) if gridbounds is not None else [box[0], box[1]] * 3
    entries = _common_entries(n, restdens * spacing ** 3, dt, h, gravity, gb, body_count=max(nb, 1))
    entries += [("restdens", "1", "float", restdens), ("stiffness", "1", "float", stiffness),
                ("viscosity", "1", "float", viscosity), ("solid_viscosity", "1", "float", solid_viscosity),
                ("youngs_modulus", "1", "float", youngs_modulus), ("poisson", "1", "float", poisson),
                ("originalpos", "3, pnum", "float", None), ("density0", "pnum", "float", None),
                ("deformation", "3, 3, pnum", "float", None), ("stress", "6, pnum", "float", None),
                ("rotation", "3, 3, pnum", "float", None),
                ("cutoff_force", "3, pnum", "float", None), ("force_elastic", "3, pnum", "float", None),
                ("force_viscous", "3, pnum", "float", None), ("padding", "pnum", "unsigned int", None),
                ("body_position", "3, body_count", "float", None),
                ("body_euler_rotation", "3, body_count", "float", None),
                ("phase", "pnum", "unsigned int", None)]
    if walls:
        entries.append(("wallbounds", "6", "float", [box[0], box[1]] * 3))
    init = {"position": pos, "n": n, "velocity": np.concatenate(vel).astype(np.float32),
            "phase": np.concatenate(phase), "body_number": np.concatenate(body),
            "body_dynamic": np.full(max(nb, 1), 2 if nb else 0, np.uint32)}
    sc = Scene(name or "mixed-%d" % n, "mixed", MIXED_KERNELS, entries, init, n)
    sc.counts = {"fluid": len(f), "cube": len(c), "ball": len(parts[2]) if nb else 0}
    return sc


def large_fluid_solid_scene(seed=0):
    """The large single scene as one interacting scene: 1,048,576 WCSPH
    particles (the 128 x 64 x 128 slab of wcsph_slab_1m), a 32^3 SVK cube
    (E = 5e4 Pa, nu = 0.35, 0.005 m spacing) resting on the slab's surface,
    and a rigid ball of radius 0.05 m (4,169 lattice particles) dropped into
    the slab beside it; dt = 2e-5 s.  The fluid's stiffness and viscosity
    are the slab's (the dam break's scaled by its 1/8 particle mass); the
    cube keeps the reference conf's solid viscosity, 6e-5."""
    return fluid_solid_scene(fluid=(128, 64, 128), cube=(32, 32, 32), ball=(0.05, (0.16, 0.40, 0.16), (0.0, 0.0, 0.0)),
                             spacing=0.005, h=0.01, box=(0.0, 1.0), stiffness=0.375, viscosity=0.025,
                             youngs_modulus=5e4, poisson=0.35, solid_viscosity=6e-5, dt=2e-5, jitter=5e-5,
                             seed=seed, name="large-fluid+cube+ball")


def solid_lattice(nx=10, ny=10, nz=40, spacing=0.01, h=0.02, material="corot", youngs_modulus=1e5,
                  poisson=0.3, density=1000.0, viscosity=6e-5, gravity=(0.0, -9.8, 0.0), dt=5e-5,
                  clamp_layers=2, jitter=0.0, seed=0, margin=None, name=None, jitter_hash=False):
    """Elastic lattice whose first `clamp_layers` layers along z belong to
    body 1, a fixed (non-dynamic) body: the clamped beam.  `jitter_hash` as
    for wcsph_block."""
    rng = np.random.default_rng(seed)
    pos = lattice(nx, ny, nz, spacing, jitter=jitter, rng=rng, hash_seed=seed if jitter_hash else None)
    n = pos.shape[0]
    ext = np.array([nx, ny, nz]) * spacing
    m = margin if margin is not None else 4 * h
    sag = max(ext) + m  # room to bend under gravity along -y
    gb = [-m, ext[0] + m, -sag, ext[1] + m, -m, ext[2] + m]
    entries = _common_entries(n, density * spacing ** 3, dt, h, gravity, gb, nplanes=0, body_count=1)
    entries += [
        ("originalpos", "3, pnum", "float", None),
        ("density0", "pnum", "float", None),
        ("stress", "6, pnum", "float", None),
        ("rotation", "3, 3, pnum", "float", None),
        ("viscosity", "1", "float", viscosity),
        ("youngs_modulus", "1", "float", youngs_modulus),
        ("poisson", "1", "float", poisson),
        ("plane_constraints", "3, 2, 0", "float", None),
        ("plane_constraints_particles", "pnum", "unsigned int", None),
        ("cutoff_force", "3, pnum", "float", None),
        ("force_elastic", "3, pnum", "float", None),
        ("force_viscous", "3, pnum", "float", None),
        ("padding", "pnum", "unsigned int", None),
        ("body_position", "3, body_count", "float", None),
        ("body_euler_rotation", "3, body_count", "float", None),
    ]
    if material == "corot":
        entries += [("strain", "6, pnum", "float", None), ("apq_temp", "3, 3, pnum", "float", None),
                    ("intermediate", "3, 3, pnum", "float", None)]
        kernels = COROT_KERNELS
    else:
        entries += [("deformation", "3, 3, pnum", "float", None)]
        kernels = SVK_KERNELS
    layer = nx * ny
    body = np.zeros(n, dtype=np.uint32)
    body[: clamp_layers * layer] = 1
    rot = np.tile(np.eye(3, dtype=np.float32), (n, 1, 1))
    init = {"position": pos, "n": n, "body_number": body, "rotation": rot, "body_dynamic": np.zeros(1, np.uint32)}
    gen = _gen(nx, ny, nz, spacing, (0.0, 0.0, 0.0), jitter, seed, clamp_layers, 1) if jitter_hash else None
    return Scene(name or "%s-%d" % (material, n), material, kernels, entries, init, n, gen)


def _dims_for(n_target, aspect=(1.0, 1.0, 1.0)):
    a = np.asarray(aspect, dtype=np.float64)
    s = (n_target / np.prod(a)) ** (1.0 / 3.0)
    d = np.maximum(2, np.round(a * s)).astype(int)
    return int(d[0]), int(d[1]), int(d[2])


MATERIALS = ("fluid", "corot", "svk")


def mix_member(material, n_target, seed=0, youngs_modulus=1e5, poisson=0.3, spacing=0.01, h=0.02, dt_fluid=1e-4,
               dt_solid=5e-5, jitter=1e-4, name=None, jitter_hash=False):
    """A scene of the batched/served mix with about n_target particles.  A
    fluid block is 1 x 1/2 x 1 and sits in a box twice its width (room to
    collapse); a solid is a 1 x 1 x 2 beam clamped at one end."""
    if material == "fluid":
        nx, ny, nz = _dims_for(n_target, (1.0, 0.5, 1.0))
        ext = max(nx, nz) * spacing
        box_hi = 2.0 * ext + 4 * h
        return wcsph_block(nx, ny, nz, spacing=spacing, h=h, box=(0.0, box_hi), jitter=jitter, seed=seed,
                           dt=dt_fluid, name=name, jitter_hash=jitter_hash)
    nx, ny, nz = _dims_for(n_target, (1.0, 1.0, 2.0))
    return solid_lattice(nx, ny, nz, spacing=spacing, h=h, material=material, youngs_modulus=youngs_modulus,
                         poisson=poisson, dt=dt_solid, clamp_layers=1, jitter=jitter, seed=seed, name=name,
                         jitter_hash=jitter_hash)


def mixed_scene(rng, index, n_range=(1000, 65536), mix=(0.6, 0.25, 0.15), e_range=(1e4, 1e6),
                svk_e_range=(1e4, 1e5), nu_range=(0.25, 0.45), prefix="b", **kw):
    """One random scene of the mix: particle count log-uniform in n_range,
    material drawn with probabilities `mix` (fluid, corotational, SVK),
    Young's modulus log-uniform in e_range (svk_e_range for SVK), Poisson
    ratio uniform in nu_range; seeded lattice jitter (see mix_member).

    SVK scenes are drawn no stiffer than 1e5 Pa: the reference's SVK
    formulation (solid_svk.cl) diverges within 2,000 substeps for a clamped
    beam under gravity once E reaches a few 1e5 Pa -- at the same physical
    time whatever the time step, and in the FP64 restatement as well -- and
    a diverged scene is not work worth timing.  The corotational model
    stays stable over the whole range."""
    n_target = math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))
    kind = int(rng.choice(3, p=np.asarray(mix) / np.sum(mix)))
    sub = int(rng.integers(1 << 30))
    material = MATERIALS[kind]
    if kind == 0:
        return mix_member(material, n_target, seed=sub, name="%s%03d-fluid" % (prefix, index), **kw)
    lo, hi = e_range if kind == 1 else svk_e_range
    E = math.exp(rng.uniform(math.log(lo), math.log(hi)))
    nu = rng.uniform(*nu_range)
    return mix_member(material, n_target, seed=sub, youngs_modulus=E, poisson=nu,
                      name="%s%03d-%s" % (prefix, index, material), **kw)


def batch_mix(count=256, seed=0, **kw):
    """`count` independent scenes of the mix (see mixed_scene)."""
    rng = np.random.default_rng(seed)
    return [mixed_scene(rng, s, **kw) for s in range(count)]
