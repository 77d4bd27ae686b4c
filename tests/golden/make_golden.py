"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout that holds the reference (SPH_REFERENCE_ROOT, default
/root/reference) after `python oracle/make_ref.py`:

    python tests/golden/make_golden.py

Writes:
  layouts.json      psdata layouts that the reference's own builder
                    (src/build_psdata.c, compiled into oracle/_ref) gives for
                    a set of specifications: the repository's conf files,
                    the scene builders' specifications and edge cases.
  kernels_*.npz     small seeded scenes run through the reference's own
                    kernels (kernels/*.cl compiled as C++ into oracle/_ref)
                    in FP32 and FP64: each kernel's inputs and outputs.
  kernels_scene_builders.npz
                    populate_position_cuboid and rotate_particles
                    (common.cl:533-604) on a few ranges and angle sets.

    python tests/golden/make_golden.py scene_builders   # only that file

The tests compare the product's builder, the C oracle and the GPU path
against these files; nothing at test time reads the reference checkout.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "opencl-sph_gb300"))

from oracle import ref  # noqa: E402
from sph import scenes  # noqa: E402

EDGE_SPECS = {
    # first field a 3-vector of doubles: the reference's alignment of the
    # first field wraps around (build_psdata.c:381)
    "double-first": "smoothingradius | 1 | double | 0.1\ngridbounds | 2, 3 | double | 0, 1, 0, 1, 0, 1\n"
                    "pnum | 1 | unsigned int | 10\nv | 3, pnum | double\nw | pnum | float\nq | 3 | double | 1, 2, 3\n",
    "mixed-types": "# comment\npnum | 1 | unsigned int | 0x10\nsmoothingradius | 1 | float | 0.25\n"
                   "gridbounds | 2, 3 | float | -1, 1, -2, 2, 0, 0.5\nk | pnum | int | -3\n"
                   "u | 2, pnum | uint | 7\nc | 5 | char\nx | 3, 2, pnum | float\n",
    "dims-by-name": "pnum | 1 | unsigned int | 5\nbodies | 1 | unsigned int | 3\nsmoothingradius | 1 | float | 0.1\n"
                    "gridbounds | 2, 3 | float | 0, 1, 0, 1, 0, 1\nbp | 3, bodies | float\nbd | bodies | unsigned int | 1, 0, 1\n"
                    "missing | 2, nosuchfield | float\n",
    "fp32-grid-truncation": "pnum | 1 | unsigned int | 8\nsmoothingradius | 1 | float | 0.1\n"
                            "gridbounds | 2, 3 | float | -2.0, 2.0, -2.0, 2.0, -2.0, 2.0\n",
}


def conf_section(path, heading):
    text = open(path).read()
    parts = text.split("$")
    for p in parts[1:]:
        title, _, body = p.partition("\n")
        if title.strip() == heading:
            return body
    raise KeyError(heading)


def layouts():
    out = {}
    specs = dict(EDGE_SPECS)
    confdir = os.path.join(ROOT, "opencl-sph_gb300", "conf")
    for f in sorted(os.listdir(confdir)):
        specs["conf/" + f] = conf_section(os.path.join(confdir, f), "psdata_specification")
    specs["scene/wcsph"] = scenes.wcsph_block(6, 5, 4).spec
    specs["scene/beam"] = scenes.solid_lattice(4, 4, 6).spec
    specs["scene/svk"] = scenes.solid_lattice(4, 4, 6, material="svk").spec
    for name, spec in specs.items():
        rs = ref.RefStore(spec)
        L = dict(rs.layout)
        L["size"] = rs.size
        gr = L["names"].index("gridres") if "gridres" in L["names"] else -1
        L["gridres"] = [int(x) for x in rs.view("gridres")] if gr >= 0 else None
        out[name] = {"spec": spec, "layout": L}
        rs.free()
    with open(os.path.join(HERE, "layouts.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("layouts.json: %d specifications" % len(out))


SAVE = ["position", "velocity", "acceleration", "force", "density", "num_neighbours", "gridcell", "gridcount",
        "celloffset", "cellparticles", "density0", "originalpos", "rotation", "strain", "stress", "apq_temp",
        "intermediate", "deformation", "cutoff_force", "force_elastic", "force_viscous", "body_position",
        "body_euler_rotation", "symmetry_planes", "plane_constraints", "plane_constraints_particles",
        "body_number", "body_dynamic", "n"]


# fields each kernel writes (only these are recorded after it runs)
OUTPUTS = {
    "compute_particle_bins": ["gridcell", "gridcount", "celloffset", "cellparticles"],
    "compute_density": ["density", "num_neighbours"],
    "compute_forces_fluids": ["force"],
    "step_forward": ["position", "velocity", "acceleration"],
    "compute_rotations_and_strains": ["rotation", "strain", "apq_temp", "intermediate"],
    "compute_deformations": ["deformation"],
    "compute_stresses": ["stress"],
    "compute_forces_solids": ["force", "force_elastic", "force_viscous", "cutoff_force"],
    "set_body_position": ["position", "velocity", "body_position"],
    "set_body_rotation": ["position", "rotation", "body_euler_rotation"],
    "apply_plane_constraints": ["position", "velocity"],
}


def _snapshot(rs, prefix, out, fields=None):
    for k in (fields or SAVE):
        if k in rs.layout["names"]:
            out[prefix + k] = np.array(rs.view(k))


def _set(rs, values):
    for k, v in values.items():
        rs.view(k)[...] = v


def run_scene(tag, scene, program, setup_values, steps, solid, planes=None, extra=None):
    rec = {"spec": np.array(scene.spec), "kernels": np.array(scene.kernel_files),
           "material": np.array(scene.material)}
    for prec in ("f32", "f64"):
        sc = scene if prec == "f32" else scene.to_double()
        rs = ref.RefStore(sc.spec)
        vals = dict(setup_values)
        _set(rs, vals)
        if planes is not None:
            rs.view("symmetry_planes")[...] = planes
        n = int(np.ravel(rs.view("n"))[0])
        _snapshot(rs, prec + "/init/", rec)
        if solid:
            for k in ("init_original_position", "compute_particle_bins", "compute_original_density"):
                rs.call(program, prec, k, n)
            _snapshot(rs, prec + "/setup/", rec)
            # deform the lattice (the same perturbation in both precisions)
            rng = np.random.default_rng(17)
            rs.view("position")[:n] += rng.normal(0, 5e-4, (n, 3)).astype(rs.view("position").dtype)
            _snapshot(rs, prec + "/deformed/", rec, ["position"])
        recipe = {"fluid": ["compute_density", "compute_forces_fluids"],
                  "corot": ["compute_density", "compute_rotations_and_strains", "compute_stresses",
                            "compute_forces_solids"],
                  "svk": ["compute_density", "compute_deformations", "compute_stresses",
                          "compute_forces_solids"]}[scene.material]
        # first substep kernel by kernel
        rs.call(program, prec, "compute_particle_bins", n)
        _snapshot(rs, prec + "/s1/compute_particle_bins/", rec, OUTPUTS["compute_particle_bins"])
        for k in recipe + ["step_forward"]:
            rs.call(program, prec, k, n)
            _snapshot(rs, prec + "/s1/" + k + "/", rec, OUTPUTS[k])
        for _ in range(steps - 1):
            rs.call(program, prec, "compute_particle_bins", n)
            for k in recipe + ["step_forward"]:
                rs.call(program, prec, k, n)
        _snapshot(rs, prec + "/final/", rec)
        if extra:
            extra(rs, program, prec, n, rec)
        rs.free()
    rec["steps"] = np.array(steps)
    np.savez_compressed(os.path.join(HERE, "kernels_%s.npz" % tag), **rec)
    print("kernels_%s.npz" % tag)


def bodies_and_constraints(rs, program, prec, n, rec):
    rs.view("body_position")[...] = np.array([[0.01, 0.02, 0.03]] + [[0, 0, 0]] * (rs.view("body_position").shape[0] - 1))
    rs.view("body_euler_rotation")[...] = np.array([[0.1, 0.2, 0.3]] + [[0, 0, 0]] * (rs.view("body_position").shape[0] - 1))
    _snapshot(rs, prec + "/body_init/", rec)
    rs.call(program, prec, "set_body_position", n, body=0, vec=(0.02, 0.0, 0.05))
    _snapshot(rs, prec + "/set_body_position/", rec, OUTPUTS["set_body_position"])
    rs.call(program, prec, "set_body_rotation", n, body=0, vec=(0.3, -0.2, 0.1))
    _snapshot(rs, prec + "/set_body_rotation/", rec, OUTPUTS["set_body_rotation"])
    if rs.view("plane_constraints").shape[0] > 0:
        pc = np.zeros(rs.view("plane_constraints").shape)
        pc[0, 0, 0], pc[0, 1, 0] = 0.01, 1.0
        pc[1, 1] = [0.6, 0.8, 0.0]
        rs.view("plane_constraints")[...] = pc
        rng = np.random.default_rng(3)
        rs.view("plane_constraints_particles")[:n] = rng.integers(0, 4, n)
        rs.view("velocity")[:n] = rng.normal(0, 0.1, (n, 3))
        _snapshot(rs, prec + "/constraints_init/", rec)
        rs.call(program, prec, "apply_plane_constraints", n)
        _snapshot(rs, prec + "/apply_plane_constraints/", rec, OUTPUTS["apply_plane_constraints"])


# (corner1, corner2, size) ranges of populate_position_cuboid: one that
# fills pnum exactly, one larger than pnum (n = pnum), one smaller (n = its
# size), and a flat one with negative extents
CUBOIDS = [((0.0, 0.0, 0.0), (0.1, 0.05, 0.07), (5, 4, 6)),
           ((-0.2, 0.1, 0.3), (0.4, 0.35, 0.9), (7, 5, 6)),
           ((0.01, 0.02, 0.03), (0.3, 0.2, 0.1), (3, 4, 5)),
           ((0.5, -0.5, 0.25), (-0.5, 0.5, 0.25), (11, 9, 2))]
ANGLES = [(0.3, -0.2, 0.1), (1.2, 0.7, -2.5), (0.0, 0.0, 3.14159265)]


def scene_builders():
    """populate_position_cuboid over CUBOIDS, then rotate_particles by each
    of ANGLES in turn, on a 120-particle store; FP32 and FP64."""
    sc = scenes.wcsph_block(6, 5, 4, jitter=0.0, seed=0, walls=False)
    rec = {"spec": np.array(sc.spec)}
    for prec in ("f32", "f64"):
        spec = sc.spec if prec == "f32" else sc.spec.replace("| float", "| double")
        for c, (c1, c2, size) in enumerate(CUBOIDS):
            rs = ref.RefStore(spec)
            rs.view("n")[...] = 0
            rs.populate_cuboid("fluid", prec, c1, c2, size)
            rec["%s/cuboid%d/position" % (prec, c)] = np.array(rs.view("position"))
            rec["%s/cuboid%d/n" % (prec, c)] = np.array(rs.view("n"))
            for a, ang in enumerate(ANGLES):
                rs.rotate("fluid", prec, ang, int(rs.view("n")[0]))
                rec["%s/cuboid%d/rotate%d/position" % (prec, c, a)] = np.array(rs.view("position"))
            rs.free()
    rec["cuboids"] = np.array([list(c1) + list(c2) + list(sz) for c1, c2, sz in CUBOIDS], dtype=np.float64)
    rec["angles"] = np.array(ANGLES, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "kernels_scene_builders.npz"), **rec)
    print("kernels_scene_builders.npz")


def main():
    if not (ref.available("kernels") and ref.available("psdata")):
        raise SystemExit("oracle/_ref is not built: run python oracle/make_ref.py first")
    if sys.argv[1:] == ["scene_builders"]:
        scene_builders()
        return
    scene_builders()
    layouts()
    fl = scenes.wcsph_block(7, 6, 5, jitter=2e-3, seed=1, walls=False)
    rng = np.random.default_rng(2)
    run_scene("fluid", fl, "fluid", {"position": fl.init["position"], "n": fl.n,
                                     "velocity": rng.normal(0, 0.05, (fl.n, 3))}, steps=5, solid=False)
    planes = np.zeros((3, 2, 3))
    for k in range(3):
        planes[k, 1, k] = 1.0
    for mat in ("corot", "svk"):
        for with_planes in (False, True):
            sc = scenes.solid_lattice(5, 4, 6, material=mat, youngs_modulus=2e4, poisson=0.3, jitter=2e-4,
                                      clamp_layers=1, seed=3)
            sc.entries = [("plane_constraints", "3, 2, 2", "float", None) if e[0] == "plane_constraints" else
                          (("symmetry_planes", "3, 2, 3", "float", None) if (e[0] == "symmetry_planes" and with_planes)
                           else e) for e in sc.entries]
            vals = dict(sc.init)
            vals["velocity"] = np.random.default_rng(4).normal(0, 0.01, (sc.n, 3))
            run_scene("%s%s" % (mat, "_planes" if with_planes else ""), sc, mat, vals, steps=3, solid=True,
                      planes=planes if with_planes else None,
                      extra=bodies_and_constraints if (mat == "corot" and not with_planes) else None)


if __name__ == "__main__":
    main()
