"""ctypes front end of the CPU oracle (liboracle.so, sph_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py use this module to check results and time
the CPU path.  The product (opencl-sph_gb300/) never imports it.

An :class:`OracleScene` owns NumPy copies of a store's fields (taken from
the arrays a ``ParticleSystem.get_fields`` returns, i.e. with the store's
dimensions reversed) in FP32 or FP64, and runs the reference's kernels on
them through the C restatement.  The substep recipes follow the reference
drivers: scripts/sph/systems.py:194-204 (corotational), :225-235 (SVK) and
src/mex/simstep_fluid.c:18-23 (fluid).
"""
import ctypes
import os
import subprocess
from ctypes import POINTER, Structure, c_double, c_float, c_int, c_uint

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

REAL_FIELDS = ["position", "velocity", "acceleration", "force", "density", "density0", "originalpos",
               "rotation", "strain", "stress", "apq_temp", "intermediate", "deformation", "cutoff_force",
               "force_elastic", "force_viscous"]
UINT_FIELDS = ["num_neighbours", "gridcell", "cellparticles"]
# per-particle widths of the fields above
WIDTH = {"position": 3, "velocity": 3, "acceleration": 3, "force": 3, "density": 1, "density0": 1,
         "originalpos": 3, "rotation": 9, "strain": 6, "stress": 6, "apq_temp": 9, "intermediate": 9,
         "deformation": 9, "cutoff_force": 3, "force_elastic": 3, "force_viscous": 3, "num_neighbours": 1,
         "gridcell": 1, "cellparticles": 1}


def build():
    """Compiles liboracle.so (gcc via oracle/Makefile)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def _state_type(real):
    P = POINTER(real)
    U = POINTER(c_uint)
    return type("state_" + real.__name__, (Structure,), {"_fields_": [
        ("n", c_uint), ("gridres", c_uint * 3),
        ("mass", real), ("timestep", real), ("smoothingradius", real),
        ("restdens", real), ("stiffness", real), ("viscosity", real),
        ("youngs_modulus", real), ("poisson", real),
        ("gravity", real * 3), ("gridbounds", real * 6),
        ("num_symmetry_planes", c_uint), ("symmetry_planes", P),
        ("num_plane_constraints", c_uint), ("plane_constraints", P),
        ("plane_constraints_particles", U),
        ("body_count", c_uint), ("body_number", U), ("body_dynamic", U),
        ("body_position", P), ("body_euler_rotation", P),
        ("position", P), ("velocity", P), ("acceleration", P), ("force", P),
        ("density", P), ("density0", P), ("originalpos", P),
        ("rotation", P), ("strain", P), ("stress", P), ("apq_temp", P), ("intermediate", P),
        ("deformation", P), ("cutoff_force", P), ("force_elastic", P), ("force_viscous", P),
        ("num_neighbours", U), ("gridcell", U), ("gridcount", U), ("celloffset", U), ("cellparticles", U),
        ("has_wallbounds", c_uint), ("wallbounds", real * 6),
        ("guards", c_int), ("nthreads", c_int),
        ("body_capacity", c_uint), ("rigid_state", POINTER(c_double)), ("rigid_offset", P),
        ("phase", U), ("has_solid_viscosity", c_uint), ("solid_viscosity", real),
    ]})

RIGID_STRIDE = 64  # ORACLE_RIGID_STRIDE


_STATES = {"f32": _state_type(c_float), "f64": _state_type(c_double)}
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
    return _lib


class OracleScene(object):
    """CPU oracle copy of one scene."""

    KERNELS = ["find_particle_bins", "sort_particles", "compute_particle_bins", "init_original_position",
               "compute_original_density", "compute_density", "compute_forces_fluids",
               "compute_rotations_and_strains", "compute_stresses_corot", "compute_forces_solids_corot",
               "compute_deformations", "compute_stresses_svk", "compute_forces_solids_svk", "step_forward",
               "apply_plane_constraints", "rigid_step"]

    def __init__(self, fields, prec="f32", nthreads=1, guards=3):
        """`fields`: name -> array as given by ParticleSystem.get_fields
        (scalars as 1-element arrays).  `guards` (see sph_oracle.h): 3
        defines the two cases where the reference yields NaN, as the CUDA
        path does; 0 reproduces the reference bit for bit."""
        self.prec = prec
        self.T = np.float32 if prec == "f32" else np.float64
        real = c_float if prec == "f32" else c_double
        st = _STATES[prec]()
        self.pnum = int(np.ravel(fields["pnum"])[0])
        P = self.pnum
        self.a = {}
        for name in REAL_FIELDS:
            shape = (P, WIDTH[name]) if WIDTH[name] > 1 else (P,)
            if name in ("rotation", "apq_temp", "intermediate", "deformation"):
                shape = (P, 3, 3)
            arr = np.zeros(shape, dtype=self.T)
            if name in fields:
                arr.reshape(-1)[:] = np.asarray(fields[name], dtype=np.float64).reshape(-1)[:arr.size]
            self.a[name] = arr
        # mixed fluid-solid scenes (extension): the per-particle phase
        extra_uint = ["phase"] if "phase" in fields else []
        for name in UINT_FIELDS + ["body_number", "plane_constraints_particles"] + extra_uint:
            arr = np.zeros(P, dtype=np.uint32)
            if name in fields:
                arr[:] = np.asarray(fields[name]).reshape(-1)[:P]
            self.a[name] = arr
        res = np.asarray(fields["gridres"]).reshape(-1).astype(np.uint32)
        C = int(np.prod(res))
        self.a["gridcount"] = np.zeros(C, np.uint32)
        self.a["celloffset"] = np.zeros(C, np.uint32)

        def planes(name):
            # stored as dims (3, 2, count): the view's shape is (count, 2, 3)
            arr = np.asarray(fields.get(name, np.zeros((0, 2, 3))), dtype=np.float64)
            cnt = arr.shape[0] if arr.ndim == 3 else 0
            out = np.zeros((max(cnt, 1), 2, 3), dtype=self.T)
            if cnt:
                out[:] = arr
            return out, cnt

        self.a["symmetry_planes"], nsp = planes("symmetry_planes")
        self.a["plane_constraints"], npc = planes("plane_constraints")
        # a copy: the oracle must not alias the store it was built from
        bd = np.array(fields.get("body_dynamic", np.zeros(1)), dtype=np.uint32).reshape(-1)
        self.a["body_dynamic"] = np.ascontiguousarray(bd if bd.size else np.zeros(1, np.uint32))
        for name in ("body_position", "body_euler_rotation"):
            v = np.asarray(fields.get(name, np.zeros((1, 3))), dtype=np.float64).reshape(-1, 3)
            self.a[name] = np.ascontiguousarray(v if v.size else np.zeros((1, 3)), dtype=self.T)

        def scal(name, default=0.0):
            return float(np.ravel(fields[name])[0]) if name in fields else default

        st.n = int(np.ravel(fields["n"])[0])
        st.gridres[:] = [int(x) for x in res]
        for name in ("mass", "timestep", "smoothingradius", "restdens", "stiffness", "viscosity",
                     "youngs_modulus", "poisson"):
            setattr(st, name, scal(name))
        st.gravity[:] = [float(x) for x in np.ravel(fields["gravity"])[:3]]
        st.gridbounds[:] = [float(x) for x in np.ravel(fields["gridbounds"])[:6]]
        st.num_symmetry_planes = nsp
        st.num_plane_constraints = npc
        st.body_count = int(scal("body_count", 0))
        if "wallbounds" in fields:
            st.has_wallbounds = 1
            st.wallbounds[:] = [float(x) for x in np.ravel(fields["wallbounds"])[:6]]
        st.guards = guards
        st.nthreads = nthreads
        if "solid_viscosity" in fields:
            st.has_solid_viscosity = 1
            st.solid_viscosity = scal("solid_viscosity")
        # rigid bodies (extension): state per body, offsets per particle
        st.body_capacity = int(self.a["body_dynamic"].size)
        self.rigid_state = np.zeros((st.body_capacity, RIGID_STRIDE), np.float64)
        self.a["rigid_offset"] = np.zeros((P, 3), dtype=self.T)
        st.rigid_state = self.rigid_state.ctypes.data_as(POINTER(c_double))
        for name, arr in self.a.items():
            ctype = c_uint if arr.dtype == np.uint32 else real
            setattr(st, name, arr.ctypes.data_as(POINTER(ctype)))
        self.state = st
        self._sfx = "_" + prec

    @property
    def n(self):
        return self.state.n

    def set_scalar(self, name, value):
        setattr(self.state, name, value)

    def call(self, kernel):
        getattr(lib(), "oracle_" + kernel + self._sfx)(ctypes.byref(self.state))

    def set_body_position(self, body, pos):
        v = np.asarray(pos, dtype=self.T)
        ptr = v.ctypes.data_as(POINTER(c_float if self.prec == "f32" else c_double))
        getattr(lib(), "oracle_set_body_position" + self._sfx)(ctypes.byref(self.state), body, ptr)

    def set_body_rotation(self, body, euler):
        v = np.asarray(euler, dtype=self.T)
        ptr = v.ctypes.data_as(POINTER(c_float if self.prec == "f32" else c_double))
        getattr(lib(), "oracle_set_body_rotation" + self._sfx)(ctypes.byref(self.state), body, ptr)

    def populate_position_cuboid(self, corner1, corner2, size):
        """populate_position_cuboid (common.cl:533-555): a lattice spanning
        corner1..corner2 with size[a] points per axis, at most pnum of them."""
        T = c_float if self.prec == "f32" else c_double
        getattr(lib(), "oracle_populate_position_cuboid" + self._sfx)(
            ctypes.byref(self.state), c_uint(self.pnum), (T * 3)(*corner1), (T * 3)(*corner2),
            (c_uint * 3)(*[int(x) for x in size]))

    def rotate_particles(self, ax, ay, az):
        """rotate_particles (common.cl:556-604)."""
        T = c_float if self.prec == "f32" else c_double
        getattr(lib(), "oracle_rotate_particles" + self._sfx)(ctypes.byref(self.state), T(ax), T(ay), T(az))

    def reset_rigid(self):
        """Rigid bodies are set up again from the particles on their next
        substep (what a host upload of positions does on the device)."""
        self.rigid_state[:, 0] = 0.0

    # the reference's driver recipes ------------------------------------------
    def setup_solid(self):
        """StrainSolid.setup (systems.py:185-192)."""
        self.call("init_original_position")
        self.call("compute_particle_bins")
        self.call("compute_original_density")

    def substep(self, material):
        self.call("compute_particle_bins")
        self.call("compute_density")
        if material == "fluid":
            self.call("compute_forces_fluids")
        elif material == "corot":
            self.call("compute_rotations_and_strains")
            self.call("compute_stresses_corot")
            self.call("compute_forces_solids_corot")
        elif material == "svk":
            self.call("compute_deformations")
            self.call("compute_stresses_svk")
            self.call("compute_forces_solids_svk")
        elif material == "mixed":
            # fluid and SVK particles in one scene (extension): the solids'
            # elastic passes, then the fluid pass, which adds the fluid pair
            # terms to the solids' elastic forces
            self.call("compute_deformations")
            self.call("compute_stresses_svk")
            self.call("compute_forces_solids_svk")
            self.call("compute_forces_fluids")
        else:
            raise ValueError(material)
        self.call("step_forward")
        self.call("rigid_step")  # rigid bodies (extension); nothing without any

    def run(self, material, steps):
        for _ in range(steps):
            self.substep(material)
