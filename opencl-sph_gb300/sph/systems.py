"""Particle systems over a psdata store, mirroring the reference's
scripts/sph/systems.py: zero-copy NumPy views of the store's fields, host/
device syncs, kernels called by name, and the material substep recipes of
``StrainSolid`` (corotational) and ``SVKSolid``, plus ``FluidSystem`` for
WCSPH (the recipe of src/mex/simstep_fluid.c:18-23, which the reference
only drives from MATLAB).

Two deliberate differences from the reference file:
  - ``sync_fields_*`` call the per-field sync functions; the reference calls
    the whole-store ones with extra arguments (systems.py:89-99), which
    copies every field on every call.
  - ``update_fused(steps)`` runs whole substeps as one CUDA graph each
    (sph_update) instead of one call per kernel.
"""
import ctypes
import os.path

import numpy as np

from . import bindings as bnd
from . import init_data, init_data_from_string, free_data

_CONF_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "conf")


class ParticleSystem(object):
    config = None
    numpy_types = {
        bnd.T_CHAR: np.dtype('S1'),
        bnd.T_UINT: np.dtype('u4'),
        bnd.T_INT: np.dtype('i4'),
        bnd.T_FLOAT32: np.dtype('f4'),
        bnd.T_FLOAT64: np.dtype('f8'),
    }

    union_types = {
        bnd.T_CHAR: 'c',
        bnd.T_UINT: 'u',
        bnd.T_INT: 'i',
        bnd.T_FLOAT32: 'f4',
        bnd.T_FLOAT64: 'f8',
    }

    def __init__(self, config=None, spec=None, kernel_files=None):
        """From a .conf file (``config`` or the class's), or from the two
        section texts (``spec`` = $psdata_specification, ``kernel_files`` =
        $opencl_kernel_files)."""
        if spec is not None:
            self._spec = (spec, kernel_files)
            self.psdata, self.psdata_opencl = init_data_from_string(spec, kernel_files)
        else:
            if config is not None:
                self.config = config
            self._spec = None
            result = init_data(self.config)
            if result is None:
                raise IOError("could not read config file {}".format(self.config))
            self.psdata, self.psdata_opencl = result
        self.fields = {}

    def _reinit(self):
        if self._spec is not None:
            return init_data_from_string(*self._spec)
        return init_data(self.config)

    def get_fields(self, *args):
        """Zero-copy views of named fields, dimensions reversed (e.g. a
        `3, pnum` field is a (pnum, 3) array) as in systems.py:34-60."""
        fields = []
        for arg in args:
            if arg not in self.fields:
                f = bnd.get_field_psdata(self.psdata, arg)
                if f == -1:
                    raise Exception("{} is not a field.".format(arg))
                nd = self.psdata.num_dimensions[f]
                off = self.psdata.dimensions_offsets[f]
                dims = [self.psdata.dimensions[off + d] for d in range(nd)]
                ftype = self.psdata.data_ptrs[f].type
                dtype = self.numpy_types[ftype]
                count = int(np.prod(dims)) if dims else 0
                addr = self.psdata.data + self.psdata.data_offsets[f]
                buf = (ctypes.c_char * (count * dtype.itemsize)).from_address(addr)
                self.fields[arg] = np.frombuffer(buf, dtype=dtype, count=count).reshape(tuple(reversed(dims)))
            fields.append(self.fields[arg])
        return tuple(fields)

    def set_fields(self, *args, **kwargs):
        host_only = len(args) > 0 and args[0]
        keys = list(kwargs.keys())
        vals = [kwargs[k] for k in keys]
        fields = self.get_fields(*keys)
        for field, val in zip(fields, vals):
            if type(val) == np.ndarray and val.size > 1:
                np.copyto(field[tuple(slice(None, s) for s in val.shape)], val, casting='unsafe')
            else:
                np.copyto(field, val, casting='unsafe')
        if not host_only:
            self.sync_fields_host_to_device(*keys)

    def sync_host_to_device(self):
        bnd.sync_psdata_host_to_device(self.psdata, self.psdata_opencl, 0)

    def sync_device_to_host(self):
        bnd.sync_psdata_device_to_host(self.psdata, self.psdata_opencl)

    def _names(self, args):
        arr = (ctypes.c_char_p * len(args))()
        arr[:] = [a.encode('utf-8') for a in args]
        return arr

    def sync_fields_host_to_device(self, *args):
        if not args:
            return self.sync_host_to_device()
        bnd.sync_psdata_fields_host_to_device(self.psdata, self.psdata_opencl, len(args), self._names(args))

    def sync_fields_device_to_host(self, *args):
        if not args:
            return self.sync_device_to_host()
        bnd.sync_psdata_fields_device_to_host(self.psdata, self.psdata_opencl, len(args), self._names(args))

    def set_body_position(self, body, position):
        p = np.ascontiguousarray(position, dtype=np.float32)
        bnd.set_body_position_device_opencl(self.psdata_opencl, body, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    def set_body_rotation(self, body, euler_angles):
        e = np.ascontiguousarray(euler_angles, dtype=np.float32)
        bnd.set_body_rotation_device_opencl(self.psdata_opencl, body, e.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    def call_for_all_particles(self, kernel):
        bnd.call_for_all_particles_device_opencl(self.psdata_opencl, kernel)

    def compute_particle_bins(self):
        bnd.compute_particle_bins_device_opencl(self.psdata_opencl)

    def synchronize(self):
        if bnd.sph_synchronize(self.psdata_opencl) != 0:
            raise bnd.SphError(bnd.last_error())

    # asynchronous transfers --------------------------------------------------
    def pin(self):
        """Page-locks the host store, so that the asynchronous transfers
        below run on the copy engines (released by unpin or free)."""
        if bnd.sph_pin_host(self.psdata, self.psdata_opencl) != 0:
            raise bnd.SphError(bnd.last_error())
        self._pinned = True

    def unpin(self):
        if bnd.sph_unpin_host(self.psdata_opencl) != 0:
            raise bnd.SphError(bnd.last_error())
        self._pinned = False

    def write_fields_async(self, *args):
        """sync_fields_host_to_device without the wait: the named fields of
        the host store must stay unchanged until a later blocking call."""
        if bnd.sph_write_fields_async(self.psdata, self.psdata_opencl, len(args), self._names(args)) != 0:
            raise bnd.SphError(bnd.last_error())

    def read_fields_async(self, *args):
        """Snapshots the named fields after the work enqueued so far and
        copies them into the host store while later substeps run; returns a
        ticket for wait_read, after which get_fields sees the snapshot."""
        t = bnd.sph_read_fields_async(self.psdata, self.psdata_opencl, len(args), self._names(args))
        if t < 0:
            raise bnd.SphError(bnd.last_error())
        return t

    def wait_read(self, ticket):
        if bnd.sph_wait_read(self.psdata_opencl, ticket) != 0:
            raise bnd.SphError(bnd.last_error())

    def wait_reads(self):
        if bnd.sph_wait_reads(self.psdata_opencl) != 0:
            raise bnd.SphError(bnd.last_error())

    def status(self):
        return bnd.sph_status(self.psdata_opencl)

    def update_fused(self, steps=1):
        if bnd.sph_update(self.psdata_opencl, steps) != 0:
            raise bnd.SphError(bnd.last_error())

    # device-resident recording ------------------------------------------------
    def record_start(self, fields, every=1, frames=1024):
        """Records `fields` on the device every `every` substeps of
        update_fused into a ring of `frames` frames (no host copy until
        record_read)."""
        names = (ctypes.c_char_p * len(fields))(*[f.encode() for f in fields])
        if bnd.sph_record_start(self.psdata_opencl, len(fields), names, int(every), int(frames)) != 0:
            raise bnd.SphError(bnd.last_error())
        self._rec = list(fields)
        self._rec_frames_n = int(frames)

    def record_stop(self):
        if bnd.sph_record_stop(self.psdata_opencl) != 0:
            raise bnd.SphError(bnd.last_error())
        self._rec = None

    def record_count(self):
        """Frames recorded so far (the ring keeps the last `frames`)."""
        return int(bnd.sph_record_count(self.psdata_opencl))

    def record_read(self, first=None, count=None):
        """The recorded frames [first, first + count) as field -> array of
        shape (count,) + the field's view shape; by default every frame the
        ring holds."""
        total = self.record_count()
        held = min(total, self._rec_frames()) if total else 0
        if first is None:
            first = total - held
        if count is None:
            count = total - first
        fb = int(bnd.sph_record_frame_bytes(self.psdata_opencl))
        buf = np.empty(count * fb, dtype=np.uint8)
        if count and bnd.sph_record_read(self.psdata_opencl, buf.ctypes.data, int(first), int(count)) != 0:
            raise bnd.SphError(bnd.last_error())
        frames = buf.reshape(count, fb)
        out, off = {}, 0
        for name in self._rec:
            view = self.get_fields(name)[0]
            nb = view.nbytes
            out[name] = frames[:, off:off + nb].copy().view(view.dtype).reshape((count,) + view.shape)
            off += nb
        return out

    def _rec_frames(self):
        return self._rec_frames_n

    def init(self, **kwargs):
        self.set_fields(**kwargs)

    def update(self):
        if not self.psdata or not self.psdata_opencl:
            self.setup()

    def free(self):
        self._release_pin()
        free_data(self.psdata, self.psdata_opencl)
        self.fields = {}

    def _release_pin(self):
        # free_data frees the host blob before the device store (the
        # reference's order), so the page-locking ends here, before either
        if getattr(self, "_pinned", False):
            self.unpin()

    def close(self):
        """Frees the store (the reference's free() rebuilds it afterwards)."""
        self._release_pin()
        free_data(self.psdata, self.psdata_opencl)
        self.fields = {}
        self.psdata = self.psdata_opencl = None


class FluidSystem(ParticleSystem):
    """WCSPH fluid: bins, density, pressure/viscosity forces, integration."""
    config = os.path.join(_CONF_DIR, "fluid.conf")

    def setup(self):
        """A fluid keeps no rest state (no original positions or rest
        densities), so there is nothing to set up before update()."""

    def update(self):
        bnd.compute_particle_bins_device_opencl(self.psdata_opencl)
        self.call_for_all_particles("compute_density")
        self.call_for_all_particles("compute_forces_fluids")
        self.call_for_all_particles("step_forward")


class StrainSolid(ParticleSystem):
    """Corotational linear-elastic solid (systems.py:169-219)."""
    config = os.path.join(_CONF_DIR, "strainsolid.conf")
    init_values = None

    def init(self, **kwargs):
        super(StrainSolid, self).init(**kwargs)
        if self.init_values is None:
            self.init_values = {k: np.copy(v) for k, v in kwargs.items()}

    # Pre-sim computation (systems.py:185-192)
    def setup(self):
        self.call_for_all_particles("init_original_position")
        bnd.compute_particle_bins_device_opencl(self.psdata_opencl)
        self.call_for_all_particles("compute_original_density")
        self.sync_device_to_host()

    def update(self):
        bnd.compute_particle_bins_device_opencl(self.psdata_opencl)
        self.call_for_all_particles("compute_density")
        self.call_for_all_particles("compute_rotations_and_strains")
        self.call_for_all_particles("compute_stresses")
        self.call_for_all_particles("compute_forces_solids")
        self.call_for_all_particles("step_forward")

    # Reset to state after init, before setup (systems.py:206-214)
    def reset(self):
        free_data(self.psdata, self.psdata_opencl)
        self.fields = {}
        self.psdata, self.psdata_opencl = self._reinit()
        self.init(**self.init_values)

    def free(self):
        super(StrainSolid, self).free()
        self.init_values = None


class SVKSolid(StrainSolid):
    """St. Venant-Kirchhoff solid (systems.py:221-235)."""
    config = os.path.join(_CONF_DIR, "svksolid.conf")
    init_values = None

    def update(self):
        bnd.compute_particle_bins_device_opencl(self.psdata_opencl)
        self.call_for_all_particles("compute_density")
        self.call_for_all_particles("compute_deformations")
        self.call_for_all_particles("compute_stresses")
        self.call_for_all_particles("compute_forces_solids")
        self.call_for_all_particles("step_forward")
