"""ctypes bindings of libsph_gb300.so (the C ABI declared in include/sph_gb300.h).

Mirrors the reference's generated bindings (scripts/sph/bindings.py): the
same struct names and layouts (``psdata``, ``psdata_opencl``, ``DataPtr``,
the ``T_*`` field types) and the same function names, so code written
against the reference's ``bnd`` module runs unchanged.  The library is
loaded from ``opencl-sph_gb300/lib/`` (or ``$SPH_GB300_LIB``); importing this
module fails loudly when it has not been built -- there is no fallback.

Every wrapped function clears the library's error slot before the call
and raises :class:`SphError` if the call recorded one (the library is put
in record-and-return mode instead of the reference's abort-on-error).
"""
import ctypes
import os
from ctypes import (POINTER, c_ulonglong, Structure, Union, c_char, c_char_p, c_double, c_float, c_int, c_int32,
                    c_size_t, c_uint, c_uint32, c_void_p)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("SPH_GB300_LIB",
                          os.path.join(os.path.dirname(_HERE), "lib", "libsph_gb300.so"))


class SphError(RuntimeError):
    """An error recorded by libsph_gb300 (the reference would have aborted)."""


if not os.path.exists(LIB_PATH):
    raise ImportError("libsph_gb300.so not found at %s; build it with "
                      "`python opencl-sph_gb300/build.py` (or __graft_entry__.build())" % LIB_PATH)

_lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)

# ---- types (src/datatypes.h, src/particle_system.h, particle_system_host.h)

T_CHAR, T_UINT, T_INT, T_FLOAT32, T_FLOAT64, TYPE_COUNT = range(6)
FieldType = c_int


class _DataUnion(Union):
    _fields_ = [("c", c_char_p), ("u", POINTER(c_uint32)), ("i", POINTER(c_int32)),
                ("f4", POINTER(c_float)), ("f8", POINTER(c_double)), ("ptr", c_void_p)]


class DataPtr(Structure):
    _anonymous_ = ("unnamed_1",)
    _fields_ = [("type", FieldType), ("unnamed_1", _DataUnion)]


class psdata(Structure):
    _fields_ = [
        ("num_fields", c_uint),
        ("names", c_char_p),
        ("names_offsets", POINTER(c_uint)),
        ("dimensions", POINTER(c_uint)),
        ("num_dimensions", POINTER(c_uint)),
        ("dimensions_offsets", POINTER(c_uint)),
        ("entry_sizes", POINTER(c_uint)),
        ("data", c_void_p),
        ("data_sizes", POINTER(c_uint)),
        ("data_offsets", POINTER(c_uint)),
        ("data_ptrs", POINTER(DataPtr)),
        ("num_host_fields", c_uint),
        ("host_names", POINTER(POINTER(c_char))),
        ("host_data", POINTER(c_void_p)),
        ("host_data_size", POINTER(c_uint)),
    ]


class psdata_cuda(Structure):
    """Same member layout as the reference's psdata_opencl."""
    _fields_ = [
        ("host_psdata", psdata),
        ("num_fields", c_uint),
        ("names", c_void_p),
        ("names_offsets", c_void_p),
        ("dimensions", c_void_p),
        ("num_dimensions", c_void_p),
        ("dimensions_offsets", c_void_p),
        ("field_types", c_void_p),
        ("entry_sizes", c_void_p),
        ("data", c_void_p),
        ("data_sizes", c_void_p),
        ("data_offsets", c_void_p),
        ("block_totals", c_void_p),
        ("backup_prefix_sum", c_void_p),
        ("num_kernels", c_size_t),
        ("kernel_names", POINTER(POINTER(c_char))),
        ("kernels", c_void_p),
        ("ps_prog", c_void_p),
        ("num_grid_cells", c_uint),
        ("po2_workgroup_size", c_size_t),
        ("num_blocks", c_uint),
    ]


class sph_lattice(Structure):
    """sph_lattice of sph_gb300.h: a lattice scene built on the device."""
    _fields_ = [
        ("nx", c_uint), ("ny", c_uint), ("nz", c_uint),
        ("clamp_layers", c_uint), ("identity_rotation", c_uint),
        ("spacing", c_double), ("jitter", c_double),
        ("origin", c_double * 3),
        ("seed", c_ulonglong),
    ]


psdata_opencl = psdata_cuda
String = c_char_p
_names = POINTER(c_char_p)

# ---- functions ------------------------------------------------------------

_lib.sph_last_error.restype = c_char_p
_lib.sph_last_error.argtypes = []
_lib.sph_clear_error.argtypes = []
_lib.sph_clear_error.restype = None
_lib.sph_set_abort_on_error.argtypes = [c_int]
_lib.sph_set_abort_on_error.restype = None
_lib.sph_set_abort_on_error(0)


def last_error():
    return _lib.sph_last_error().decode("utf-8", "replace")


def _encode(args):
    return [a.encode("utf-8") if isinstance(a, str) else a for a in args]


def _wrap(name, argtypes, restype, checked=True):
    f = getattr(_lib, name)
    f.argtypes = argtypes
    f.restype = restype
    if not checked:
        return f

    def call(*args):
        _lib.sph_clear_error()
        r = f(*_encode(args))
        msg = _lib.sph_last_error()
        if msg:
            raise SphError("%s: %s" % (name, msg.decode("utf-8", "replace")))
        return r

    call.__name__ = name
    call.raw = f
    return call


_SIGS = {
    # store (build_psdata.h, particle_system.h)
    "build_psdata_from_string": ([POINTER(psdata), String], None),
    "build_psdata": ([POINTER(psdata), String], None),
    "display_psdata": ([psdata, POINTER(c_char_p)], None),
    "get_field_psdata": ([psdata, String], c_int),
    "set_field_psdata": ([POINTER(psdata), String, c_void_p, c_uint, c_uint], None),
    "psdata_names_size": ([psdata], c_uint),
    "psdata_dimensions_size": ([psdata], c_uint),
    "psdata_data_size": ([psdata], c_uint),
    "create_host_field_psdata": ([POINTER(psdata), String, c_void_p, c_uint], c_int),
    "get_host_field_psdata": ([POINTER(psdata), String], c_int),
    "free_psdata": ([POINTER(psdata)], None),
    # config / logging
    "load_config": ([String], c_int),
    "get_config_section": ([String], c_char_p),
    "unload_config": ([], None),
    "set_log_level": ([c_uint], None),
    # device driver (particle_system_host.h)
    "init_cuda": ([], None),
    "terminate_cuda": ([], None),
    "create_psdata_cuda": ([POINTER(psdata), String], psdata_cuda),
    "free_psdata_cuda": ([POINTER(psdata_cuda)], None),
    "sync_psdata_device_to_host": ([psdata, psdata_cuda], None),
    "sync_psdata_fields_device_to_host": ([psdata, psdata_cuda, c_size_t, _names], None),
    "sync_psdata_host_to_device": ([psdata, psdata_cuda, c_int], None),
    "sync_psdata_fields_host_to_device": ([psdata, psdata_cuda, c_size_t, _names], None),
    "populate_position_cuboid_device_cuda": ([psdata_cuda] + [c_float] * 6 + [c_uint] * 3, None),
    "rotate_particles_device_cuda": ([psdata_cuda, c_float, c_float, c_float], None),
    "call_for_all_particles_device_cuda": ([psdata_cuda, String], None),
    "compute_particle_bins_device_cuda": ([psdata_cuda], None),
    "compute_density_device_cuda": ([psdata_cuda], None),
    "compute_forces_device_cuda": ([psdata_cuda], None),
    "step_forward_device_cuda": ([psdata_cuda], None),
    "set_body_position_device_cuda": ([psdata_cuda, c_uint, POINTER(c_float)], None),
    "set_body_rotation_device_cuda": ([psdata_cuda, c_uint, POINTER(c_float)], None),
    # reference names
    "init_opencl": ([], None),
    "terminate_opencl": ([], None),
    "create_psdata_opencl": ([POINTER(psdata), String], psdata_cuda),
    "free_psdata_opencl": ([POINTER(psdata_cuda)], None),
    "populate_position_cuboid_device_opencl": ([psdata_cuda] + [c_float] * 6 + [c_uint] * 3, None),
    "rotate_particles_device_opencl": ([psdata_cuda, c_float, c_float, c_float], None),
    "call_for_all_particles_device_opencl": ([psdata_cuda, String], None),
    "compute_particle_bins_device_opencl": ([psdata_cuda], None),
    "compute_density_device_opencl": ([psdata_cuda], None),
    "compute_forces_device_opencl": ([psdata_cuda], None),
    "step_forward_device_opencl": ([psdata_cuda], None),
    "set_body_position_device_opencl": ([psdata_cuda, c_uint, POINTER(c_float)], None),
    "set_body_rotation_device_opencl": ([psdata_cuda, c_uint, POINTER(c_float)], None),
    # additions
    "sph_synchronize": ([psdata_cuda], c_int),
    "sph_pin_host": ([psdata, psdata_cuda], c_int),
    "sph_unpin_host": ([psdata_cuda], c_int),
    "sph_write_fields_async": ([psdata, psdata_cuda, c_size_t, _names], c_int),
    "sph_read_fields_async": ([psdata, psdata_cuda, c_size_t, _names], ctypes.c_longlong),
    "sph_wait_read": ([psdata_cuda, ctypes.c_longlong], c_int),
    "sph_wait_reads": ([psdata_cuda], c_int),
    "sph_update": ([psdata_cuda, c_uint], c_int),
    "sph_record_start": ([psdata_cuda, c_size_t, _names, c_uint, c_uint], c_int),
    "sph_record_stop": ([psdata_cuda], c_int),
    "sph_record_count": ([psdata_cuda], c_ulonglong),
    "sph_record_frame_bytes": ([psdata_cuda], c_size_t),
    "sph_record_read": ([psdata_cuda, c_void_p, c_ulonglong, c_uint], c_int),
    "sph_status": ([psdata_cuda], c_uint),
    "sph_clear_status": ([psdata_cuda], None),
    "sph_version": ([], c_char_p),
    "sph_stream": ([psdata_cuda], c_void_p),
    "sph_graph_kernel_count": ([psdata_cuda], c_uint),
    "sph_profile_substep": ([psdata_cuda, c_uint, POINTER(c_float), POINTER(c_char_p), c_uint], c_int),
    # batched / served forms (opaque sph_batch*)
    "sph_batch_create": ([], c_void_p),
    "sph_batch_free": ([c_void_p], None),
    "sph_scene_bytes": ([POINTER(psdata), String], c_size_t),
    "sph_batch_add": ([c_void_p, POINTER(psdata), String], c_int),
    "sph_batch_remove": ([c_void_p, c_int], c_int),
    "sph_batch_step": ([c_void_p, c_uint], c_int),
    "sph_batch_set_steps": ([c_void_p, c_int, c_uint], c_int),
    "sph_batch_steps_left": ([c_void_p, c_int], c_uint),
    "sph_batch_read": ([c_void_p, c_int, POINTER(psdata)], c_int),
    "sph_batch_synchronize": ([c_void_p], c_int),
    "sph_batch_read_field": ([c_void_p, c_int, String, POINTER(psdata)], c_int),
    "sph_batch_read_field_async": ([c_void_p, c_int, String, POINTER(psdata)], c_int),
    "sph_batch_add_lattice": ([c_void_p, POINTER(psdata), String, POINTER(sph_lattice)], c_int),
    "sph_batch_pin_host": ([c_void_p, c_int, POINTER(psdata)], c_int),
    "sph_batch_unpin_host": ([c_void_p, c_int], c_int),
    "sph_batch_read_field_many": ([c_void_p, POINTER(c_int), c_uint, String, POINTER(POINTER(psdata))], c_int),
    "sph_batch_read_field_many_async": ([c_void_p, POINTER(c_int), c_uint, String, POINTER(POINTER(psdata))],
                                        ctypes.c_longlong),
    "sph_batch_wait_read": ([c_void_p, ctypes.c_longlong], c_int),
    "sph_batch_write_field_many_async": ([c_void_p, POINTER(c_int), c_uint, String, POINTER(POINTER(psdata))],
                                         c_int),
    "sph_batch_write_fields_many_async": ([c_void_p, POINTER(c_int), c_uint, c_uint, POINTER(c_char_p),
                                           POINTER(POINTER(psdata))], c_int),
    "sph_batch_wait_reads": ([c_void_p], c_int),
    "sph_batch_profile": ([c_void_p, c_uint, POINTER(c_float), POINTER(c_char_p), c_uint], c_int),
    "sph_batch_bytes": ([c_void_p], c_size_t),
    "sph_batch_size": ([c_void_p], c_uint),
    "sph_batch_tune": ([c_void_p, c_uint, c_uint, c_uint], c_int),
    "sph_batch_kernel_count": ([c_void_p], c_uint),
    "sph_batch_stream": ([c_void_p], c_void_p),
    "sph_batch_status": ([c_void_p, c_int], c_uint),
}

for _n, (_a, _r) in _SIGS.items():
    globals()[_n] = _wrap(_n, _a, _r)

library = _lib


# ---- helpers over a psdata struct ----------------------------------------

_NP = {T_UINT: "u4", T_INT: "i4", T_FLOAT32: "f4", T_FLOAT64: "f8", T_CHAR: "S1"}


def field_names(ps):
    """Names of the store's fields, in storage order."""
    base = c_void_p.from_buffer(ps, psdata.names.offset).value
    return [ctypes.string_at(base + ps.names_offsets[f]).decode() for f in range(ps.num_fields)]


def field_view(ps, f):
    """Zero-copy NumPy view of field index f, dimensions reversed (a
    `3, pnum` field is (pnum, 3))."""
    import numpy as np
    nd = ps.num_dimensions[f]
    off = ps.dimensions_offsets[f]
    dims = [ps.dimensions[off + d] for d in range(nd)]
    dtype = np.dtype(_NP[ps.data_ptrs[f].type])
    count = 1
    for d in dims:
        count *= d
    buf = (ctypes.c_char * (count * dtype.itemsize)).from_address(ps.data + ps.data_offsets[f])
    return np.frombuffer(buf, dtype=dtype, count=count).reshape(tuple(reversed(dims)))


def store_views(ps):
    """name -> view for every field of the store."""
    return {name: field_view(ps, f) for f, name in enumerate(field_names(ps))}
