"""The reference's own CPU code, compiled by make_ref.py into oracle/_ref/.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).  Two libraries:

* libref_psdata.so -- the reference's host store builder
  (src/build_psdata.c & co.), used to pin the product's builder layout;
* libref_kernels.so -- the reference's kernels/*.cl compiled as C++ (one
  program per material and precision), used to pin the C restatement and
  as the timed reference CPU baseline.

Both exist only where make_ref.py could run; :func:`available` says so.
"""
import ctypes
import os
from ctypes import POINTER, Structure, c_char_p, c_double, c_float, c_int, c_uint, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
KERNELS_LIB = os.path.join(REF_DIR, "libref_kernels.so")
PSDATA_LIB = os.path.join(REF_DIR, "libref_psdata.so")

PROGRAM_OF = {"fluid": "fluid", "corot": "corot", "svk": "svk"}


class psdata(Structure):
    """src/particle_system.h:18-48"""
    _fields_ = [("num_fields", c_uint), ("names", c_void_p), ("names_offsets", POINTER(c_uint)),
                ("dimensions", POINTER(c_uint)), ("num_dimensions", POINTER(c_uint)),
                ("dimensions_offsets", POINTER(c_uint)), ("entry_sizes", POINTER(c_uint)),
                ("data", c_void_p), ("data_sizes", POINTER(c_uint)), ("data_offsets", POINTER(c_uint)),
                ("data_ptrs", c_void_p), ("num_host_fields", c_uint), ("host_names", c_void_p),
                ("host_data", c_void_p), ("host_data_size", POINTER(c_uint))]


def available(what="kernels"):
    return os.path.exists(KERNELS_LIB if what == "kernels" else PSDATA_LIB)


_klib = None
_plib = None


def kernels_lib():
    global _klib
    if _klib is None:
        _klib = ctypes.CDLL(KERNELS_LIB)
    return _klib


def psdata_lib():
    global _plib
    if _plib is None:
        _plib = ctypes.CDLL(PSDATA_LIB)
        _plib.build_psdata_from_string.argtypes = [POINTER(psdata), c_char_p]
        _plib.build_psdata_from_string.restype = None
        _plib.free_psdata.argtypes = [POINTER(psdata)]
        _plib.free_psdata.restype = None
        _plib.set_log_level.argtypes = [c_uint]
        _plib.set_log_level(5)
    return _plib


_prod = None


def product_builder_lib():
    """The product's library under a ctypes handle of its own, typed for the
    psdata struct above: configuring it leaves the product's bindings (which
    load the same library through another handle) untouched."""
    global _prod
    if _prod is None:
        from sph import bindings as bnd
        _prod = ctypes.CDLL(bnd.LIB_PATH)
        _prod.build_psdata_from_string.argtypes = [POINTER(psdata), c_char_p]
        _prod.build_psdata_from_string.restype = None
        _prod.free_psdata.argtypes = [POINTER(psdata)]
        _prod.free_psdata.restype = None
    return _prod


def layout(ps):
    """(names, entry_sizes, data_sizes, data_offsets, dims) of a psdata."""
    nf = ps.num_fields
    names = [ctypes.string_at(ps.names + ps.names_offsets[f]).decode() for f in range(nf)]
    dims = []
    for f in range(nf):
        o = ps.dimensions_offsets[f]
        dims.append([ps.dimensions[o + d] for d in range(ps.num_dimensions[f])])
    return {
        "names": names,
        "entry_sizes": [ps.entry_sizes[f] for f in range(nf)],
        "data_sizes": [ps.data_sizes[f] for f in range(nf)],
        "data_offsets": [ps.data_offsets[f] for f in range(nf)],
        "dims": dims,
    }


class RefStore(object):
    """A store built by the reference's own builder, with NumPy views.

    Where libref_psdata.so was not built (a machine without the reference
    checkout), the product's builder makes the store instead; its layout is
    pinned to the reference builder's by tests/test_psdata.py."""

    def __init__(self, spec):
        self.ps = psdata()
        self._own = available("psdata")
        if self._own:
            psdata_lib().build_psdata_from_string(ctypes.byref(self.ps), spec.encode())
        else:
            product_builder_lib().build_psdata_from_string(ctypes.byref(self.ps), spec.encode())
        self.layout = layout(self.ps)
        self.size = self.layout["data_offsets"][-1] + self.layout["data_sizes"][-1]

    def view(self, name):
        L = self.layout
        f = L["names"].index(name)
        es = L["entry_sizes"][f]
        text = {4: np.float32, 8: np.float64}
        dtype = np.dtype(text[es]) if name not in _UINTS else np.dtype(np.uint32)
        count = L["data_sizes"][f] // es
        buf = (ctypes.c_char * L["data_sizes"][f]).from_address(self.ps.data + L["data_offsets"][f])
        return np.frombuffer(buf, dtype=dtype, count=count).reshape(tuple(reversed(L["dims"][f])))

    def call(self, program, prec, kernel, global_size, nthreads=1, body=0, vec=None):
        fn = getattr(kernels_lib(), "ref_%s_%s_call" % (program, prec))
        real = c_float if prec == "f32" else c_double
        fn.restype = c_int
        v = (real * 3)(*(vec if vec is not None else (0, 0, 0)))
        ps = self.ps
        rc = fn(kernel.encode(), c_uint(global_size), c_int(nthreads), ps.num_fields, ps.names, ps.names_offsets,
                ps.dimensions, ps.num_dimensions, ps.dimensions_offsets, ps.entry_sizes, c_void_p(ps.data),
                ps.data_sizes, ps.data_offsets, c_uint(body), v)
        if rc != 0:
            raise RuntimeError("reference kernel %s/%s returned %d" % (program, kernel, rc))

    def _pso(self):
        ps = self.ps
        return (ps.num_fields, ps.names, ps.names_offsets, ps.dimensions, ps.num_dimensions, ps.dimensions_offsets,
                ps.entry_sizes, c_void_p(ps.data), ps.data_sizes, ps.data_offsets)

    def populate_cuboid(self, program, prec, corner1, corner2, size):
        """populate_position_cuboid (common.cl:533-555) over its 3-D range."""
        fn = getattr(kernels_lib(), "ref_%s_%s_populate_cuboid" % (program, prec))
        real = c_float if prec == "f32" else c_double
        fn.restype = c_int
        rc = fn(*self._pso(), (real * 3)(*corner1), (real * 3)(*corner2), (c_uint * 3)(*size))
        if rc != 0:
            raise RuntimeError("reference populate_position_cuboid returned %d" % rc)

    def rotate(self, program, prec, angles, global_size):
        """rotate_particles (common.cl:556-604) over `global_size` items."""
        fn = getattr(kernels_lib(), "ref_%s_%s_rotate" % (program, prec))
        real = c_float if prec == "f32" else c_double
        fn.restype = c_int
        rc = fn(*self._pso(), c_uint(global_size), real(angles[0]), real(angles[1]), real(angles[2]))
        if rc != 0:
            raise RuntimeError("reference rotate_particles returned %d" % rc)

    def free(self):
        if self.ps.num_fields:
            if self._own:
                psdata_lib().free_psdata(ctypes.byref(self.ps))
            else:
                product_builder_lib().free_psdata(ctypes.byref(self.ps))
            self.ps.num_fields = 0


# fields whose type is unsigned int in every conf
_UINTS = {"pnum", "n", "gridres", "gridcell", "gridcount", "celloffset", "cellparticles", "num_neighbours",
          "body_number", "body_count", "body_dynamic", "plane_constraints_particles", "padding", "rigid_mask"}
