"""The store builder against the reference's own builder on seeded random
specifications (CPU).

Each specification is drawn from the grammar that src/build_psdata.c parses
(create_psdata_field_spec, build_psdata.c:183-313): a line per field,
`name | dims | type | defaults`, dimensions given as numbers (strtol base
0: decimal, hex, octal) or as the name of an earlier unsigned scalar,
every type spelling of src/stringly.c (char, unsigned int / uint, int,
float / float32, double / float64), default values in the spellings
strtol/strtof/strtod accept, comment and blank lines, and irregular
spacing.  Both builders make the store; names, dimensions, entry sizes,
data sizes, offsets (including the first field's wrapped alignment,
build_psdata.c:381), field types, the grid arrays and every byte of the
data blob must agree, and so must the store's queries and writes
(src/particle_system.c:84-112: get_field_psdata, set_field_psdata,
psdata_names_size, psdata_dimensions_size, psdata_data_size).

Specifications stay inside what the reference defines: the three grid
fields are present with one float type (build_psdata.c:43-84 dereferences
and asserts them), a named dimension refers to a scalar that has a value
(get_value reads its data), a multi-dimensional field's first dimension is
not zero (its alignment divides by it), and default values either cover
the whole field or are absent (a partial list makes the reference copy
past its buffer).

Runs where oracle/_ref/libref_psdata.so was built from the reference's
sources; skipped elsewhere.
"""
import ctypes

import numpy as np
import pytest

from oracle import ref
from sph import bindings as bnd

pytestmark = pytest.mark.skipif(not ref.available("psdata"), reason="reference builder not built")

SIZES = {"char": 1, "unsigned int": 4, "uint": 4, "int": 4, "float": 4, "float32": 4, "double": 8, "float64": 8}
PARSED = {"unsigned int", "int", "float", "double"}  # types whose default values the reference reads
N_SPECS = 2000


def _int_text(rng, v):
    form = rng.integers(4)
    if form == 0 and v >= 0:
        return hex(v)
    if form == 1 and 0 <= v < 4096:
        return "0" + oct(v)[2:] if v else "0"
    return str(v)


def _value_text(rng, t):
    if t in ("float", "double"):
        x = float(rng.standard_normal() * 10.0 ** int(rng.integers(-8, 9)))
        form = rng.integers(5)
        if form == 0:
            return repr(x)
        if form == 1:
            return "%.4e" % x
        if form == 2:
            return str(int(rng.integers(-300, 300)))
        if form == 3:
            return "0x1.8p%d" % int(rng.integers(-20, 20))
        return "%.9g" % x
    if t == "int":
        return _int_text(rng, int(rng.integers(-2 ** 31, 2 ** 31)))
    # unsigned int: strtol, then the conversion to unsigned
    v = int(rng.integers(-50, 2 ** 32)) if rng.integers(4) else int(rng.integers(-50, 50))
    return _int_text(rng, v)


def _type_text(rng, t):
    if t == "unsigned int" and rng.integers(3) == 0:
        return "unsigned   int"
    return t


def _line(rng, parts):
    sep = [" | ", "|", " |  ", "  | "][int(rng.integers(4))]
    return sep.join(parts)


def random_spec(rng):
    """One specification: pnum first, then the other fields in drawn order
    with smoothingradius and gridbounds placed among them."""
    real = "double" if rng.integers(3) == 0 else "float"
    pnum = int(rng.integers(1, 65))
    h = float(np.float32(rng.uniform(0.02, 0.5)))
    lo = [float(np.float32(rng.uniform(-2.0, 0.0))) for _ in range(3)]
    hi = [float(np.float32(lo[d] + h * rng.uniform(1.5, 30.0))) for d in range(3)]
    bounds = ", ".join("%r, %r" % (lo[d], hi[d]) for d in range(3))
    lines = [_line(rng, ["pnum", "1", _type_text(rng, "unsigned int"), _int_text(rng, pnum)])]
    scalars = {"pnum": pnum}  # unsigned scalars with values: usable as dimensions by name
    for f in range(int(rng.integers(0, 10))):
        name = "f%d_%d" % (f, int(rng.integers(1000)))
        if rng.integers(4) == 0:
            v = int(rng.integers(0, 7))
            scalars[name] = v
            lines.append(_line(rng, [name, "1", "unsigned int", str(v)]))
            continue
        t = list(SIZES)[int(rng.integers(len(SIZES)))]
        ndim = int(rng.integers(1, 5))
        dims, words = [], []
        for d in range(ndim):
            choice = rng.integers(5)
            # a multi-dimensional field's first dimension may not be zero
            may_be_zero = d > 0 or ndim == 1
            known = [k for k in scalars if may_be_zero or scalars[k] > 0]
            if choice == 0 and known:
                k = known[int(rng.integers(len(known)))]
                dims.append(scalars[k])
                words.append(k)
            elif choice == 1 and may_be_zero:
                dims.append(0)  # a name no earlier field has: dimension 0
                words.append("nosuch%d" % f)
            else:
                v = int(rng.integers(1, 7))
                dims.append(v)
                words.append(_int_text(rng, v))
        entries = int(np.prod(dims))
        parts = [name, (", " if rng.integers(2) else ",").join(words), _type_text(rng, t)]
        if t in PARSED and entries * SIZES[t] <= 256 and rng.integers(3):
            room = 256 // SIZES[t] - entries  # values past the field's end are read and dropped
            n_vals = entries + int(rng.integers(0, room // 4 + 1))
            parts.append(", ".join(_value_text(rng, t) for _ in range(n_vals)))
        elif t not in PARSED and rng.integers(2):
            parts.append("1, 2, 3")  # the reference reads no defaults for this spelling
        lines.append(_line(rng, parts))
    for g in (_line(rng, ["smoothingradius", "1", real, repr(h)]),
              _line(rng, ["gridbounds", "2, 3" if rng.integers(2) else "2,3", real, bounds])):
        lines.insert(int(rng.integers(1, len(lines) + 1)), g)
    out = []
    for ln in lines:
        if rng.integers(8) == 0:
            out.append("# a comment | 3 | float")
        if rng.integers(8) == 0:
            out.append("")
        out.append(ln)
    return "\n".join(out) + ("\n" if rng.integers(2) else "")


def _layout(ps):
    nf = ps.num_fields
    dims = []
    for f in range(nf):
        o = ps.dimensions_offsets[f]
        dims.append([ps.dimensions[o + d] for d in range(ps.num_dimensions[f])])
    return {"entry_sizes": [ps.entry_sizes[f] for f in range(nf)],
            "data_sizes": [ps.data_sizes[f] for f in range(nf)],
            "data_offsets": [ps.data_offsets[f] for f in range(nf)], "dims": dims}


def _types(data_ptrs, n, stride):
    base = ctypes.cast(data_ptrs, ctypes.c_void_p).value
    return [ctypes.c_int.from_address(base + f * stride).value for f in range(n)]


def _blob(ptr, size):
    return ctypes.string_at(ptr, size) if size else b""


def reference_store_functions():
    lib = ref.psdata_lib()
    for fn in ("psdata_names_size", "psdata_dimensions_size"):
        getattr(lib, fn).argtypes = [ref.psdata]
        getattr(lib, fn).restype = ctypes.c_uint
    lib.get_field_psdata.argtypes = [ref.psdata, ctypes.c_char_p]
    lib.get_field_psdata.restype = ctypes.c_int
    lib.set_field_psdata.argtypes = [ctypes.POINTER(ref.psdata), ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint,
                                     ctypes.c_uint]
    lib.set_field_psdata.restype = None
    return lib


@pytest.mark.parametrize("block", range(4))
def test_builder_equals_reference_builder_on_random_specs(block):
    rng = np.random.default_rng(1000 + block)
    stride = ctypes.sizeof(bnd.DataPtr)
    lib = reference_store_functions()
    for case in range(N_SPECS // 4):
        spec = random_spec(rng)
        rs = ref.RefStore(spec)
        ps = bnd.psdata()
        bnd.build_psdata_from_string(ctypes.byref(ps), spec.encode())
        try:
            assert bnd.field_names(ps) == rs.layout["names"], spec
            got = _layout(ps)
            for k in ("entry_sizes", "data_sizes", "data_offsets", "dims"):
                assert got[k] == rs.layout[k], (k, spec)
            n = ps.num_fields
            assert _types(ps.data_ptrs, n, stride) == _types(rs.ps.data_ptrs, n, stride), spec
            assert bnd.psdata_data_size(ps) == rs.size, spec
            assert _blob(ps.data, rs.size) == _blob(rs.ps.data, rs.size), spec
            for fn in ("psdata_names_size", "psdata_dimensions_size"):
                assert getattr(bnd, fn)(ps) == getattr(lib, fn)(rs.ps), (fn, spec)
            names = rs.layout["names"]
            for name in names + ["nosuch", "", names[0] + "x"]:
                assert bnd.get_field_psdata(ps, name) == lib.get_field_psdata(rs.ps, name.encode()), (name, spec)
            # set_field_psdata: bytes at an offset inside a field (the
            # reference checks only the name)
            for _ in range(4):
                f = int(rng.integers(len(names)))
                ds = rs.layout["data_sizes"][f]
                if ds == 0:
                    continue
                off = int(rng.integers(ds))
                size = int(rng.integers(1, ds - off + 1))
                src = ctypes.create_string_buffer(bytes(rng.integers(0, 256, size, dtype=np.uint8)), size)
                bnd.set_field_psdata(ctypes.byref(ps), names[f], ctypes.addressof(src), size, off)
                lib.set_field_psdata(ctypes.byref(rs.ps), names[f].encode(), ctypes.addressof(src), size, off)
            bnd.set_field_psdata(ctypes.byref(ps), "nosuch", ctypes.addressof(src), 1, 0)
            lib.set_field_psdata(ctypes.byref(rs.ps), b"nosuch", ctypes.addressof(src), 1, 0)
            assert _blob(ps.data, rs.size) == _blob(rs.ps.data, rs.size), spec
        finally:
            bnd.free_psdata(ctypes.byref(ps))
            rs.free()


def _printed(call):
    """What `call` writes to the process's standard output (C stdio)."""
    import os
    import sys
    import tempfile
    libc = ctypes.CDLL(None)
    sys.stdout.flush()
    libc.fflush(None)
    with tempfile.TemporaryFile() as tmp:
        saved = os.dup(1)
        os.dup2(tmp.fileno(), 1)
        try:
            call()
            libc.fflush(None)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        tmp.seek(0)
        return tmp.read()


def test_display_psdata_prints_what_the_reference_prints():
    """display_psdata (particle_system.c:38-82): the same text for every
    field of seeded random stores (8-byte entries as %g, 4-byte ones as
    their bits with %u, 1-byte ones not at all; fields of more than three
    dimensions print their name only)."""
    lib = ref.psdata_lib()
    lib.display_psdata.argtypes = [ref.psdata, ctypes.c_void_p]
    lib.display_psdata.restype = None
    rng = np.random.default_rng(77)
    for case in range(100):
        spec = random_spec(rng)
        rs = ref.RefStore(spec)
        ps = bnd.psdata()
        bnd.build_psdata_from_string(ctypes.byref(ps), spec.encode())
        try:
            want = _printed(lambda: lib.display_psdata(rs.ps, None))
            got = _printed(lambda: bnd.display_psdata(ps, None))
            assert want and got == want, spec
        finally:
            bnd.free_psdata(ctypes.byref(ps))
            rs.free()


def test_specifications_the_reference_cannot_build_are_errors():
    """Where the reference's builder divides by zero (a multi-dimensional
    field whose first dimension is 0, e.g. gridcount of a grid narrower
    than one cell along x: its alignment divides by it), this builder
    reports an error instead."""
    spec = ("pnum | 1 | unsigned int | 4\nsmoothingradius | 1 | float | 0.5\n"
            "gridbounds | 2, 3 | float | 0, 0.2, 0, 1, 0, 1\nposition | 3, pnum | float\n")
    ps = bnd.psdata()
    with pytest.raises(bnd.SphError):
        bnd.build_psdata_from_string(ctypes.byref(ps), spec)
    # a multi-dimensional field whose first dimension names no field (0)
    spec = ("pnum | 1 | unsigned int | 4\nsmoothingradius | 1 | float | 0.1\n"
            "gridbounds | 2, 3 | float | 0, 1, 0, 1, 0, 1\nx | nosuch, pnum | float\n")
    with pytest.raises(bnd.SphError):
        bnd.build_psdata_from_string(ctypes.byref(ps), spec)


def test_host_fields_equal_the_reference():
    """create_host_field_psdata / get_host_field_psdata
    (particle_system.c:116-164) on seeded random sequences of names
    (repeats included) and sizes: the same indices, names and sizes."""
    lib = ref.psdata_lib()
    lib.create_host_field_psdata.argtypes = [ctypes.POINTER(ref.psdata), ctypes.c_char_p, ctypes.c_void_p,
                                             ctypes.c_uint]
    lib.create_host_field_psdata.restype = ctypes.c_int
    lib.get_host_field_psdata.argtypes = [ctypes.POINTER(ref.psdata), ctypes.c_char_p]
    lib.get_host_field_psdata.restype = ctypes.c_int
    libc = ctypes.CDLL(None)
    libc.malloc.restype = ctypes.c_void_p
    libc.malloc.argtypes = [ctypes.c_size_t]
    rng = np.random.default_rng(88)
    for case in range(20):
        spec = random_spec(rng)
        rs = ref.RefStore(spec)
        ps = bnd.psdata()
        bnd.build_psdata_from_string(ctypes.byref(ps), spec)
        try:
            pool = ["h%d" % k for k in range(5)] + ["position_mex", ""]
            for _ in range(int(rng.integers(1, 12))):
                name = pool[int(rng.integers(len(pool)))]
                size = int(rng.integers(0, 64))
                # both stores own (and free) their buffers
                a = lib.create_host_field_psdata(ctypes.byref(rs.ps), name.encode(), libc.malloc(max(size, 1)), size)
                b = bnd.create_host_field_psdata(ctypes.byref(ps), name, libc.malloc(max(size, 1)), size)
                assert a == b, (case, name)
                for q in pool + ["nosuch"]:
                    assert (bnd.get_host_field_psdata(ctypes.byref(ps), q)
                            == lib.get_host_field_psdata(ctypes.byref(rs.ps), q.encode())), (case, q)
            assert ps.num_host_fields == rs.ps.num_host_fields
            sizes = ctypes.cast(rs.ps.host_data_size, ctypes.POINTER(ctypes.c_uint))
            assert [ps.host_data_size[i] for i in range(ps.num_host_fields)] == \
                [sizes[i] for i in range(rs.ps.num_host_fields)]
        finally:
            bnd.free_psdata(ctypes.byref(ps))
            rs.free()
