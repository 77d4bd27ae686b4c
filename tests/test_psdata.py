"""Host store (no GPU): the product's psdata builder against the layouts
the reference's own builder produced (tests/golden/layouts.json, made by
tests/golden/make_golden.py), the config reader, field access and errors."""
import ctypes
import json
import os

import numpy as np
import pytest

from sph import bindings as bnd
from sph import init_data_cpu, free_data_cpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "layouts.json")
CONF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "opencl-sph_gb300", "conf")

with open(GOLDEN) as _f:
    LAYOUTS = json.load(_f)


def layout_of(ps):
    nf = ps.num_fields
    names = bnd.field_names(ps)
    dims = []
    for f in range(nf):
        o = ps.dimensions_offsets[f]
        dims.append([ps.dimensions[o + d] for d in range(ps.num_dimensions[f])])
    return {"names": names, "entry_sizes": [ps.entry_sizes[f] for f in range(nf)],
            "data_sizes": [ps.data_sizes[f] for f in range(nf)],
            "data_offsets": [ps.data_offsets[f] for f in range(nf)], "dims": dims}


@pytest.mark.parametrize("name", sorted(LAYOUTS))
def test_layout_matches_reference_builder(name):
    g = LAYOUTS[name]
    ps = init_data_cpu(g["spec"])
    got = layout_of(ps)
    for k in ("names", "entry_sizes", "data_sizes", "data_offsets", "dims"):
        assert got[k] == g["layout"][k], k
    assert bnd.psdata_data_size(ps) == g["layout"]["size"]
    if g["layout"]["gridres"] is not None:
        assert list(bnd.store_views(ps)["gridres"]) == g["layout"]["gridres"]
    free_data_cpu(ps)


def test_default_values_and_types():
    ps = init_data_cpu(LAYOUTS["mixed-types"]["spec"])
    v = bnd.store_views(ps)
    assert v["pnum"][0] == 16                      # strtol base 0: 0x10
    assert v["smoothingradius"].dtype == np.float32 and v["smoothingradius"][0] == np.float32(0.25)
    assert np.all(v["k"][:1] == -3)                 # one value given, the rest zero
    assert np.all(v["u"] == 0)                      # "uint" spelling takes no default values
    assert list(v["gridres"]) == [8, 16, 2]
    free_data_cpu(ps)


def test_dimension_by_name_and_missing_name():
    ps = init_data_cpu(LAYOUTS["dims-by-name"]["spec"])
    v = bnd.store_views(ps)
    assert v["bp"].shape == (3, 3)
    assert list(v["bd"]) == [1, 0, 1]
    assert v["missing"].shape == (0, 2)
    free_data_cpu(ps)


def test_field_access_and_set_field():
    ps = init_data_cpu(LAYOUTS["scene/wcsph"]["spec"])
    f = bnd.get_field_psdata(ps, "position")
    assert f >= 0 and bnd.get_field_psdata(ps, "nonexistent") == -1
    vals = np.arange(6, dtype=np.float32)
    bnd.set_field_psdata(ctypes.byref(ps), "position", vals.ctypes.data, vals.nbytes, 12)
    pos = bnd.store_views(ps)["position"]
    assert np.array_equal(pos[1:3].ravel(), vals)
    assert bnd.psdata_names_size(ps) == sum(len(n) + 1 for n in bnd.field_names(ps))
    free_data_cpu(ps)


def test_config_sections_and_missing_file():
    assert bnd.load_config(os.path.join(CONF, "fluid.conf")) == 0
    spec = bnd.get_config_section("psdata_specification")
    files = bnd.get_config_section("opencl_kernel_files")
    assert b"pnum" in spec and files.strip() == b"common, fluids"
    assert bnd.get_config_section("no_such_section") is None
    bnd.unload_config()
    assert bnd.load_config("/nonexistent/file.conf") == 1


def test_build_psdata_from_file(tmp_path):
    ps = bnd.psdata()
    # a spec file whose last byte is overwritten by the terminator, as the
    # reference's build_psdata does
    path = str(tmp_path / "spec.txt")
    with open(path, "w") as f:
        f.write(LAYOUTS["fp32-grid-truncation"]["spec"] + "\n")
    bnd.build_psdata(ctypes.byref(ps), path)
    assert list(bnd.store_views(ps)["gridres"]) == [39, 39, 39]  # 4 / (double)0.1f truncates to 39
    bnd.free_psdata(ctypes.byref(ps))


def test_missing_grid_fields_is_an_error():
    with pytest.raises(bnd.SphError):
        init_data_cpu("pnum | 1 | unsigned int | 4\nposition | 3, pnum | float\n")


def test_host_fields():
    ps = init_data_cpu(LAYOUTS["scene/wcsph"]["spec"])
    buf = ctypes.cast(ctypes.create_string_buffer(8), ctypes.c_void_p)
    # ownership passes to the store (freed by free_psdata): use malloc'd memory
    libc = ctypes.CDLL(None)
    libc.malloc.restype = ctypes.c_void_p
    libc.malloc.argtypes = [ctypes.c_size_t]
    mem = libc.malloc(16)
    i = bnd.create_host_field_psdata(ctypes.byref(ps), "extra", mem, 16)
    assert i == 0 and bnd.get_host_field_psdata(ctypes.byref(ps), "extra") == 0
    assert bnd.get_host_field_psdata(ctypes.byref(ps), "other") == -1
    del buf
    free_data_cpu(ps)


def test_init_data_from_dict(monkeypatch):
    import sph
    spec = LAYOUTS["scene/wcsph"]["spec"]
    seen = []
    # the device store needs a GPU: record the kernel-file section instead
    monkeypatch.setattr(sph, "init_data_opencl", lambda ps, files: seen.append(files) or "device")
    for form in (spec, spec.splitlines()):
        ps, dev = sph.init_data_from_dict({"psdata_specification": form, "opencl_kernel_files": "common, fluids"})
        assert dev == "device" and seen[-1] == "common, fluids"
        ref = init_data_cpu(spec)
        assert layout_of(ps) == layout_of(ref)
        free_data_cpu(ps)
        free_data_cpu(ref)
    with pytest.raises(KeyError):
        sph.init_data_from_dict({"psdata_specification": spec})
