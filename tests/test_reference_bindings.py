"""The reference's own Python layer against libsph_gb300.so, unmodified.

The reference's ctypesgen bindings (scripts/sph/bindings.py) load
``libSPH`` through their own loader, which searches LD_LIBRARY_PATH among
other places (bindings.py:454-529, 603-608).  Here a directory holding
``libSPH.so`` -> libsph_gb300.so is put on that path, and the reference's
package (scripts/sph/__init__.py, bindings.py, systems.py) is imported from
the reference checkout as it is.  On the CPU it then builds, queries and
frees host stores through the reference's own functions, and the
reference's ParticleSystem.get_fields (systems.py:33-60, the data_ptrs
union views) reads the fields this library laid out.  Device stores need a
GPU; the device recipes run through the mirror package in the -m gpu
tests (the reference checkout is not available where those run).

Skipped where the reference checkout is absent.
"""
import ctypes
import importlib.util
import os
import sys

import numpy as np
import pytest

from sph import bindings as own

REF = os.environ.get("SPH_REFERENCE_ROOT", "/root/reference")
REF_PKG = os.path.join(REF, "scripts", "sph")

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF_PKG, "bindings.py")),
                                reason="reference checkout not available")


@pytest.fixture(scope="module")
def refsph(tmp_path_factory):
    d = tmp_path_factory.mktemp("libdir")
    os.symlink(own.LIB_PATH, str(d / "libSPH.so"))
    old = os.environ.get("LD_LIBRARY_PATH")
    os.environ["LD_LIBRARY_PATH"] = str(d) + ((":" + old) if old else "")
    try:
        spec = importlib.util.spec_from_file_location("refsph", os.path.join(REF_PKG, "__init__.py"),
                                                      submodule_search_locations=[REF_PKG])
        mod = importlib.util.module_from_spec(spec)
        sys.modules["refsph"] = mod
        spec.loader.exec_module(mod)
        systems = importlib.import_module("refsph.systems")
    finally:
        if old is None:
            del os.environ["LD_LIBRARY_PATH"]
        else:
            os.environ["LD_LIBRARY_PATH"] = old
    yield mod, systems
    for k in [k for k in sys.modules if k == "refsph" or k.startswith("refsph.")]:
        del sys.modules[k]


def test_reference_bindings_load_this_library(refsph):
    mod, _ = refsph
    bnd = mod.bindings
    # the library the reference's loader found is this one (same exports)
    assert hasattr(bnd._libs["SPH"], "sph_update") and hasattr(bnd._libs["SPH"], "create_psdata_opencl")
    # the structs the reference's bindings declare have this library's sizes
    assert ctypes.sizeof(bnd.psdata) == ctypes.sizeof(own.psdata)
    assert ctypes.sizeof(bnd.psdata_opencl) == ctypes.sizeof(own.psdata_opencl)


def test_reference_python_builds_queries_and_frees_stores(refsph):
    mod, systems = refsph
    bnd = mod.bindings
    conf = os.path.join(REF, "conf", "strainsolid.conf")
    assert bnd.load_config(conf) == 0
    spec = bnd.get_config_section("psdata_specification")
    files = bnd.get_config_section("opencl_kernel_files")
    assert "solid_corotation" in str(files)
    ps = mod.init_data_cpu(spec)
    bnd.unload_config()
    assert bnd.get_field_psdata(ps, "position") >= 0 and bnd.get_field_psdata(ps, "no_such_field") == -1
    assert bnd.psdata_data_size(ps) > 0
    # the reference's own field views (systems.py:33-60) over this library's store
    view = systems.ParticleSystem.__new__(systems.ParticleSystem)
    view.psdata, view.fields = ps, {}
    pos, rot, pnum, res = view.get_fields("position", "rotation", "pnum", "gridres")
    assert pos.shape == (4096, 3) and rot.shape == (4096, 3, 3) and int(pnum[0]) == 4096
    # gridbounds [-1, 1]^3 over h = 0.2: 2 / (double)0.2f truncates to 9 (build_psdata.c:92-98)
    assert [int(x) for x in res] == [9, 9, 9]
    pos[:] = np.arange(3 * 4096, dtype=np.float32).reshape(4096, 3)
    # the same bytes through this library's own views
    assert np.array_equal(own.store_views(ps)["position"], pos)
    # set_field_psdata through the reference's binding
    vals = (ctypes.c_float * 3)(1.5, 2.5, 3.5)
    bnd.set_field_psdata(ctypes.byref(ps), "gravity", vals, 12, 0)
    assert list(view.get_fields("gravity")[0]) == [1.5, 2.5, 3.5]
    mod.free_data_cpu(ps)
