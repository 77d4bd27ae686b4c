"""The C-ABI library (no GPU): it loads, exports every function that
include/sph_gb300.h declares, and its struct layouts match the
reference's (psdata, psdata_opencl) so the reference's ctypes bindings can
bind it; the header compiles as C11 and C++, and a C program linked
against the library reads a conf and builds a store."""
import ctypes
import os
import re
import subprocess

from sph import bindings as bnd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        text = re.sub(r"//[^\n]*", " ", text)
        text = re.sub(r"^\s*#[^\n]*", " ", text, flags=re.M)
        text = re.sub(r"typedef\s+struct\s*\{.*?\}\s*\w+\s*;", " ", text, flags=re.S)
        text = re.sub(r"typedef[^;]*;", " ", text)
        for m in re.finditer(r"([A-Za-z_]\w*)\s*\(([^;{}]*)\)\s*;", text):
            names.append(m.group(1))
    return names


def exported():
    out = subprocess.run(["nm", "-D", "--defined-only", bnd.LIB_PATH], capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if " T " in line}


def test_every_declared_function_is_exported():
    decl = declared_functions()
    assert len(decl) > 40
    syms = exported()
    missing = [d for d in decl if d not in syms]
    assert not missing, missing


def test_opencl_aliases_present():
    syms = exported()
    for base in ["init_%s", "terminate_%s", "create_psdata_%s", "free_psdata_%s",
                 "call_for_all_particles_device_%s", "compute_particle_bins_device_%s",
                 "set_body_position_device_%s", "set_body_rotation_device_%s"]:
        assert base % "opencl" in syms and base % "cuda" in syms


def test_struct_layouts_match_the_reference():
    # psdata: 15 members (particle_system.h:18-48); psdata_opencl: 21
    # members (particle_system_host.h:7-47), pointer-sized cl_* slots
    # num_fields (+pad), 10 pointers, num_host_fields (+pad), 3 pointers
    assert ctypes.sizeof(bnd.psdata) == 8 + 8 * 10 + 8 + 8 * 3
    assert [f[0] for f in bnd.psdata_opencl._fields_][:2] == ["host_psdata", "num_fields"]
    assert bnd.psdata_opencl.ps_prog.offset == bnd.psdata_opencl.kernels.offset + 8
    assert len(bnd.psdata_opencl._fields_) == 21


def test_errors_are_recorded_not_aborted():
    """A failing call records a message instead of aborting the process."""
    pso = bnd.psdata_cuda()
    try:
        bnd.call_for_all_particles_device_opencl(pso, "compute_density")
        raised = False
    except bnd.SphError as e:
        raised = "not a live device store" in str(e)
    assert raised
    assert bnd.sph_version().startswith(b"sph_gb300")


def test_missing_library_fails_loudly():
    """Without the compiled library the package does not import: there is
    no CPU fallback behind the interface."""
    import sys
    code = "import sys; sys.path.insert(0, %r); import sph" % os.path.join(ROOT, "opencl-sph_gb300")
    env = dict(os.environ, SPH_GB300_LIB=os.path.join(ROOT, "no-such-dir", "libsph_gb300.so"))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "libsph_gb300.so not found" in r.stderr


C_DRIVER = r"""
#include <stdio.h>
#include <string.h>
#include "sph_gb300.h"

/* A C caller of the store and config functions: what the reference's own
 * C code (or a MEX front end) would call, with no GPU. */
int main(int argc, char **argv) {
    if (argc < 2) return 2;
    if (load_config(argv[1]) != 0) return 3;
    const char *spec = get_config_section("psdata_specification");
    const char *files = get_config_section("opencl_kernel_files");
    if (!spec || !files) return 4;
    psdata ps;
    memset(&ps, 0, sizeof ps);
    build_psdata_from_string(&ps, spec);
    int f = get_field_psdata(ps, "gridres");
    if (f < 0) return 5;
    const unsigned int *res = (const unsigned int *)((const char *)ps.data + ps.data_offsets[f]);
    printf("fields %u size %u names %u dims %u gridres %u %u %u files %zu\n", ps.num_fields,
           psdata_data_size(ps), psdata_names_size(ps), psdata_dimensions_size(ps), res[0], res[1], res[2],
           strlen(files));
    float h = 0.5f;
    set_field_psdata(&ps, "smoothingradius", &h, sizeof h, 0);
    int s = get_field_psdata(ps, "smoothingradius");
    printf("h %g type %d\n", (double)*(const float *)((const char *)ps.data + ps.data_offsets[s]),
           (int)ps.data_ptrs[s].type);
    free_psdata(&ps);
    unload_config();
    return 0;
}
"""


def test_header_compiles_and_links_from_c_and_cpp(tmp_path):
    """include/sph_gb300.h is valid C11 and C++ (extern "C" guards), and a
    C program that includes it links against the library and reads a conf
    and a store as the Python bindings do."""
    src = tmp_path / "driver.c"
    src.write_text(C_DRIVER)
    conf = os.path.join(ROOT, "opencl-sph_gb300", "conf", "fluid.conf")
    libdir = os.path.dirname(bnd.LIB_PATH)
    outs = []
    for comp, flags in (("gcc", ["-std=c11"]), ("g++", ["-x", "c++", "-std=c++17"])):
        exe = tmp_path / ("driver_" + comp.replace("+", "p"))
        cmd = [comp] + flags + ["-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                                "-x", "none", bnd.LIB_PATH, "-Wl,-rpath," + libdir, "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        run = subprocess.run([str(exe), conf], capture_output=True, text=True, timeout=60)
        assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
        outs.append([ln for ln in run.stdout.splitlines() if ln.startswith(("fields", "h "))])
    assert outs[0] == outs[1]
    # the same figures through the Python bindings
    assert bnd.load_config(conf) == 0
    spec = bnd.get_config_section("psdata_specification")
    files = bnd.get_config_section("opencl_kernel_files")
    bnd.unload_config()
    ps = bnd.psdata()
    bnd.build_psdata_from_string(ctypes.byref(ps), spec)
    res = list(bnd.store_views(ps)["gridres"])
    want = "fields %d size %d names %d dims %d gridres %d %d %d files %d" % (
        ps.num_fields, bnd.psdata_data_size(ps), bnd.psdata_names_size(ps), bnd.psdata_dimensions_size(ps),
        res[0], res[1], res[2], len(files))
    bnd.free_psdata(ctypes.byref(ps))
    assert outs[0][0] == want
    assert outs[0][1] == "h 0.5 type %d" % 3  # T_FLOAT32
