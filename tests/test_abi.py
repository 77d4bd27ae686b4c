"""The C-ABI library (no GPU): it loads, exports every function that
include/sph_gb300.h declares, and its struct layouts match the
reference's (psdata, psdata_opencl) so the reference's ctypes bindings can
bind it."""
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
