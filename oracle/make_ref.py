"""Build the reference's own CPU code into oracle/_ref/ (test infrastructure).

Recipe, run in the container that holds the reference checkout
(``SPH_REFERENCE_ROOT``, default ``/root/reference``):

1. Kernels.  For each material program (the ``$opencl_kernel_files`` lists
   of conf/fluid.conf, conf/strainsolid.conf and conf/svksolid.conf) the
   reference's kernels/*.cl files are concatenated, exactly as
   build_program() does (src/opencl/particle_system_host.c:184-313), into
   one C++ translation unit per precision.  Two mechanical rewrites are
   applied and nothing else is edited:
     - ``(float3)(a,b,c)`` style vector literals become ``make_float3(a,b,c)``
       (C++ would read them as a cast of a comma expression);
     - for the FP64 program, the type names ``float``/``float3`` become
       ``double``/``double3`` (float literals such as ``0.5f`` are kept).
   The per-field ``<name>_f`` / ``<name>_m`` macros that the reference
   prepends (particle_system_host.c:316-359) are generated with the field
   index looked up by name at call time.  The OpenCL built-ins come from
   ref_shim.h.  Per-particle kernels run as an OpenMP loop over the global
   id.  Kernels that need work-group semantics are driven by hand here:
   zero_gridcount/count_particles_in_bins/prefix_sum/
   copy_celloffset_to_backup/insert_particles_in_bin_array are replaced by
   a serial stable counting sort, and set_body_position/set_body_rotation
   run serially with particle 0 last so every particle reads the old pose.
2. Host store.  src/build_psdata.c, particle_system.c, config.c, note.c and
   stringly.c are compiled against a one-line stub ``CL/opencl.h`` into
   libref_psdata.so, giving the reference's own psdata layouts.  The
   sources (and the headers they include) are copied, unedited, into
   oracle/_ref/host/src/ first, so that a machine that receives oracle/_ref/
   without the reference checkout builds the same library.

Outputs go to oracle/_ref/ only (git-ignored).  When the reference checkout
is absent (a machine that only received this repository and oracle/_ref/),
the generated kernel sources and the copied host sources already in
oracle/_ref/ are compiled.  Nothing in the product imports this module.
"""
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("SPH_REFERENCE_ROOT", "/root/reference")

# material program -> reference kernel file list (the confs' $opencl_kernel_files)
PROGRAMS = {
    "fluid": ["common", "fluids"],
    "corot": ["common", "solids", "solid_corotation", "constraints", "rigidbody"],
    "svk": ["common", "solids", "solid_svk", "constraints"],
}
HOST_SOURCES = ["build_psdata.c", "particle_system.c", "config.c", "note.c", "stringly.c"]

_LITERAL = re.compile(r"\(\s*(float3|double3|uint3)\s*\)\s*\(")
_USE_FIELD = re.compile(r"USE_FIELD(?:_FIRST_VALUE)?\(\s*(\w+)\s*,")
_FIELD_INDEX = re.compile(r"\b(\w+)_f\b")
_PSO_KERNEL = re.compile(r"kernel\s+void\s+(\w+)\s*\(\s*PSO_ARGS\s*\)")


def _rewrite(src, fp64):
    if fp64:
        src = re.sub(r"\bfloat3\b", "double3", src)
        src = re.sub(r"\bfloat\b", "double", src)
    return _LITERAL.sub(lambda m: "make_" + m.group(1) + "(", src)


def _generate_program(key, files, prec):
    fp64 = prec == "f64"
    src = ""
    for f in files:
        with open(os.path.join(REF, "kernels", f + ".cl")) as fh:
            src += fh.read()
    fields = sorted({m for m in _USE_FIELD.findall(src) if m != "name"} |
                    {m for m in _FIELD_INDEX.findall(src)})
    kernels = _PSO_KERNEL.findall(src)
    src = _rewrite(src, fp64)
    ns = "ref_%s_%s" % (key, prec)
    real = "double" if fp64 else "float"
    out = []
    w = out.append
    w("// generated by oracle/make_ref.py from the reference's kernels/%s.cl -- do not edit\n"
      % ",".join(files))
    w("#include <math.h>\n#include <stddef.h>\n#include <stdint.h>\n#include <string.h>\n"
      "#include <stdlib.h>\n#include <type_traits>\n#include <vector>\n")
    w("namespace %s {\n#include \"../ref_shim.h\"\n" % ns)
    for f in fields:
        w("static int FIDX_%s = -1;\n" % f)
    w("#define kernel\n#define global\n#define local\n#define constant\n#define private\n")
    for f in fields:
        w("#define %s_f FIDX_%s\n" % (f, f))
        w("#define %s_m (((char *) data) + data_offsets[FIDX_%s])\n" % (f, f))
    w("#line 1 \"%s\"\n" % "+".join(files))
    w(src)
    w("\n#undef kernel\n#undef global\n#undef local\n#undef constant\n#undef private\n")
    w("typedef void (*kfn)(uint, char *, uint *, uint *, uint *, uint *, uint *, void *, uint *, uint *);\n")
    w("static const struct { const char *name; kfn fn; } KERNELS[] = {\n")
    for k in kernels:
        w("    {\"%s\", %s},\n" % (k, k))
    w("};\n")
    w("static const char *FIELDS[] = {%s};\n" % ", ".join('"%s"' % f for f in fields))
    w("static int *FIDX[] = {%s};\n" % ", ".join("&FIDX_%s" % f for f in fields))
    w("}  // namespace %s\n\n" % ns)
    w(_DRIVER.replace("@NS@", ns).replace("@REAL@", real)
      .replace("@HAS_BODY@", "1" if "rigidbody" in files else "0"))
    path = os.path.join(OUT, ns + ".cpp")
    with open(path, "w") as fh:
        fh.write("".join(out))
    return path


# Host-side driver appended to each generated program (own code).
_DRIVER = r'''
#define PSO_PARAMS unsigned num_fields, char *names, unsigned *names_offsets, unsigned *dimensions, \
    unsigned *num_dimensions, unsigned *dimensions_offsets, unsigned *entry_sizes, void *data,      \
    unsigned *data_sizes, unsigned *data_offsets
#define PSO_PASS num_fields, names, names_offsets, dimensions, num_dimensions, dimensions_offsets, \
    entry_sizes, data, data_sizes, data_offsets

/* Looks the program's fields up in the store: 0, or -(100 + k) when field
 * k is missing (the reference's program build fails in that case). */
static int @NS@_resolve(unsigned num_fields, char *names, unsigned *names_offsets) {
    using namespace @NS@;
    for (unsigned k = 0; k < sizeof(FIELDS) / sizeof(FIELDS[0]); ++k) {
        *FIDX[k] = -1;
        for (unsigned f = 0; f < num_fields; ++f)
            if (strcmp(names + names_offsets[f], FIELDS[k]) == 0) { *FIDX[k] = (int)f; break; }
        if (*FIDX[k] < 0) return -(100 + (int)k);
    }
    return 0;
}

/* populate_position_cuboid (common.cl:533-555) over its 3-D range, one
 * work item at a time; returns 0 or the field lookup's error. */
extern "C" int @NS@_populate_cuboid(PSO_PARAMS, const @REAL@ *c1, const @REAL@ *c2, const unsigned *size) {
    using namespace @NS@;
    int rc = @NS@_resolve(num_fields, names, names_offsets);
    if (rc) return rc;
    vec3<@REAL@> a = {c1[0], c1[1], c1[2]}, b = {c2[0], c2[1], c2[2]};
    uint3 sz = {size[0], size[1], size[2]};
    g_work_dim = 3;
    for (unsigned k = 0; k < size[2]; ++k)
        for (unsigned j = 0; j < size[1]; ++j)
            for (unsigned i = 0; i < size[0]; ++i) {
                g_global_id = i;
                g_global_id_yz[0] = j;
                g_global_id_yz[1] = k;
                populate_position_cuboid(PSO_PASS, a, b, sz);
            }
    g_work_dim = 1;
    return 0;
}

/* rotate_particles (common.cl:556-604) over `global_size` work items. */
extern "C" int @NS@_rotate(PSO_PARAMS, unsigned global_size, @REAL@ ax, @REAL@ ay, @REAL@ az) {
    using namespace @NS@;
    int rc = @NS@_resolve(num_fields, names, names_offsets);
    if (rc) return rc;
    for (unsigned i = 0; i < global_size; ++i) {
        g_global_id = i;
        rotate_particles(PSO_PASS, ax, ay, az);
    }
    return 0;
}

/* Returns 0, or -1 for an unknown kernel, or the field lookup's error. */
extern "C" int @NS@_call(const char *kernel_name, unsigned global_size, int nthreads, PSO_PARAMS,
                         unsigned body, const @REAL@ *vec3arg) {
    using namespace @NS@;
    int rc = @NS@_resolve(num_fields, names, names_offsets);
    if (rc) return rc;
    if (nthreads < 1) nthreads = 1;
    auto run_all = [&](kfn fn, unsigned count) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
        for (long i = 0; i < (long)count; ++i) {
            g_global_id = (size_t)i;
            fn(PSO_PASS);
        }
    };
    if (strcmp(kernel_name, "compute_particle_bins") == 0) {
        kfn bins = nullptr;
        for (auto &k : KERNELS) if (strcmp(k.name, "find_particle_bins") == 0) bins = k.fn;
        unsigned n = *(unsigned *)(((char *)data) + data_offsets[FIDX_n]);
        run_all(bins, n);
        unsigned *res = (unsigned *)(((char *)data) + data_offsets[FIDX_gridres]);
        unsigned *cell = (unsigned *)(((char *)data) + data_offsets[FIDX_gridcell]);
        unsigned *count = (unsigned *)(((char *)data) + data_offsets[FIDX_gridcount]);
        unsigned *off = (unsigned *)(((char *)data) + data_offsets[FIDX_celloffset]);
        unsigned *parts = (unsigned *)(((char *)data) + data_offsets[FIDX_cellparticles]);
        size_t C = (size_t)res[0] * res[1] * res[2];
        memset(count, 0, C * sizeof(unsigned));
        for (unsigned i = 0; i < n; ++i) count[cell[i]]++;
        unsigned run = 0;
        for (size_t c = 0; c < C; ++c) { off[c] = run; run += count[c]; }
        std::vector<unsigned> cursor(off, off + C);
        for (unsigned i = 0; i < n; ++i) parts[cursor[cell[i]]++] = i;
        return 0;
    }
#if @HAS_BODY@
    if (strcmp(kernel_name, "set_body_position") == 0 || strcmp(kernel_name, "set_body_rotation") == 0) {
        @NS@::vec3<@REAL@> v = {vec3arg[0], vec3arg[1], vec3arg[2]};
        bool pos = kernel_name[9] == 'p';
        for (long i = (long)global_size - 1; i >= 0; --i) {
            g_global_id = (size_t)i;
            if (pos) set_body_position(PSO_PASS, body, v);
            else set_body_rotation(PSO_PASS, body, v);
        }
        return 0;
    }
#endif
    for (auto &k : KERNELS)
        if (strcmp(k.name, kernel_name) == 0) { run_all(k.fn, global_size); return 0; }
    return -1;
}
extern "C" const char *@NS@_field(unsigned k) {
    using namespace @NS@;
    return k < sizeof(FIELDS) / sizeof(FIELDS[0]) ? FIELDS[k] : nullptr;
}
'''


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("command failed: " + " ".join(cmd))


def generate():
    """Write the generated sources into oracle/_ref/ (needs the reference)."""
    os.makedirs(OUT, exist_ok=True)
    paths = []
    for key, files in PROGRAMS.items():
        for prec in ("f32", "f64"):
            paths.append(_generate_program(key, files, prec))
    host = os.path.join(OUT, "host")
    os.makedirs(os.path.join(host, "CL"), exist_ok=True)
    with open(os.path.join(host, "CL", "opencl.h"), "w") as fh:
        fh.write("typedef void *cl_mem; typedef void *cl_kernel; typedef void *cl_program;\n")
    # the host builder's sources and headers, as they are
    src_copy = os.path.join(host, "src")
    if os.path.isdir(src_copy):
        shutil.rmtree(src_copy)
    shutil.copytree(os.path.join(REF, "src"), src_copy,
                    ignore=shutil.ignore_patterns("mex", "*.o", "*.so"))
    return paths


def compile_all(jobs=8):
    """Compile whatever generated sources exist in oracle/_ref/."""
    cpps = sorted(os.path.join(OUT, f) for f in os.listdir(OUT) if f.endswith(".cpp"))
    flags = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fopenmp",
             "-w"]
    objs = [p[:-4] + ".o" for p in cpps]
    with ThreadPoolExecutor(jobs) as ex:
        list(ex.map(lambda a: _run(["g++"] + flags + ["-c", a[0], "-o", a[1]]), zip(cpps, objs)))
    lib = os.path.join(OUT, "libref_kernels.so")
    _run(["g++", "-shared", "-fopenmp", "-o", lib] + objs + ["-lm"])
    built = [lib]
    src_dir = os.path.join(REF, "src")
    if not os.path.isdir(src_dir):
        src_dir = os.path.join(OUT, "host", "src")
    if all(os.path.exists(os.path.join(src_dir, f)) for f in HOST_SOURCES):
        inc = os.path.join(OUT, "host")
        srcs = [os.path.join(src_dir, s) for s in HOST_SOURCES]
        plib = os.path.join(OUT, "libref_psdata.so")
        _run(["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-w", "-I" + inc, "-I" + src_dir,
              "-o", plib] + srcs + ["-lm"])
        built.append(plib)
    return built


def main():
    if os.path.isdir(os.path.join(REF, "kernels")):
        generate()
    elif not (os.path.isdir(OUT) and any(f.endswith(".cpp") for f in os.listdir(OUT))):
        print("make_ref: no reference checkout and no generated sources; nothing to build")
        return 0
    for p in compile_all():
        print("built", os.path.relpath(p, os.path.dirname(HERE)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
