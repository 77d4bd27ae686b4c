"""bench.py's reference arm on the CPU (it needs no GPU): one JSON line with
the contract's keys, on the same config as the GPU arm, timing the
reference's own kernels (oracle/_ref) where they were built and the oracle
port elsewhere, without loading the sph package or the CUDA library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_arm(*extra):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "dam-8k",
           "--steps", "2", "--warmup", "3"] + list(extra)
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    sys.path.insert(0, ROOT)
    import bench
    from oracle import ref
    d = run_arm()
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"] == bench.workload_config("dam-8k", 0, standalone=True)
    assert d["config"] == bench.workload_config("dam-8k", 0)  # the GPU arm's
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1
    assert cb["kind"] == ("reference" if ref.available() else "port")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_maps_no_library_of_the_product():
    """The arm's process maps the reference's libraries and none of this
    repository's CUDA library (checked from inside the process)."""
    probe = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'dam-8k', "
             "'--steps', '1', '--warmup', '3'];\n"
             "try:\n    runpy.run_path('bench.py', run_name='__main__')\n"
             "except SystemExit:\n    pass\n"
             "maps = open('/proc/self/maps').read()\n"
             "print('MAPPED', 'libsph_gb300' in maps, 'libref_kernels' in maps)")
    out = subprocess.run([sys.executable, "-c", probe], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    flags = [ln for ln in out.stdout.splitlines() if ln.startswith("MAPPED")][0].split()
    assert flags[1] == "False"
    sys.path.insert(0, ROOT)
    from oracle import ref
    assert flags[2] == str(ref.available())
