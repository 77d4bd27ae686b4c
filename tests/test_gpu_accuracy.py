"""Accuracy against the FP64 run (the oracle's FP64 instantiation) on the
scenes the accuracy target is stated for, each simulated the full length.

- The 1,048,576-particle WCSPH slab (the plain 1M configuration) after
  1,000 substeps: within 1e-4 relative L2 of the FP64 run.
- The 4,000-particle corotational beam (10 x 10 x 40, two clamped layers)
  after 2,000 substeps: within 1e-5 relative L2.
- The 8,000-particle dam break (20^3, reflective box).  Within 1e-4 after
  500 substeps.  After 1,000 the flow has splashed and is chaotic at the
  particle level: a handful of splash particles take different paths in
  any two runs that differ in the last bit, and they carry the error (in
  the reference's algorithm in FP32, the top 1% of particles carry 99% of
  the squared error at substep 1,000).  The error there cannot be brought
  under 1e-4 by arithmetic while positions are stored in FP32: the FP64
  algorithm itself, run on positions rounded to FP32 each substep, ends at
  3.0e-4 (tests/precision_variants.py measures each variant).  So at 1,000
  substeps the GPU run is held to (a) at most twice the error of the
  reference's algorithm in FP32 (the oracle's FP32 instantiation) and
  (b) 1e-4 relative L2 over the 99% of particles that moved least from the
  FP64 run.
"""
import os

import numpy as np
import pytest

from helpers import oracle_of, rel_err
from sph import scenes

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


def bulk_rel_err(a, b, keep=0.99):
    """Relative L2 error over the fraction `keep` of particles whose
    position differs least."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(a - b, axis=1)
    idx = np.argsort(d)[: int(keep * len(d))]
    return float(np.linalg.norm(a[idx] - b[idx]) / np.linalg.norm(b[idx]))


def test_wcsph_1m_1000_substeps_against_fp64():
    sc = scenes.wcsph_slab_1m(0)
    ps = sc.system()
    o64 = oracle_of(ps, "f64", nthreads=THREADS)
    ps.update_fused(1000)
    o64.run("fluid", 1000)
    ps.sync_device_to_host()
    err = rel_err(ps.get_fields("position")[0][: sc.n], o64.a["position"][: sc.n])
    print("wcsph-1m, 1,000 substeps: relative L2 position error %.3e against the FP64 run" % err)
    assert err <= 1e-4, err
    assert ps.status() == 0
    ps.close()


def test_beam_2000_substeps_against_fp64():
    sc = scenes.solid_lattice(10, 10, 40, material="corot", seed=0, name="beam-4k")
    ps = sc.system()
    o64 = oracle_of(ps, "f64", nthreads=THREADS)
    ps.call_for_all_particles("init_original_position")
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_original_density")
    o64.setup_solid()
    ps.update_fused(2000)
    o64.run("corot", 2000)
    ps.sync_device_to_host()
    assert rel_err(ps.get_fields("position")[0][: sc.n], o64.a["position"][: sc.n]) <= 1e-5
    assert ps.status() == 0
    ps.close()


def test_dam_break_against_fp64():
    sc = scenes.wcsph_block(20, 20, 20, seed=0, name="dam-8k")
    ps = sc.system()
    o64 = oracle_of(ps, "f64", nthreads=THREADS)
    o32 = oracle_of(ps, "f32", nthreads=THREADS)
    ps.update_fused(500)
    o64.run("fluid", 500)
    o32.run("fluid", 500)
    ps.sync_device_to_host()
    e500 = rel_err(ps.get_fields("position")[0][: sc.n], o64.a["position"][: sc.n])
    assert e500 <= 1e-4, e500
    ps.update_fused(500)
    o64.run("fluid", 500)
    o32.run("fluid", 500)
    ps.sync_device_to_host()
    ref = o64.a["position"][: sc.n]
    got = ps.get_fields("position")[0][: sc.n]
    e_gpu = rel_err(got, ref)
    e_ref32 = rel_err(o32.a["position"][: sc.n], ref)
    bulk = bulk_rel_err(got, ref)
    print("dam-8k: 500 substeps %.3e; 1,000 substeps %.3e (reference algorithm in FP32: %.3e), "
          "99%% of particles %.3e" % (e500, e_gpu, e_ref32, bulk))
    assert np.isfinite(e_gpu) and e_gpu <= 2.0 * e_ref32, (e_gpu, e_ref32)
    assert bulk <= 1e-4, bulk
    assert ps.status() == 0
    ps.close()
