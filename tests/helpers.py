"""Shared helpers: host stores, oracle copies and comparisons."""
import numpy as np

from sph import bindings as bnd
from sph import init_data_cpu, free_data_cpu
from oracle.oracle import OracleScene


def host_store(scene, **extra):
    """A host-only psdata for `scene` with its initial values (no GPU)."""
    ps = init_data_cpu(scene.spec)
    v = bnd.store_views(ps)
    for k, val in dict(scene.init, **extra).items():
        v[k][...] = val
    return ps, v


def oracle_of(system_or_views, prec="f32", nthreads=4, guards=3):
    views = system_or_views if isinstance(system_or_views, dict) else bnd.store_views(system_or_views.psdata)
    return OracleScene(views, prec, nthreads=nthreads, guards=guards)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def max_rel(a, b):
    """max |a-b| / max |b|"""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a - b)))
