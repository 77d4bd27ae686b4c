"""GPU: sph_compute_particle_bins_noalloc, the neighbour-grid sort for
callers that cannot allocate device memory -- engines whose own pool owns
all device memory, real-time loops that cannot afford cudaMalloc's implicit
synchronisation (see include/sph_gb300.h).

It must give the cell tables of the store path's compute_particle_bins
(the existing entry point) bit for bit -- the tolerance the other tests
use for integer outputs -- on two calls in a row, the second after the
first has left its state in the shared scratch array.  Collected last so
that a stop at the first failure has run every other test first; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from sph import bindings as bnd
from sph import scenes

pytestmark = pytest.mark.gpu

_fn = bnd.library.sph_compute_particle_bins_noalloc
_fn.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                ctypes.c_void_p]
_fn.restype = ctypes.c_int


def store_tables(scene, pos):
    """The existing entry point: compute_particle_bins on a device store."""
    ps = scene.system()
    ps.set_fields(position=pos)
    ps.compute_particle_bins()
    ps.sync_device_to_host()
    out = [np.array(a) for a in ps.get_fields("gridcell", "gridcount", "celloffset", "cellparticles", "gridres",
                                              "gridbounds")]
    ps.close()
    return out


def noalloc_tables(pos, res, bounds):
    """The no-alloc entry point on device copies of the inputs; returns the
    four tables and the status word it ORed its bits into."""
    import torch
    n = pos.shape[0]
    cells = int(np.prod(res))
    d_pos = torch.from_numpy(np.ascontiguousarray(pos, dtype=np.float32).reshape(-1)).cuda()
    d_gb = torch.from_numpy(np.ascontiguousarray(bounds, dtype=np.float32).ravel()).cuda()
    cell = torch.full((max(n, 1),), 0xDEAD, dtype=torch.int32, device="cuda")
    count = torch.full((cells,), 7, dtype=torch.int32, device="cuda")   # stale values must not survive
    off = torch.zeros(cells, dtype=torch.int32, device="cuda")
    parts = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = _fn(d_pos.data_ptr() if n else None, n, d_gb.data_ptr(), int(res[0]), int(res[1]), int(res[2]),
             cell.data_ptr(), count.data_ptr(), off.data_ptr(), parts.data_ptr(), status.data_ptr(), None)
    assert rc == 0, bnd.last_error()
    torch.cuda.synchronize()
    as_u32 = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
    return as_u32(cell)[:n], as_u32(count), as_u32(off), as_u32(parts)[:n], int(as_u32(status)[0])


def test_noalloc_bins_equal_store_path_two_calls():
    # call 1: particles outside the grid and a cell of 100 (crowded-cell path)
    a = scenes.wcsph_block(12, 10, 11, jitter=1e-4, seed=3)
    pa = a.init["position"].copy()
    rng = np.random.default_rng(5)
    pa[:40] = rng.uniform(-0.3, -0.01, size=(40, 3))
    pa[40:140] = 0.105 + rng.uniform(0, 0.004, size=(100, 3))
    # call 2: a different size and grid, ordinary occupancy
    b = scenes.wcsph_block(17, 9, 13, spacing=0.008, h=0.017, box=(0.0, 0.35), jitter=2e-3, seed=9)
    pb = b.init["position"].copy()
    for scene, pos, outside in ((a, pa, True), (b, pb, False)):
        cell, count, off, parts, res, bounds = store_tables(scene, pos)
        got = noalloc_tables(pos, res, bounds)
        n = scene.n
        assert np.array_equal(got[0], cell[:n])
        assert np.array_equal(got[1], count.ravel())
        assert np.array_equal(got[2], off.ravel())
        assert np.array_equal(got[3], parts[:n])
        # bit 1: particles outside gridbounds were clamped into edge cells
        assert got[4] == (2 if outside else 0), got[4]


def test_noalloc_empty_scene_gives_empty_cells():
    # a call with particles first, so that the empty call must clear them
    a = scenes.wcsph_block(6, 5, 7, jitter=1e-4, seed=2)
    _, _, _, _, res, bounds = store_tables(a, a.init["position"])
    noalloc_tables(a.init["position"], res, bounds)
    cell, count, off, parts, status = noalloc_tables(np.zeros((0, 3), np.float32), res, bounds)
    assert cell.size == 0 and parts.size == 0
    assert not count.any() and not off.any() and status == 0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    dummy = torch.zeros(16, device="cuda")
    p = dummy.data_ptr()
    assert _fn(p, (1 << 20) + 1, p, 4, 4, 4, p, p, p, p, None, None) == -1
    assert "exceed" in bnd.last_error()
    assert _fn(p, 1, p, 1 << 11, 1 << 11, 2, p, p, p, p, None, None) == -1
    assert "cells" in bnd.last_error()
