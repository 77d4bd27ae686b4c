"""GPU parity: neighbour grid, density, WCSPH forces, integration.

Each test runs the CUDA path through the C ABI and the CPU oracle
(oracle/sph_oracle.c, itself pinned bit-exact to the reference's kernels)
on the same store.  Tolerances:
  - integer and index outputs (gridcell, gridcount, celloffset,
    cellparticles, num_neighbours): bit-exact;
  - density: max |d| <= 1e-5 of max |rho| (poly6 evaluated from r^2 and
    summed per stencil row with the row sums Kahan-compensated, the oracle
    sums pow() terms plainly);
  - forces: max |d| <= 1e-4 of max |f| on identical inputs;
  - positions after N substeps: relative L2 error <= 1e-5.
"""
import numpy as np
import pytest

from helpers import max_rel, oracle_of, rel_err
from sph import scenes

pytestmark = pytest.mark.gpu


def _bins_equal(ps, orc, n):
    ps.sync_device_to_host()
    cell, count, off, parts = ps.get_fields("gridcell", "gridcount", "celloffset", "cellparticles")
    orc.call("compute_particle_bins")
    assert np.array_equal(cell[:n], orc.a["gridcell"][:n])
    assert np.array_equal(count.ravel(), orc.a["gridcount"])
    assert np.array_equal(off.ravel(), orc.a["celloffset"])
    assert np.array_equal(parts[:n], orc.a["cellparticles"][:n])


@pytest.mark.parametrize("jitter", [0.0, 1e-4, 3e-3])
def test_bins_bitexact(jitter):
    sc = scenes.wcsph_block(13, 9, 11, jitter=jitter, seed=11)
    ps = sc.system()
    orc = oracle_of(ps)
    ps.compute_particle_bins()
    _bins_equal(ps, orc, sc.n)
    assert ps.status() == 0
    ps.close()


def test_bins_outside_grid_and_crowded_cells():
    """Particles outside gridbounds clamp into edge cells (status bit 1);
    a cell with more than 32 particles takes the block-sort path."""
    sc = scenes.wcsph_block(10, 10, 10, jitter=1e-4, seed=3)
    pos = sc.init["position"].copy()
    rng = np.random.default_rng(5)
    pos[:40] = rng.uniform(-0.3, -0.01, size=(40, 3))           # below the box: corner cell
    pos[40:140] = 0.105 + rng.uniform(0, 0.004, size=(100, 3))  # 100 in one cell
    pos[140:180] = rng.uniform(0.45, 0.9, size=(40, 3))         # above the box
    ps = sc.system()
    ps.set_fields(position=pos)
    orc = oracle_of(ps)
    ps.compute_particle_bins()
    _bins_equal(ps, orc, sc.n)
    assert ps.status() & 2
    ps.close()


def test_substep_on_crowded_outside_and_ragged_scene_against_oracle():
    """One fused substep of a scene that holds a crowded cluster (stencil
    rows of more than 64 candidates: the scan path), particles clamped into
    edge cells from below and above the grid, and n < pnum, against the
    oracle: cell tables and neighbour counts exact, densities within 1e-5,
    velocities within 1e-5 and positions within 1e-6 (relative L2)."""
    sc = scenes.wcsph_block(10, 10, 10, jitter=1e-4, seed=17, walls=False)
    pos = sc.init["position"].copy()
    rng = np.random.default_rng(8)
    pos[:30] = rng.uniform(-0.3, -0.01, size=(30, 3))            # below the box
    pos[30:130] = 0.105 + rng.uniform(0, 0.006, size=(100, 3))   # 100 within 0.006 m
    pos[130:160] = rng.uniform(0.45, 0.9, size=(30, 3))          # above the box
    n = sc.n - 37
    ps = sc.system()
    ps.set_fields(position=pos, n=n)
    orc = oracle_of(ps)
    ps.update_fused(1)
    orc.run("fluid", 1)
    ps.sync_device_to_host()
    for f in ("gridcell", "cellparticles", "num_neighbours"):
        assert np.array_equal(ps.get_fields(f)[0][:n], orc.a[f][:n]), f
    assert orc.a["num_neighbours"][30:130].min() > 64
    assert max_rel(ps.get_fields("density")[0][:n], orc.a["density"][:n]) <= 1e-5
    assert rel_err(ps.get_fields("velocity")[0][:n], orc.a["velocity"][:n]) <= 1e-5
    assert rel_err(ps.get_fields("position")[0][:n], orc.a["position"][:n]) <= 1e-6
    assert ps.status() & 2
    ps.close()


@pytest.mark.parametrize("n_active", [0, 1, 777])
def test_bins_ragged_n(n_active):
    sc = scenes.wcsph_block(10, 10, 10, jitter=1e-4, seed=9)
    ps = sc.system()
    ps.set_fields(n=n_active)
    orc = oracle_of(ps)
    ps.compute_particle_bins()
    _bins_equal(ps, orc, n_active)
    ps.call_for_all_particles("compute_density")
    ps.sync_device_to_host()
    orc.call("compute_density")
    assert np.array_equal(ps.get_fields("num_neighbours")[0][:n_active], orc.a["num_neighbours"][:n_active])
    ps.close()


def test_reference_kernel_sequence_equals_fused_bins():
    """find_particle_bins, zero_gridcount, count_particles_in_bins,
    prefix_sum, copy_celloffset_to_backup, insert_particles_in_bin_array
    called by name give compute_particle_bins' tables."""
    sc = scenes.wcsph_block(9, 9, 9, jitter=2e-3, seed=2)
    ps = sc.system()
    orc = oracle_of(ps)
    for k in ["find_particle_bins", "zero_gridcount", "count_particles_in_bins", "prefix_sum",
              "copy_celloffset_to_backup", "insert_particles_in_bin_array"]:
        ps.call_for_all_particles(k)
    _bins_equal(ps, orc, sc.n)
    ps.close()


def test_density_and_neighbour_sets():
    sc = scenes.wcsph_block(14, 12, 10, jitter=2e-3, seed=4)
    ps = sc.system()
    orc = oracle_of(ps)
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_density")
    ps.sync_device_to_host()
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    n = sc.n
    nn, rho = ps.get_fields("num_neighbours", "density")
    assert np.array_equal(nn[:n], orc.a["num_neighbours"][:n])
    assert max_rel(rho[:n], orc.a["density"][:n]) <= 1e-5


def test_forces_on_identical_inputs():
    sc = scenes.wcsph_block(12, 12, 12, jitter=1e-3, seed=6)
    ps = sc.system()
    rng = np.random.default_rng(1)
    ps.set_fields(velocity=rng.normal(0, 0.05, size=(sc.n, 3)).astype(np.float32))
    orc = oracle_of(ps)
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    ps.compute_particle_bins()
    ps.set_fields(density=orc.a["density"])  # the oracle's density as input
    ps.call_for_all_particles("compute_forces_fluids")
    orc.call("compute_forces_fluids")
    ps.sync_device_to_host()
    f = ps.get_fields("force")[0][: sc.n]
    assert max_rel(f, orc.a["force"][: sc.n]) <= 1e-4
    ps.close()


@pytest.mark.parametrize("box", [(-1.9, -1.5), (1.7, 2.1)])
def test_forces_in_the_cube_band(box):
    """APPLY_CUBE_BOUNDS (common.cl:37-43): a block straddling the band
    0.2 inside -2 or 2 on every axis, so some particles take the band's
    double-precision update and the others the plain force; the band's
    tests run in FP32 against the floats just outside its bounds."""
    sc = scenes.wcsph_block(12, 12, 12, box=box, jitter=1e-3, seed=7, walls=False)
    pos = np.asarray(sc.init["position"][: sc.n])
    inside = (pos <= -1.8000000715255737) | (pos >= 1.8000000715255737)
    assert inside.any() and (~inside).any()
    ps = sc.system()
    orc = oracle_of(ps)
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    ps.compute_particle_bins()
    ps.set_fields(density=orc.a["density"])
    ps.call_for_all_particles("compute_forces_fluids")
    orc.call("compute_forces_fluids")
    ps.sync_device_to_host()
    f = ps.get_fields("force")[0][: sc.n]
    assert max_rel(f, orc.a["force"][: sc.n]) <= 1e-4
    ps.close()


@pytest.mark.parametrize("planes", [False, True])
def test_named_forces_walk_masks_only_right_after_density(planes):
    """A named compute_forces_fluids called right after a named
    compute_density walks the masks that pass recorded; with any call in
    between (here a status query) it scans.  Both give the same bits, and
    the count the density pass left is the force pass's."""
    sc = scenes.wcsph_block(12, 10, 12, jitter=1e-3, seed=12)
    if planes:
        # mirror planes through the box corner, normals along the axes
        sc.entries = [("symmetry_planes", "3, 2, 3", "float", None) if e[0] == "symmetry_planes" else e
                      for e in sc.entries]
        sp = np.zeros((3, 2, 3), np.float32)
        for k in range(3):
            sp[k, 1, k] = 1.0
        sc.init = dict(sc.init, symmetry_planes=sp)
    a, b = sc.system(), sc.system()
    rng = np.random.default_rng(3)
    vel = rng.normal(0, 0.05, size=(sc.n, 3)).astype(np.float32)
    for ps in (a, b):
        ps.set_fields(velocity=vel)
        ps.compute_particle_bins()
        ps.call_for_all_particles("compute_density")
    a.call_for_all_particles("compute_forces_fluids")  # the masked walk
    assert b.status() == 0  # a call in between: the scan
    b.call_for_all_particles("compute_forces_fluids")
    a.sync_device_to_host()
    b.sync_device_to_host()
    n = sc.n
    for f in ("force", "density", "num_neighbours"):
        assert np.array_equal(a.get_fields(f)[0][:n], b.get_fields(f)[0][:n]), f
    orc = oracle_of(b)
    orc.call("compute_particle_bins")
    orc.call("compute_density")
    assert np.array_equal(a.get_fields("num_neighbours")[0][:n], orc.a["num_neighbours"][:n])
    a.close()
    b.close()


@pytest.mark.parametrize("walls", [False, True])
def test_trajectory_named_and_fused(walls):
    """N substeps through the reference's kernel names and through the
    CUDA-graph substep agree with the oracle."""
    sc = scenes.wcsph_block(12, 10, 12, jitter=1e-4, seed=8, walls=walls)
    steps = 40
    a = sc.system()
    b = sc.system()
    orc = oracle_of(a)
    for _ in range(steps):
        a.compute_particle_bins()
        for k in ["compute_density", "compute_forces_fluids", "step_forward"]:
            a.call_for_all_particles(k)
    b.update_fused(steps)
    orc.run("fluid", steps)
    a.sync_device_to_host()
    b.sync_device_to_host()
    n = sc.n
    pa = a.get_fields("position")[0][:n]
    pb = b.get_fields("position")[0][:n]
    assert np.array_equal(pa, pb), "named and fused paths differ"
    assert rel_err(pa, orc.a["position"][:n]) <= 1e-5
    a.close()
    b.close()


def test_error_vs_fp64_run():
    """FP32 GPU trajectory against the all-FP64 oracle run of the scene."""
    sc = scenes.wcsph_block(10, 10, 10, jitter=1e-4, seed=12)
    ps = sc.system()
    o64 = oracle_of(ps, prec="f64")
    steps = 100
    ps.update_fused(steps)
    o64.run("fluid", steps)
    ps.sync_device_to_host()
    err = rel_err(ps.get_fields("position")[0][: sc.n], o64.a["position"][: sc.n])
    assert err <= 1e-4
    ps.close()


def test_coincident_particles_stay_finite():
    """Two distinct particles at the same position: the reference's force
    divides by their zero distance (NaN); here the pair contributes
    nothing, as in the oracle with its guards on."""
    sc = scenes.wcsph_block(8, 8, 8, jitter=1e-4, seed=2, walls=False)
    ps = sc.system()
    pos = sc.init["position"].copy()
    pos[100] = pos[101]
    ps.set_fields(position=pos)
    orc = oracle_of(ps)
    ps.update_fused(1)
    orc.run("fluid", 1)
    ps.sync_device_to_host()
    p = ps.get_fields("position")[0][: sc.n]
    assert np.isfinite(p).all() and ps.status() == 0
    assert rel_err(p, orc.a["position"][: sc.n]) <= 1e-6
    ps.close()


def test_status_nonfinite():
    sc = scenes.wcsph_block(8, 8, 8, jitter=1e-4, seed=1)
    ps = sc.system()
    pos = sc.init["position"].copy()
    pos[5] = np.nan
    ps.set_fields(position=pos)
    ps.update_fused(1)
    assert ps.status() & 1
    ps.close()


def test_fused_masks_with_crowded_stencils_equal_named_scan():
    """The fused substep walks the density pass's candidate masks (at most
    512 candidates per particle) and scans the stencil beyond that; both
    must give the named path's result bit for bit."""
    sc = scenes.wcsph_block(12, 12, 12, jitter=1e-4, seed=13, walls=True)
    pos = sc.init["position"].copy()
    rng = np.random.default_rng(3)
    pos[:600] = 0.2 + rng.uniform(-0.008, 0.008, size=(600, 3))  # > 512 candidates each
    a = sc.system()
    b = sc.system()
    a.set_fields(position=pos)
    b.set_fields(position=pos)
    for _ in range(3):
        a.compute_particle_bins()
        for k in ["compute_density", "compute_forces_fluids", "step_forward"]:
            a.call_for_all_particles(k)
    b.update_fused(3)
    a.sync_device_to_host()
    b.sync_device_to_host()
    n = sc.n
    for f in ("position", "velocity", "force", "density"):
        assert np.array_equal(a.get_fields(f)[0][:n], b.get_fields(f)[0][:n]), f
    a.close()
    b.close()


def test_device_recording_equals_host_syncs():
    """Positions recorded on the device every 3 substeps equal the ones a
    host sync after every 3 substeps sees; the ring keeps the last frames."""
    sc = scenes.wcsph_block(10, 8, 10, jitter=1e-4, seed=21)
    a = sc.system()
    a.record_start(["position", "velocity"], every=3, frames=4)
    a.update_fused(20)  # 6 frames recorded: after substeps 3, 6, ..., 18
    assert a.record_count() == 6
    rec = a.record_read()
    assert rec["position"].shape == (4,) + a.get_fields("position")[0].shape
    b = sc.system()
    want = []
    for _ in range(6):
        b.update_fused(3)
        b.sync_device_to_host()
        want.append((np.array(b.get_fields("position")[0]), np.array(b.get_fields("velocity")[0])))
    for f in range(4):
        assert np.array_equal(rec["position"][f], want[2 + f][0])
        assert np.array_equal(rec["velocity"][f], want[2 + f][1])
    # recording can be restarted and stopped; without it update is unchanged
    a.record_stop()
    a.update_fused(1)
    a.close()
    b.close()


def test_async_store_transfers_match_blocking_syncs():
    """The store's asynchronous transfers give what the blocking syncs give:
    a read holds the fields as of its place in the stream although later
    substeps run while it is written, an asynchronous upload acts like the
    blocking one, and pipelined reads end on the final state."""
    sc = scenes.wcsph_block(14, 10, 12, jitter=1e-4, seed=21)
    a, b = sc.system(), sc.system()
    a.pin()
    a.pin()  # pinning twice is harmless
    a.update_fused(3)
    b.update_fused(3)
    t = a.read_fields_async("position", "velocity")
    a.update_fused(4)
    a.wait_read(t)
    b.sync_fields_device_to_host("position", "velocity")
    pa, va = (np.array(x) for x in a.get_fields("position", "velocity"))
    pb, vb = b.get_fields("position", "velocity")
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    # an asynchronous upload of gravity, then pipelined reads
    b.update_fused(4)
    for ps in (a, b):
        ps.get_fields("gravity")[0][:] = (0.5, -3.0, 0.25)
        ps.get_fields("timestep")[0][:] = 0.9 * ps.get_fields("timestep")[0]
    # (a pinned store's small fields go by one copy kernel reading the
    # mapped host store)
    a.write_fields_async("gravity", "timestep")
    b.sync_fields_host_to_device("gravity", "timestep")
    prev = None
    for _ in range(5):
        a.update_fused(1)
        tk = a.read_fields_async("position")
        if prev is not None:
            a.wait_read(prev)
        prev = tk
    a.wait_reads()
    b.update_fused(5)
    b.sync_fields_device_to_host("position")
    assert np.array_equal(np.array(a.get_fields("position")[0]), np.array(b.get_fields("position")[0]))
    # a blocking sync after reads in flight sees the newest state
    a.update_fused(2)
    b.update_fused(2)
    a.read_fields_async("position")
    a.sync_fields_device_to_host("velocity", "position")
    b.sync_fields_device_to_host("velocity", "position")
    assert np.array_equal(np.array(a.get_fields("position")[0]), np.array(b.get_fields("position")[0]))
    with pytest.raises(Exception):
        a.read_fields_async("no_such_field")
    with pytest.raises(Exception):
        a.wait_read(10 ** 9)
    a.unpin()
    a.close()
    b.close()


def test_known_answers_single_particle_and_pair():
    """Hand-checkable cases on the CUDA path: a lone particle's density is
    its own weight m 315/(64 pi h^3) with one neighbour (itself) and no
    force but gravity; two particles at distance r < h have equal densities
    m (W(0) + W(r)), two neighbours each, and equal and opposite forces
    along the line between them."""
    one = scenes.wcsph_block(1, 1, 1, jitter=0.0, walls=False, gravity=(0.0, 0.0, 0.0))
    ps = one.system()
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_density")
    ps.call_for_all_particles("compute_forces_fluids")
    ps.sync_device_to_host()
    h = float(ps.get_fields("smoothingradius")[0].ravel()[0])
    m = float(ps.get_fields("mass")[0].ravel()[0])
    pi = float(np.float32(3.1415926535))
    w0 = 315.0 / (64.0 * pi * h ** 3)
    assert ps.get_fields("density")[0][0] == pytest.approx(m * w0, rel=1e-6)
    assert int(ps.get_fields("num_neighbours")[0][0]) == 1
    assert np.all(ps.get_fields("force")[0][0] == 0.0)
    ps.close()

    two = scenes.wcsph_block(2, 1, 1, spacing=0.013, jitter=0.0, walls=False, gravity=(0.0, 0.0, 0.0))
    ps = two.system()
    ps.compute_particle_bins()
    ps.call_for_all_particles("compute_density")
    ps.call_for_all_particles("compute_forces_fluids")
    ps.sync_device_to_host()
    m = float(ps.get_fields("mass")[0].ravel()[0])
    x = ps.get_fields("position")[0][:2].astype(np.float64)
    r = float(np.linalg.norm(x[1] - x[0]))
    want = m * 315.0 / (64.0 * pi * h ** 9) * ((h * h) ** 3 + (h * h - r * r) ** 3)
    rho = ps.get_fields("density")[0][:2]
    assert rho[0] == rho[1] and rho[0] == pytest.approx(want, rel=1e-5)
    assert list(ps.get_fields("num_neighbours")[0][:2]) == [2, 2]
    f = ps.get_fields("force")[0][:2].astype(np.float64)
    assert np.all(f[0] == -f[1]) and f[0][0] != 0.0
    assert f[0][1] == 0.0 and f[0][2] == 0.0
    ps.close()
