"""GPU: the batched and served forms.

A scene advanced inside a batch (any mix of fluid, corotational and SVK
scenes, added and removed while others run, any launch shape) must give
bit-identical results to the same scene run alone through the drop-in
path, which the other GPU tests tie to the oracle.  The serving loop must
return, for every request, the same result as the request run alone.
"""
import numpy as np
import pytest

from helpers import oracle_of, rel_err
from sph import scenes
from sph.batch import Batch
from sph.serving import Server, poisson_requests, release

pytestmark = pytest.mark.gpu


def alone(scene, steps):
    ps = scene.system()
    if scene.material != "fluid":
        ps.call_for_all_particles("init_original_position")
        ps.compute_particle_bins()
        ps.call_for_all_particles("compute_original_density")
    ps.update_fused(steps)
    ps.sync_device_to_host()
    pos = np.array(ps.get_fields("position")[0][: scene.n])
    vel = np.array(ps.get_fields("velocity")[0][: scene.n])
    ps.close()
    return pos, vel


def mix(seed=0):
    return [
        scenes.wcsph_block(9, 6, 9, jitter=1e-4, seed=seed + 1, name="f1"),
        scenes.solid_lattice(5, 5, 9, material="corot", youngs_modulus=3e4, jitter=1e-4, seed=seed + 2,
                             clamp_layers=1, name="c1"),
        scenes.wcsph_block(13, 7, 11, jitter=1e-4, seed=seed + 3, name="f2"),
        scenes.solid_lattice(6, 5, 7, material="svk", youngs_modulus=5e4, poisson=0.35, jitter=1e-4,
                             seed=seed + 4, clamp_layers=1, name="s1"),
    ]


def test_batch_matches_scenes_alone():
    scs = mix()
    steps = 12
    b = Batch()
    ids = [b.add(s) for s in scs]
    b.step(steps)
    for s, sid in zip(scs, ids):
        v = b.read(sid)
        pos, vel = alone(s, steps)
        assert np.array_equal(v["position"][: s.n], pos), s.name
        assert np.array_equal(v["velocity"][: s.n], vel), s.name
        assert b.status(sid) == 0
    b.close()


def test_batch_matches_oracle():
    scs = mix(seed=10)
    steps = 10
    b = Batch()
    ids = [b.add(s) for s in scs]
    orcs = []
    for s in scs:
        ps = Batch.host_store(s)
        from sph import bindings as bnd
        o = oracle_of(bnd.store_views(ps))
        if s.material != "fluid":
            o.setup_solid()
        orcs.append((o, ps))
    b.step(steps)
    for s, sid, (o, ps) in zip(scs, ids, orcs):
        o.run(s.material, steps)
        v = b.read(sid)
        assert rel_err(v["position"][: s.n], o.a["position"][: s.n]) <= 1e-5, s.name
        assert np.array_equal(v["num_neighbours"][: s.n], o.a["num_neighbours"][: s.n]), s.name
    b.close()


def test_scenes_join_and_leave_while_others_run():
    a, c, f2, s1 = mix(seed=20)
    b = Batch()
    ia = b.add(a)
    ic = b.add(c)
    b.step(5)
    i2 = b.add(f2)          # joins after 5 substeps
    b.step(4)
    b.remove(ia)            # leaves after 9
    is1 = b.add(s1)         # joins after 9
    b.step(3)
    assert np.array_equal(b.read(ic)["position"][: c.n], alone(c, 12)[0])
    assert np.array_equal(b.read(i2)["position"][: f2.n], alone(f2, 7)[0])
    assert np.array_equal(b.read(is1)["position"][: s1.n], alone(s1, 3)[0])
    b.close()


@pytest.mark.parametrize("shape", [(128, 64, 0), (512, 256, 304), (256, 128, 152)])
def test_launch_shape_does_not_change_results(shape):
    scs = mix(seed=30)
    ref = Batch()
    ids = [ref.add(s) for s in scs]
    ref.step(6)
    want = [np.array(ref.read(i)["position"]) for i in ids]
    ref.close()
    b = Batch()
    b.tune(*shape)
    ids = [b.add(s) for s in scs]
    b.step(6)
    for i, w in zip(ids, want):
        assert np.array_equal(b.read(i)["position"], w)
    b.close()


def test_served_results_equal_alone():
    def make(rng, i):
        kind = i % 3
        if kind == 0:
            return scenes.wcsph_block(int(rng.integers(6, 11)), 6, int(rng.integers(6, 11)), seed=i, name="r%d" % i)
        mat = "corot" if kind == 1 else "svk"
        return scenes.solid_lattice(5, 5, int(rng.integers(6, 10)), material=mat, seed=i, clamp_layers=1,
                                    name="r%d" % i)
    reqs = poisson_requests(rate=200.0, duration=0.06, make_scene=make, steps_range=(3, 17), seed=4)
    assert len(reqs) >= 6
    srv = Server(budget_bytes=40e6, max_chunk=4)
    stats = srv.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs) and stats["p99_s"] >= stats["p50_s"] > 0
    for r in reqs:
        pos, vel = alone(r.scene, r.steps)
        assert np.array_equal(r.result["position"], pos), r.scene.name
        assert np.array_equal(r.result["velocity"], vel), r.scene.name
    release(reqs)


def test_step_quota_idles_scene():
    """A scene whose quota runs out stays unchanged while the batch goes
    on; given a new quota it resumes exactly where it stopped."""
    scs = mix(seed=40)
    b = Batch()
    ids = [b.add(s) for s in scs]
    b.set_steps(ids[0], 5)
    b.set_steps(ids[1], 0)
    b.step(9)
    assert b.steps_left(ids[0]) == 0 and b.steps_left(ids[1]) == 0
    assert b.steps_left(ids[2]) == Batch.UNLIMITED
    pos, vel = alone(scs[0], 5)
    v = b.read(ids[0])
    assert np.array_equal(v["position"][: scs[0].n], pos) and np.array_equal(v["velocity"][: scs[0].n], vel)
    p1 = b.read(ids[1])["position"][: scs[1].n]
    assert np.array_equal(p1, np.asarray(scs[1].init["position"], np.float32).reshape(p1.shape))
    for k in (2, 3):
        pos, _ = alone(scs[k], 9)
        assert np.array_equal(b.read(ids[k])["position"][: scs[k].n], pos), scs[k].name
    b.set_steps(ids[0], 3)
    b.step(4)
    assert b.steps_left(ids[0]) == 0
    pos, vel = alone(scs[0], 8)
    v = b.read(ids[0])
    assert np.array_equal(v["position"][: scs[0].n], pos) and np.array_equal(v["velocity"][: scs[0].n], vel)
    b.close()


def test_read_fields_async_equals_read():
    scs = mix(seed=50)
    b = Batch()
    ids = [b.add(s) for s in scs]
    b.step(4)
    want = {sid: np.array(b.read(sid)["position"]) for sid in ids}
    b.step(3)
    got = b.read_fields(ids, "velocity")
    for sid in ids:
        assert np.array_equal(got[sid], b.read(sid)["velocity"])
    got = b.read_fields(ids, "position")
    for sid, s in zip(ids, scs):
        assert not np.array_equal(got[sid][: s.n], want[sid][: s.n])  # it moved on
        assert np.array_equal(got[sid], b.read(sid)["position"])
    b.close()


def test_pinned_read_fields_one_kernel():
    """Pinned stores are written by one copy kernel, the others by copies:
    either way each store's field equals a full read, and the other fields
    of a pinned store are left alone.  Removing a pinned scene unpins it."""
    scs = mix(seed=51)
    b = Batch()
    ids = [b.add(s) for s in scs]
    for sid in ids[::2]:
        b.pin(sid)
    b.pin(ids[0])  # pinning twice is harmless
    b.step(5)
    before = {sid: np.array(b.scenes[sid].views["velocity"]) for sid in ids}
    got = b.read_fields(ids, "position")
    for sid in ids:
        assert np.array_equal(b.scenes[sid].views["velocity"], before[sid])
    for sid in ids:
        want = np.array(got[sid])
        assert np.array_equal(want, b.read(sid)["position"])
    b.step(2)
    b.unpin(ids[2])
    got = b.read_fields(ids[:3], "velocity")
    for sid in ids[:3]:
        assert np.array_equal(np.array(got[sid]), b.read(sid)["velocity"])
    b.remove(ids[0])
    got = b.read_fields(ids[1:], "position")
    assert all(np.isfinite(v).all() for v in got.values())
    b.close()


def test_async_reads_are_snapshots():
    """An asynchronous read holds the field as of its place in the stream,
    although later substeps run while it is written; an unpinned store is
    refused."""
    from sph import bindings as bnd
    scs = mix(seed=52)
    b = Batch()
    ids = [b.add(s) for s in scs]
    for sid in ids:
        b.pin(sid)
    b.step(2)
    t1 = b.read_fields_async(ids, "position")
    b.step(3)
    b.wait_read(t1)
    snap = {sid: np.array(b.scenes[sid].views["position"]) for sid in ids}
    ref = Batch()
    rids = [ref.add(s) for s in scs]
    ref.step(2)
    want = ref.read_fields(rids, "position")
    for sid, rid in zip(ids, rids):
        assert np.array_equal(snap[sid], want[rid])
    ref.close()
    # several reads in flight, then all waited for
    tickets = [b.read_fields_async(ids, "position")]
    b.step(1)
    tickets.append(b.read_fields_async(ids, "velocity"))
    tickets.append(b.read_fields_async(ids, "position"))
    b.wait_reads()
    got = {sid: (np.array(b.scenes[sid].views["position"]), np.array(b.scenes[sid].views["velocity"])) for sid in ids}
    for sid in ids:
        full = b.read(sid)
        assert np.array_equal(got[sid][0], full["position"])
        assert np.array_equal(got[sid][1], full["velocity"])
    b.unpin(ids[1])
    with pytest.raises(bnd.SphError):
        b.read_fields_async(ids, "position")
    b.close()


def test_solids_with_and_without_planes_in_one_batch():
    """A solid with symmetry planes takes the separate stress and step
    passes; the plane-free solids beside it in the same launches take the
    fused ones.  Each scene equals itself alone."""
    pl = scenes.solid_lattice(5, 5, 7, material="corot", youngs_modulus=3e4, jitter=1e-4, seed=71, clamp_layers=1,
                              name="planes")
    pl.entries = [("symmetry_planes", "3, 2, 3", "float", None) if e[0] == "symmetry_planes" else e
                  for e in pl.entries]
    sp = np.zeros((3, 2, 3), np.float32)
    for k in range(3):
        sp[k, 1, k] = 1.0
    pl.init = dict(pl.init, symmetry_planes=sp)
    scs = [pl] + mix(seed=72)
    b = Batch()
    ids = [b.add(s) for s in scs]
    b.step(12)
    for sc, sid in zip(scs, ids):
        pos, vel = alone(sc, 12)
        v = b.read(sid)
        assert np.array_equal(v["position"][: sc.n], pos), sc.name
        assert np.array_equal(v["velocity"][: sc.n], vel), sc.name
    b.close()


@pytest.mark.parametrize("material", ["fluid", "corot", "svk"])
def test_device_lattice_equals_host_built_scene(material):
    """A lattice scene built on the device (sph_batch_add_lattice) holds the
    same store as the host-built scene uploaded whole, and runs the same."""
    sc = scenes.mix_member(material, 3000, seed=123457, jitter_hash=True, name="dev-" + material)
    a, b = Batch(), Batch()
    ia, ib = a.add_lattice(sc), b.add(sc)
    va, vb = a.read(ia), b.read(ib)
    for f in va:
        assert np.array_equal(va[f], vb[f]), f
    a.step(10)
    b.step(10)
    va, vb = a.read(ia), b.read(ib)
    assert np.array_equal(va["position"], vb["position"]) and np.array_equal(va["velocity"], vb["velocity"])
    a.close()
    b.close()


def test_served_device_built_scenes_equal_alone():
    def make(rng, i):
        mat = scenes.MATERIALS[i % 3]
        return scenes.mix_member(mat, int(rng.integers(800, 3000)), seed=i + 17, jitter_hash=True, name="d%d" % i)
    reqs = poisson_requests(rate=200.0, duration=0.05, make_scene=make, steps_range=(3, 15), seed=9)
    assert len(reqs) >= 5
    stats = Server(budget_bytes=60e6, max_chunk=4).run(reqs, realtime=False)
    assert stats["requests"] == len(reqs)
    for r in reqs:
        pos, vel = alone(r.scene, r.steps)
        assert np.array_equal(r.result["position"], pos), r.scene.name
        assert np.array_equal(r.result["velocity"], vel), r.scene.name
    release(reqs)


def test_ragged_and_empty_scenes_in_a_batch():
    """Scenes with fewer active particles than their capacity, and with none,
    run beside full ones: the ragged scene equals itself alone, the empty
    one is left as it was."""
    full = scenes.wcsph_block(8, 6, 8, seed=61, name="full")
    ragged = scenes.wcsph_block(9, 6, 9, seed=62, name="ragged", pnum=600)
    ragged.init = dict(ragged.init, n=400)
    empty = scenes.wcsph_block(6, 6, 6, seed=63, name="empty")
    empty.init = dict(empty.init, n=0)
    b = Batch()
    ids = [b.add(s) for s in (full, ragged, empty)]
    b.step(10)
    pos, _ = alone(ragged, 10)
    assert np.array_equal(b.read(ids[1])["position"][:400], pos[:400])
    e = b.read(ids[2])["position"]
    assert np.array_equal(e[: empty.n], np.asarray(empty.init["position"], np.float32).reshape(e[: empty.n].shape))
    assert all(b.status(i) == 0 for i in ids)
    b.close()


def test_empty_store_fused_substeps():
    sc = scenes.wcsph_block(6, 6, 6, seed=64)
    sc.init = dict(sc.init, n=0)
    ps = sc.system()
    ps.update_fused(5)
    ps.sync_device_to_host()
    assert ps.status() == 0
    assert np.array_equal(ps.get_fields("position")[0][: sc.n],
                          np.asarray(sc.init["position"], np.float32).reshape(-1, 3))
    ps.close()


def test_batched_writes_equal_host_uploads():
    """sph_batch_write_field_many_async and its several-field form: per-substep inputs (each scene's
    time step and gravity changed before every substep) give the results of
    the same scenes run alone with the same values uploaded through the
    drop-in's blocking sync; bad writes are refused."""
    scs = mix(seed=10)
    steps = 6
    dts = {s.name: [float(s.param("timestep")) * (1.0 + 0.05 * k) for k in range(steps)] for s in scs}
    gs = {s.name: [np.array([0.3 * k, -9.8, 0.1 * k], np.float32) for k in range(steps)] for s in scs}
    b = Batch()
    ids = [b.add(s) for s in scs]
    for k in range(steps):
        for s, sid in zip(scs, ids):
            v = b.scenes[sid].views
            v["timestep"][...] = dts[s.name][k]
            v["gravity"][...] = gs[s.name][k]
        if k % 2:
            # both fields in one call (sph_batch_write_fields_many_async)
            b.write_fields_async(ids, "timestep", "gravity")
        else:
            b.write_fields_async(ids, "timestep")
            b.write_fields_async(ids, "gravity")
        # the stores may change at once: the next write overwrites them
        for sid in ids:
            b.scenes[sid].views["timestep"][...] = -1.0
        b.step(1)
    got = {s.name: np.array(b.read(sid)["position"][: s.n]) for s, sid in zip(scs, ids)}
    with pytest.raises(Exception, match="gridres"):
        b.write_fields_async(ids[:1], "gridres")
    with pytest.raises(Exception, match="gridres"):
        b.write_fields_async(ids[:1], "timestep", "gridres")
    b.close()
    for s in scs:
        ps = s.system()
        if s.material != "fluid":
            ps.call_for_all_particles("init_original_position")
            ps.compute_particle_bins()
            ps.call_for_all_particles("compute_original_density")
        for k in range(steps):
            ps.set_fields(timestep=dts[s.name][k], gravity=gs[s.name][k])
            ps.update_fused(1)
        ps.sync_device_to_host()
        assert np.array_equal(ps.get_fields("position")[0][: s.n], got[s.name]), s.name
        ps.close()
