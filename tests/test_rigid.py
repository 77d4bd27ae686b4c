"""Rigid bodies (an extension: the reference's bodies are only fixed or
kinematic).  A body whose body_dynamic is 2 moves rigidly under the sum of
its particles' forces; see kernels_rigid.cuh and oracle_rigid_step.

No reference implementation exists, so parity is pinned by physics on the
FP64 oracle -- momentum and angular momentum conservation, rigidity,
free fall -- and the CUDA path is checked against the oracle."""
import numpy as np
import pytest

from helpers import host_store, oracle_of, rel_err
from sph import free_data_cpu, scenes


def _oracle(scene, prec="f64"):
    ps, views = host_store(scene)
    o = oracle_of(views, prec)
    free_data_cpu(ps)
    return o


def _momenta(o, body_mask):
    m = float(o.state.mass)
    x = o.a["position"][body_mask].astype(np.float64)
    v = o.a["velocity"][body_mask].astype(np.float64)
    c = x.mean(axis=0)
    return m * v.sum(axis=0), m * np.cross(x - c, v).sum(axis=0), c


def _pair_dists(x):
    x = np.asarray(x, dtype=np.float64)
    d = x[:, None, :] - x[None, :, :]
    return np.sqrt((d * d).sum(-1))


def free_ball(**kw):
    args = dict(radius=0.035, spacing=0.01, center=(0.2, 0.2, 0.2), velocity=(0.1, 0.0, 0.05),
                omega=(0.0, 1.0, 3.0), gravity=(0.0, 0.0, 0.0), viscosity=0.0, jitter=0.0)
    args.update(kw)
    return scenes.rigid_body_scene(**args)


def test_oracle_free_body_conserves_momentum_and_shape():
    sc = free_ball()
    o = _oracle(sc)
    body = np.asarray(sc.init["body_number"]) == 1
    P0, L0, c0 = _momenta(o, body)
    d0 = _pair_dists(o.a["position"][body])
    steps, dt = 200, float(o.state.timestep)
    o.run("fluid", steps)
    P1, L1, c1 = _momenta(o, body)
    assert np.linalg.norm(P1 - P0) <= 1e-9 * np.linalg.norm(P0)
    assert np.linalg.norm(L1 - L0) <= 1e-6 * np.linalg.norm(L0)
    # the centre moves uniformly; the shape does not change
    assert np.allclose(c1, c0 + np.array([0.1, 0.0, 0.05]) * steps * dt, rtol=0, atol=1e-9)
    assert np.max(np.abs(_pair_dists(o.a["position"][body]) - d0)) <= 1e-12
    # and it turned: the angular velocity it was given, about 3 rad/s * 0.02 s
    st = o.rigid_state[0]
    assert st[0] == 2.0 and abs(np.degrees(2 * np.arccos(min(1.0, st[10]))) - np.degrees(0.02 * np.sqrt(10))) < 0.05


def test_oracle_free_fall():
    sc = free_ball(gravity=(0.0, -9.8, 0.0), omega=(0.0, 0.0, 0.0), velocity=(0.0, 0.0, 0.0))
    o = _oracle(sc)
    body = np.asarray(sc.init["body_number"]) == 1
    steps, dt = 100, float(o.state.timestep)
    g = float(np.float32(9.8))  # the store's float gravity
    o.run("fluid", steps)
    v = o.a["velocity"][body].astype(np.float64)
    assert np.allclose(v, [0.0, -g * steps * dt, 0.0], rtol=0, atol=1e-10)
    # semi-implicit Euler: y(N) = y0 - g dt^2 N (N + 1) / 2
    st = o.rigid_state[0]
    y0 = float(np.mean(np.asarray(sc.init["position"], np.float64)[body, 1]))
    assert abs(st[5] - (y0 - g * dt * dt * steps * (steps + 1) / 2)) < 1e-12


def test_oracle_ball_in_fluid_stays_rigid_and_fluid_moves():
    sc = scenes.rigid_body_scene(radius=0.03, fluid=(10, 8, 10), center=(0.05, 0.13, 0.05))
    o = _oracle(sc, "f32")
    body = np.asarray(sc.init["body_number"]) == 1
    d0 = _pair_dists(o.a["position"][body])
    x0 = o.a["position"].copy()
    o.run("fluid", 50)
    assert np.max(np.abs(_pair_dists(o.a["position"][body]) - d0)) <= 2e-6  # float positions
    assert np.max(np.abs(o.a["position"][~body] - x0[~body])) > 1e-5
    assert np.all(np.isfinite(o.a["position"]))


# ---- the CUDA path --------------------------------------------------------------------


def _gpu_run(scene, steps, named=False):
    ps = scene.system()
    if named:
        for _ in range(steps):
            ps.compute_particle_bins()
            ps.call_for_all_particles("compute_density")
            ps.call_for_all_particles("compute_forces_fluids")
            ps.call_for_all_particles("step_forward")
    else:
        ps.update_fused(steps)
    ps.sync_device_to_host()
    out = {k: np.array(ps.get_fields(k)[0][: scene.n]) for k in ("position", "velocity")}
    assert ps.status() == 0
    ps.close()
    return out


@pytest.mark.gpu
def test_gpu_rigid_ball_in_fluid_matches_oracle():
    sc = scenes.rigid_body_scene(radius=0.03, fluid=(10, 8, 10), center=(0.05, 0.13, 0.05))
    steps = 40
    g = _gpu_run(sc, steps)
    o = _oracle(sc, "f32")
    o.run("fluid", steps)
    assert rel_err(g["position"], o.a["position"][: sc.n]) < 1e-5
    assert rel_err(g["velocity"], o.a["velocity"][: sc.n]) < 1e-3
    body = np.asarray(sc.init["body_number"]) == 1
    d0 = _pair_dists(np.asarray(sc.init["position"])[body])
    assert np.max(np.abs(_pair_dists(g["position"][body]) - d0)) <= 2e-6


@pytest.mark.gpu
def test_gpu_rigid_free_body_conserves_momentum():
    sc = free_ball()
    body = np.asarray(sc.init["body_number"]) == 1
    g = _gpu_run(sc, 200)
    o = _oracle(sc)
    o.run("fluid", 200)
    # FP64 body state, FP32 particles: the two runs agree to float rounding
    assert rel_err(g["position"], o.a["position"][: sc.n]) < 1e-6
    m = float(o.state.mass)
    P = m * g["velocity"][body].astype(np.float64).sum(axis=0)
    assert np.linalg.norm(P - m * body.sum() * np.array([0.1, 0.0, 0.05])) <= 1e-5 * np.linalg.norm(P)


@pytest.mark.gpu
def test_gpu_rigid_named_kernels_equal_fused():
    sc = scenes.rigid_body_scene(radius=0.03, fluid=(8, 6, 8), center=(0.04, 0.11, 0.04))
    a = _gpu_run(sc, 12)
    b = _gpu_run(sc, 12, named=True)
    assert np.array_equal(a["position"], b["position"]) and np.array_equal(a["velocity"], b["velocity"])


@pytest.mark.gpu
def test_gpu_rigid_scene_in_batch_equals_alone():
    from sph.batch import Batch
    rig = scenes.rigid_body_scene(radius=0.03, fluid=(8, 6, 8), center=(0.04, 0.11, 0.04), name="rig")
    other = scenes.wcsph_block(9, 6, 9, seed=5, name="f")
    free = free_ball(name="free")
    b = Batch()
    ids = [b.add(s) for s in (other, rig, free)]
    b.step(15)
    for sc, sid in ((rig, ids[1]), (free, ids[2])):
        want = _gpu_run(sc, 15)
        v = b.read(sid)
        assert np.array_equal(v["position"][: sc.n], want["position"]), sc.name
        assert np.array_equal(v["velocity"][: sc.n], want["velocity"]), sc.name
    b.close()


def three_balls(**kw):
    args = dict(spacing=0.01, gravity=(0.0, 0.0, 0.0), viscosity=0.0, jitter=0.0,
                balls=[(0.025, (0.1, 0.2, 0.2), (0.2, 0.0, 0.0), (0.0, 0.0, 2.0)),
                       (0.035, (0.3, 0.2, 0.2), (0.0, 0.1, 0.0), (1.0, 0.0, 0.0)),
                       (0.03, (0.2, 0.3, 0.1), (0.0, 0.0, -0.1), (0.0, 3.0, 0.0))])
    args.update(kw)
    return scenes.rigid_body_scene(**args)


def test_oracle_several_bodies_move_independently():
    sc = three_balls()
    o = _oracle(sc)
    bn = np.asarray(sc.init["body_number"])
    d0 = [_pair_dists(o.a["position"][bn == b]) for b in (1, 2, 3)]
    P0 = [_momenta(o, bn == b)[0] for b in (1, 2, 3)]
    o.run("fluid", 100)
    for b in (1, 2, 3):
        P1, _, _ = _momenta(o, bn == b)
        assert np.linalg.norm(P1 - P0[b - 1]) <= 1e-9 * np.linalg.norm(P0[b - 1])
        assert np.max(np.abs(_pair_dists(o.a["position"][bn == b]) - d0[b - 1])) <= 1e-12
    assert np.all(o.rigid_state[:, 0] == 2.0)


@pytest.mark.gpu
def test_gpu_several_bodies_match_oracle():
    """Three balls dropping onto a fluid block (surface at y = 0.065) within
    the smoothing length: each body's reduction is its own."""
    sc = three_balls(fluid=(12, 6, 12), gravity=(0.0, -9.8, 0.0), viscosity=0.2, jitter=1e-4,
                     balls=[(0.02, (0.03, 0.09, 0.03), (0.0, -0.5, 0.0), (0.0, 0.0, 2.0)),
                            (0.025, (0.09, 0.095, 0.04), (0.0, -0.3, 0.1), (1.0, 0.0, 0.0)),
                            (0.02, (0.06, 0.09, 0.1), (0.1, -0.4, 0.0), (0.0, 3.0, 0.0))])
    steps = 40
    g = _gpu_run(sc, steps)
    o = _oracle(sc, "f32")
    o.run("fluid", steps)
    assert rel_err(g["position"], o.a["position"][: sc.n]) < 1e-5
    assert rel_err(g["velocity"], o.a["velocity"][: sc.n]) < 1e-3
    bn = np.asarray(sc.init["body_number"])
    x0 = np.asarray(sc.init["position"])
    for b in (1, 2, 3):
        d0 = _pair_dists(x0[bn == b])
        assert np.max(np.abs(_pair_dists(g["position"][bn == b]) - d0)) <= 2e-6
    assert np.max(np.abs(g["position"][bn == 0] - x0[bn == 0])) > 1e-5  # the fluid felt them
