"""Host-side scene builders: the counter-based lattice jitter that the
device builder (sph_batch_add_lattice) reproduces."""
import numpy as np

from sph import scenes

MASK = (1 << 64) - 1


def _splitmix64_py(x):
    """splitmix64 written out with Python integers (the check on the
    vectorised numpy form)."""
    z = (x + 0x9E3779B97F4A7C15) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


def test_splitmix64_matches_integer_form():
    xs = [0, 1, 2, 12345, (1 << 32) + 7, (1 << 63) + 11, MASK]
    got = scenes.splitmix64(np.array(xs, dtype=np.uint64))
    assert [int(v) for v in got] == [_splitmix64_py(x) for x in xs]


def test_hash_jitter_bounds_and_determinism():
    j = scenes.hash_jitter(5000, seed=42, jitter=1e-4)
    assert j.shape == (5000, 3) and np.all(np.abs(j) <= 1e-4)
    assert abs(j.mean()) < 5e-6 and np.array_equal(j, scenes.hash_jitter(5000, 42, 1e-4))
    assert not np.array_equal(j, scenes.hash_jitter(5000, 43, 1e-4))
    # the first values, from the integer form
    u = [(_splitmix64_py(42 * (1 << 32) + c) >> 11) * 2.0 ** -53 for c in range(6)]
    assert np.array_equal(j.ravel()[:6], [1e-4 * (2.0 * v - 1.0) for v in u])


def test_jitter_hash_scenes_carry_their_lattice():
    f = scenes.wcsph_block(6, 5, 4, seed=7, jitter_hash=True)
    assert f.gen["nx"] == 6 and f.gen["clamp_layers"] == 0
    pos = scenes.lattice(6, 5, 4, 0.01, origin=f.gen["origin"], jitter=1e-4, hash_seed=7)
    assert np.array_equal(f.init["position"], pos)
    s = scenes.solid_lattice(4, 4, 8, material="svk", clamp_layers=1, jitter=1e-4, seed=3, jitter_hash=True)
    assert s.gen["clamp_layers"] == 1 and s.gen["identity_rotation"] == 1
    assert scenes.wcsph_block(6, 5, 4, seed=7).gen is None
