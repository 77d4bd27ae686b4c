"""Double-precision tests of the reference restated in FP32.

- The cube band (APPLY_CUBE_BOUNDS, common.cl:37-43): the device compares a
  float position against the floats just outside -2 + (double)0.2f and
  2 - (double)0.2f (SPH_CUBE_BAND_LO/HI in kernels_fluid.cuh) instead of
  converting it to double.
- The symmetry-plane distance floor ((double)jd < 1.0e-5 in the SYMMETRY
  blocks, e.g. common.cl:647-686): jd <= the float just below 1e-5
  (SPH_PLANE_EPS_BELOW in kernels_common.cuh).

For every float near the bounds both forms agree."""
import numpy as np

LO = np.float32(float.fromhex("-0x1.cccccep+0"))
HI = np.float32(float.fromhex("0x1.cccccep+0"))


def _around(x, count=20000):
    out = [np.float32(x)]
    up = dn = np.float32(x)
    for _ in range(count):
        up = np.nextafter(up, np.float32(np.inf))
        dn = np.nextafter(dn, np.float32(-np.inf))
        out += [up, dn]
    return np.array(out, dtype=np.float32)


def test_band_bounds_equal_double_tests():
    band = float(np.float32(0.2))
    for p in np.concatenate([_around(-1.8), _around(1.8), np.float32([-np.inf, np.inf, 0.0, -2.0, 2.0])]):
        d = float(p)
        assert (d < -2.0 + band) == bool(p <= LO), p
        assert (d > 2.0 - band) == bool(p >= HI), p


def test_bounds_lie_between_floats():
    band = float(np.float32(0.2))
    assert float(LO) < -2.0 + band < float(np.nextafter(LO, np.float32(np.inf)))
    assert float(np.nextafter(HI, np.float32(-np.inf))) < 2.0 - band < float(HI)


EPS_BELOW = np.float32(float.fromhex("0x1.4f8b58p-17"))


def test_plane_floor_equals_double_test():
    for jd in np.concatenate([_around(1.0e-5), np.float32([0.0, np.inf])]):
        assert (float(jd) < 1.0e-5) == bool(jd <= EPS_BELOW), jd
    assert float(EPS_BELOW) < 1.0e-5 < float(np.nextafter(EPS_BELOW, np.float32(np.inf)))
