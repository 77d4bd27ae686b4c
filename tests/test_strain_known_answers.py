"""Uniaxial stretch of a corotational bar: the analytic known answers of the
reference's strain test (scripts/straintest.py), driven by its recipe.

The reference's StrainTest (straintest.py:18-247) constrains the two end
faces of a bar to planes normal to the axis (init_plane_constraints,
:96-111), moves the planes apart a little every substep and then holds
them (init_run_path, :119-147), and per substep uploads the planes, runs
StrainSolid.update() -- bins, density, rotations and strains, stresses,
forces, step (systems.py:194-204) -- and then apply_plane_constraints
(run, :198-246).  Here the bar (21 x 9 x 9 particles at 0.01 m, h = 0.02
m, E = 1e5 Pa, nu = 0.3, the conf's viscosity 6e-5) is stretched by
eps = 1% over 200 substeps and held for 2,300.  In the bar's middle
(|x - centre| <= 0.05 m, |y|, |z| <= 0.015 m from the axis) the mean
strain and stress must give the linear-elastic answers:
  eps_xx ~ eps           (within 10%: SPH gradient deficiency, end effects)
  eps_yy / eps_xx ~ -nu  (within 0.03)
  sig_xx ~ E eps_xx      (within 5%)
  sig_yy ~ 0             (within 5% of E eps)
Measured with the C oracle: eps_xx = 0.955 eps, eps_yy / eps_xx = -0.309,
sig_xx = 0.99 E eps_xx, sig_yy = -0.017 E eps.

The CPU test runs the recipe on the oracle (the reference's algorithm);
the GPU test runs it through the library's named kernels with the
plane-constraint uploads of the reference's driver, checks the same known
answers, and checks the final state against the oracle's.
"""
import os

import numpy as np
import pytest

from helpers import host_store, max_rel, oracle_of, rel_err
from sph import scenes

E, NU, EPS = 1e5, 0.3, 0.01
RAMP, HOLD = 200, 2300


def bar():
    sc = scenes.solid_lattice(21, 9, 9, spacing=0.01, h=0.02, material="corot", youngs_modulus=E, poisson=NU,
                              gravity=(0.0, 0.0, 0.0), dt=5e-5, clamp_layers=0, jitter=0.0, seed=0, name="strain-bar")
    # two constraint planes (the reference conf's plane_constraints is 3, 2, 4)
    sc.entries = [("plane_constraints", "3, 2, 2", "float", None) if e[0] == "plane_constraints" else e
                  for e in sc.entries]
    pos = sc.init["position"]
    lo, hi = float(pos[:, 0].min()), float(pos[:, 0].max())
    pcp = np.zeros(sc.n, np.uint32)
    pcp[pos[:, 0] == lo] = 1 << 0
    pcp[pos[:, 0] == hi] = 1 << 1
    sc.init["plane_constraints_particles"] = pcp
    centre = pos.astype(np.float64).mean(axis=0)
    d = np.abs(pos - centre)
    middle = (d[:, 0] <= 0.05) & (d[:, 1] <= 0.015) & (d[:, 2] <= 0.015)
    return sc, lo, hi, middle


def planes_at(step, lo, hi):
    """The two planes (point, normal) of substep `step`: the end faces moved
    apart linearly over RAMP substeps to eps of the length, then held."""
    f = min(1.0, (step + 1) / RAMP)
    half = 0.5 * (hi - lo) * EPS * f
    pc = np.zeros((2, 2, 3), np.float32)
    pc[0, 0, 0], pc[0, 1, 0] = lo - half, 1.0
    pc[1, 0, 0], pc[1, 1, 0] = hi + half, 1.0
    return pc


def check_known_answers(strain, stress):
    exx, eyy, ezz = (float(x) for x in strain.mean(axis=0)[:3])
    sxx, syy = (float(x) for x in stress.mean(axis=0)[:2])
    assert abs(exx / EPS - 1.0) <= 0.10, exx / EPS
    assert abs(eyy / exx + NU) <= 0.03 and abs(ezz / exx + NU) <= 0.03, (eyy / exx, ezz / exx)
    assert abs(sxx / (E * exx) - 1.0) <= 0.05, sxx / (E * exx)
    assert abs(syy) <= 0.05 * E * EPS, syy / (E * EPS)
    return exx / EPS, eyy / exx, sxx / (E * exx), syy / (E * EPS)


def run_oracle(sc, lo, hi):
    _, v = host_store(sc)
    o = oracle_of(v, "f32", nthreads=os.cpu_count() or 4)
    o.setup_solid()
    for s in range(RAMP + HOLD):
        o.a["plane_constraints"][...] = planes_at(s, lo, hi)
        o.substep("corot")
        o.call("apply_plane_constraints")
    return o


def test_uniaxial_known_answers_oracle():
    sc, lo, hi, middle = bar()
    o = run_oracle(sc, lo, hi)
    n = sc.n
    got = check_known_answers(o.a["strain"][:n][middle], o.a["stress"][:n][middle])
    print("oracle: eps_xx/eps %.3f, eps_yy/eps_xx %.3f, sig_xx/(E eps_xx) %.3f, sig_yy/(E eps) %.3f" % got)


@pytest.mark.gpu
def test_uniaxial_known_answers_named_kernels():
    from sph.systems import StrainSolid
    sc, lo, hi, middle = bar()
    ss = StrainSolid(spec=sc.spec, kernel_files=sc.kernel_files)
    ss.init(**sc.init)
    ss.setup()
    for s in range(RAMP + HOLD):
        ss.set_fields(True, plane_constraints=planes_at(s, lo, hi))
        ss.sync_fields_host_to_device("plane_constraints")
        ss.update()
        ss.call_for_all_particles("apply_plane_constraints")
    ss.sync_device_to_host()
    n = sc.n
    strain, stress = ss.get_fields("strain", "stress")
    got = check_known_answers(strain[:n][middle], stress[:n][middle])
    print("GPU: eps_xx/eps %.3f, eps_yy/eps_xx %.3f, sig_xx/(E eps_xx) %.3f, sig_yy/(E eps) %.3f" % got)
    o = run_oracle(sc, lo, hi)
    assert rel_err(ss.get_fields("position")[0][:n], o.a["position"][:n]) <= 1e-5
    assert max_rel(strain[:n][middle], o.a["strain"][:n][middle]) <= 1e-3
    assert ss.status() == 0
    ss.close()
