"""Error of precision variants of the 8,000-particle dam break against the
FP64 run, every 100 substeps up to 1,000 (a script, not a test: under a
minute on 8 host cores).

    python tests/precision_variants.py [substeps]

Every variant is the reference's algorithm (the C oracle) on the same scene;
they differ only in what is kept in FP32:
  fp32             the reference's algorithm in FP32 (forces, state)
  fp32+fp64state   FP32 forces, position and velocity integrated and kept in
                   FP64 (the forces see the state rounded to FP32)
  fp64+fp32pos     FP64 everything, but the forces see positions rounded to
                   FP32 each substep: the error that storing positions in
                   the store's FP32 fields alone causes
and, for the FP32 run, how the error is spread: the share of the squared
error carried by the 1% of particles that moved farthest from the FP64 run,
and the relative L2 error over the other 99%.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, os.path.join(ROOT, "opencl-sph_gb300"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

from helpers import host_store, rel_err  # noqa: E402
from oracle.oracle import OracleScene  # noqa: E402
from sph import scenes  # noqa: E402


def main(steps=1000, threads=os.cpu_count() or 4):
    sc = scenes.wcsph_block(20, 20, 20, seed=0, name="dam-8k")
    _, v = host_store(sc)
    n = sc.n
    o64 = OracleScene(v, "f64", nthreads=threads)
    o32 = OracleScene(v, "f32", nthreads=threads)
    ofs = OracleScene(v, "f32", nthreads=threads)   # FP32 forces, FP64 state
    ofp = OracleScene(v, "f64", nthreads=threads)   # FP64 forces on FP32-rounded positions
    m = float(v["mass"][0])
    dt = float(v["timestep"][0])
    g = np.array(v["gravity"][:3], np.float64)
    wb = np.array(v["wallbounds"], np.float64).reshape(3, 2)
    xs = ofs.a["position"][:n].astype(np.float64)
    vs = ofs.a["velocity"][:n].astype(np.float64)
    xp = ofp.a["position"][:n].copy()
    vp = ofp.a["velocity"][:n].copy()

    def step64(x, vel, f):
        # step_forward (common.cl:691-722) with the reflective box, in FP64
        vel += dt * (f / m + g)
        x += dt * vel
        for ax in range(3):
            lo, hi = wb[ax]
            below, above = x[:, ax] < lo, x[:, ax] > hi
            x[below, ax] = 2 * lo - x[below, ax]
            vel[below, ax] *= -1
            x[above, ax] = 2 * hi - x[above, ax]
            vel[above, ax] *= -1

    forces = ("compute_particle_bins", "compute_density", "compute_forces_fluids")
    t0 = time.time()
    print("substep  fp32       fp32+fp64state  fp64+fp32pos  | fp32: top-1% share  other 99%")
    for s in range(1, steps + 1):
        o64.substep("fluid")
        o32.substep("fluid")
        for k in forces:
            ofs.call(k)
        step64(xs, vs, ofs.a["force"][:n].astype(np.float64))
        ofs.a["position"][:n] = xs.astype(np.float32)
        ofs.a["velocity"][:n] = vs.astype(np.float32)
        ofp.a["position"][:n] = xp.astype(np.float32).astype(np.float64)
        ofp.a["velocity"][:n] = vp
        for k in forces:
            ofp.call(k)
        step64(xp, vp, ofp.a["force"][:n].copy())
        if s % 100 == 0:
            ref = o64.a["position"][:n]
            d2 = np.sum((o32.a["position"][:n] - ref) ** 2, axis=1)
            order = np.argsort(d2)
            keep = order[: int(0.99 * n)]
            top = float(d2[order[int(0.99 * n):]].sum() / d2.sum())
            bulk = rel_err(o32.a["position"][:n][keep], ref[keep])
            print("%7d  %.3e  %.3e       %.3e     | %.2f                %.3e   (%.0f s)"
                  % (s, rel_err(o32.a["position"][:n], ref), rel_err(xs, ref), rel_err(xp, ref), top, bulk,
                     time.time() - t0), flush=True)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 1000)
