"""Autotuner for the batched form's launch shape.

Times a scratch copy of a scene set over candidate launch shapes -- threads
per block for the particle/cell kernels and for the pair kernels, and the
persistent-grid cap (blocks per launch, as multiples of the SM count) --
and returns the fastest.  The cell size stays the reference's (h: the cell
tables are psdata fields whose shape the store fixes), and the counting
sort has one pass (its key is the cell index).
"""
import itertools
import time

from .batch import Batch

DEFAULT_SMS = 152


def candidates(sms=DEFAULT_SMS):
    for block, pair, cap in itertools.product((128, 256, 512), (64, 128, 256), (0, 2 * sms, 4 * sms, 8 * sms)):
        yield block, pair, cap


def tune(scenes, steps=4, cands=None, verbose=False):
    """Returns ((block, pair_block, grid_cap), seconds per substep, table)."""
    b = Batch()
    try:
        for s in scenes:
            b.add(s)
        table = []
        for c in (cands or list(candidates())):
            b.tune(*c)
            b.step(1)  # capture + warm
            b.synchronize()
            t0 = time.perf_counter()
            b.step(steps)
            b.synchronize()
            dt = (time.perf_counter() - t0) / steps
            table.append((c, dt))
            if verbose:
                print("tune", c, "%.3f ms" % (dt * 1e3))
        best = min(table, key=lambda x: x[1])
        return best[0], best[1], table
    finally:
        b.close()
