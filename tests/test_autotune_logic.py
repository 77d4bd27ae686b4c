"""The launch-shape autotuner's host logic on the CPU, over a stand-in
batch whose substep time depends on the shape: every candidate is applied
and timed after a warm-up substep, the fastest wins, and the scratch batch
is closed."""
import sph.autotune as autotune


class Clock(object):
    now = 0.0

    @staticmethod
    def perf_counter():
        return Clock.now


def test_tuner_times_every_candidate_and_picks_the_fastest(monkeypatch):
    log = []

    class FakeBatch(object):
        def __init__(self):
            self.shape = None
            self.added = 0
            self.closed = False
            log.append(self)

        def add(self, scene):
            self.added += 1

        def tune(self, block, pair, cap):
            self.shape = (block, pair, cap)

        def step(self, n):
            block, pair, cap = self.shape
            # fastest at (256, 128, 0); warm-up substeps are as slow as the rest
            Clock.now += n * (1.0 + abs(block - 256) / 1000.0 + abs(pair - 128) / 500.0 + cap / 1e5)

        def synchronize(self):
            pass

        def close(self):
            self.closed = True

    monkeypatch.setattr(autotune, "Batch", FakeBatch)
    monkeypatch.setattr(autotune, "time", Clock)
    cands = list(autotune.candidates(sms=152))
    assert len(cands) == 36 and (256, 128, 0) in cands and (512, 64, 8 * 152) in cands
    best, secs, table = autotune.tune(["a", "b", "c"], steps=3, cands=cands)
    assert best == (256, 128, 0) and secs == 1.0
    assert [c for c, _ in table] == cands
    assert log[0].added == 3 and log[0].closed
