"""The serving loop's host logic on the CPU, over a stand-in batch that
counts substeps: first-come-first-served admission, the HBM budget and the
resident-particle cap (with the lone-request exception), quotas that stop
each scene after exactly its requested substeps, and continuous batching
(a request that arrives while others run joins the next chunk)."""
import types

import pytest

import sph.serving as serving


class FakeClock(object):
    """The server's clock: a substep takes 10 ms of virtual time."""
    now = 0.0

    @staticmethod
    def perf_counter():
        return FakeClock.now

    @staticmethod
    def sleep(s):
        FakeClock.now += s


class FakeBatch(object):
    """Counts each scene's substeps as the device would: a scene advances
    min(chunk, quota) substeps per step() and then idles."""
    events = []

    def __init__(self):
        self.scenes = {}
        self.next = 0
        self.closed = False

    # the static builders Server.prepare calls
    @staticmethod
    def host_store(scene):
        return ("host", scene.name)

    @staticmethod
    def lattice_store(scene):
        return ("lattice", scene.name)

    @staticmethod
    def scene_bytes(scene, host):
        return 1000 * scene.n

    def tune(self, *args):
        pass

    @property
    def bytes(self):
        return sum(1000 * s["scene"].n for s in self.scenes.values())

    def _add(self, scene):
        sid = self.next
        self.next += 1
        self.scenes[sid] = {"scene": scene, "quota": None, "done": 0}
        FakeBatch.events.append(("add", scene.name, self.bytes, sum(s["scene"].n for s in self.scenes.values())))
        return sid

    def add(self, scene, ps=None):
        assert ps == ("host", scene.name)
        return self._add(scene)

    def add_lattice(self, scene, ps=None):
        assert ps == ("lattice", scene.name)
        return self._add(scene)

    def set_steps(self, sid, n):
        self.scenes[sid]["quota"] = int(n)

    def step(self, n):
        FakeBatch.events.append(("step", n, sorted(s["scene"].name for s in self.scenes.values())))
        FakeClock.now += 0.01 * n
        for s in self.scenes.values():
            k = min(n, s["quota"])
            s["done"] += k
            s["quota"] -= k

    def synchronize(self):
        pass

    def status(self, sid):
        return 0

    def read(self, sid):
        s = self.scenes[sid]
        n = s["scene"].n
        return {"position": [[float(s["done"])] * 3] * n, "velocity": [[0.0] * 3] * n}

    def remove(self, sid):
        s = self.scenes.pop(sid)
        FakeBatch.events.append(("remove", s["scene"].name, s["done"]))

    def close(self):
        self.closed = True


def scene(name, n, gen=False):
    return types.SimpleNamespace(name=name, n=n, gen=gen)


@pytest.fixture
def fake(monkeypatch):
    FakeBatch.events = []
    FakeClock.now = 0.0
    monkeypatch.setattr(serving, "Batch", FakeBatch)
    monkeypatch.setattr(serving, "time", FakeClock)
    return FakeBatch


def test_each_request_runs_exactly_its_substeps(fake):
    reqs = [serving.Request(i, scene("s%d" % i, 100 + i, gen=i % 2 == 0), steps, arrival)
            for i, (steps, arrival) in enumerate([(7, 0.0), (30, 0.0), (3, 0.01), (12, 0.02), (1, 0.5)])]
    stats = serving.Server(budget_bytes=1e12, max_chunk=5).run(reqs, realtime=False)
    done = {e[1]: e[2] for e in fake.events if e[0] == "remove"}
    assert done == {"s%d" % r.id: r.steps for r in reqs}
    assert all(r.result["position"][0][0] == float(r.steps) for r in reqs)
    assert stats["requests"] == 5 and stats["status_failed"] == 0
    assert all(r.done >= r.admitted >= r.arrival for r in reqs)
    assert stats["particle_steps"] == sum(r.scene.n * r.steps for r in reqs)


def test_admission_is_first_come_first_served_within_budget_and_cap(fake):
    sizes = [400, 300, 500, 200, 100, 600]
    reqs = [serving.Request(i, scene("s%d" % i, n), 10, 0.0) for i, n in enumerate(sizes)]
    srv = serving.Server(budget_bytes=1000 * 900, max_chunk=4, max_particles=800)
    srv.run(reqs, realtime=False)
    adds = [e for e in fake.events if e[0] == "add"]
    assert [e[1] for e in adds] == ["s%d" % i for i in range(len(sizes))]  # arrival order
    for _, name, bytes_after, resident_after in adds:
        assert bytes_after <= 1000 * 900 and resident_after <= 800
    # s2 (500 particles) waited for s0 and s1 to finish; s3 and s4 queued
    # behind it although they fit (first come, first served)
    order = [(e[0], e[1]) for e in fake.events if e[0] in ("add", "remove")]
    assert order.index(("add", "s2")) > order.index(("remove", "s1"))
    assert order.index(("add", "s3")) > order.index(("add", "s2"))


def test_lone_request_larger_than_budget_still_runs(fake):
    reqs = [serving.Request(0, scene("big", 5000), 4, 0.0), serving.Request(1, scene("small", 10), 4, 0.0)]
    stats = serving.Server(budget_bytes=1000, max_chunk=8, max_particles=100).run(reqs, realtime=False)
    names = [e[1] for e in fake.events if e[0] == "remove"]
    assert names == ["big", "small"]  # the small one waited: first come, first served
    assert stats["peak_resident"] == 1


def test_late_arrivals_join_running_chunks(fake):
    """A request that arrives while another runs is admitted at the next
    chunk boundary and shares the following chunks with it."""
    reqs = [serving.Request(0, scene("long", 50), 40, 0.0), serving.Request(1, scene("late", 20), 6, 0.12)]
    serving.Server(budget_bytes=1e12, max_chunk=5).run(reqs, realtime=True)
    steps = [e for e in fake.events if e[0] == "step"]
    assert steps[0][2] == ["long"] and any(e[2] == ["late", "long"] for e in steps)
    removed = [e[1] for e in fake.events if e[0] == "remove"]
    assert removed == ["late", "long"]  # the short request finished first
    late = reqs[1]
    assert 0.12 <= late.admitted <= 0.12 + 0.05 + 1e-9  # at the first chunk boundary after arriving
    assert late.done - late.admitted == pytest.approx(0.10)  # two chunks of 5 substeps
