"""Served form: a request loop with continuous batching.

Requests (a scene and a substep count) arrive over time.  The server keeps
one :class:`~sph.batch.Batch` on the device; whenever it is between
chunks it admits every arrived request whose store fits in the HBM budget
(first come, first served), advances all resident scenes together by a
chunk of substeps -- no longer than the shortest remaining request, so no
scene overshoots its count -- and retires finished scenes, reading their
results back and freeing their memory for the next admissions.  Scenes
that arrive while others run join at the next chunk boundary, and their
work shares the same launches; a scene's result is the same as when it
runs alone (the batch kernels treat scenes independently).

Reports p50/p99 time to completion (arrival -> result on the host) beside
aggregate particle-steps/s.
"""
import collections
import time

import numpy as np

from . import free_data_cpu
from .batch import Batch


class Request(object):
    def __init__(self, rid, scene, steps, arrival):
        self.id = rid
        self.scene = scene
        self.steps = int(steps)
        self.arrival = float(arrival)
        self.host = None       # prebuilt host store (the request payload)
        self.bytes = 0
        self.admitted = None
        self.done = None
        self.remaining = self.steps
        self.result = None

    @property
    def work(self):
        return self.scene.n * self.steps


def poisson_requests(rate, duration, make_scene, steps_range, seed=0):
    """Poisson arrivals at `rate`/s over `duration` s; `make_scene(rng, i)`
    builds each request's scene; steps uniform in steps_range."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        out.append(Request(len(out), make_scene(rng, len(out)), rng.integers(steps_range[0], steps_range[1] + 1), t))
    return out


class Server(object):
    def __init__(self, budget_bytes=150e9, max_chunk=50, keep_results=True, tune=None):
        self.budget = float(budget_bytes)
        self.max_chunk = int(max_chunk)
        self.keep = keep_results
        self.tune = tune

    def prepare(self, requests):
        """Builds each request's host store ahead of its arrival."""
        for r in requests:
            if r.host is None:
                r.host = Batch.host_store(r.scene)
                r.bytes = Batch.scene_bytes(r.scene, r.host)

    def run(self, requests, realtime=True):
        """Serves `requests` (arrival times in seconds from the start).
        With realtime=False arrivals are taken as already due when the
        server is idle (no sleeping), i.e. time is compressed."""
        self.prepare(requests)
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        batch = Batch()
        if self.tune:
            batch.tune(*self.tune)
        active = {}
        t0 = time.perf_counter()
        skew = 0.0

        def clock():
            return time.perf_counter() - t0 + skew

        chunks = 0
        peak_resident = 0
        peak_bytes = 0
        while pending or active:
            now = clock()
            while pending and pending[0].arrival <= now:
                r = pending[0]
                if active and batch.bytes + r.bytes > self.budget:
                    break
                pending.popleft()
                sid = batch.add(r.scene, ps=r.host)
                r.host = None  # owned by the batch now
                r.admitted = clock()
                active[sid] = r
            if not active:
                if pending:
                    wait = pending[0].arrival - clock()
                    if wait > 0:
                        if realtime:
                            time.sleep(wait)
                        else:
                            skew += wait
                continue
            peak_resident = max(peak_resident, len(active))
            peak_bytes = max(peak_bytes, batch.bytes)
            chunk = min(self.max_chunk, min(r.remaining for r in active.values()))
            batch.step(chunk)
            batch.synchronize()
            chunks += 1
            for sid, r in list(active.items()):
                r.remaining -= chunk
                if r.remaining == 0:
                    if self.keep:
                        v = batch.read(sid)
                        r.result = {"position": np.array(v["position"][: r.scene.n]),
                                    "velocity": np.array(v["velocity"][: r.scene.n])}
                    batch.remove(sid)
                    r.done = clock()
                    del active[sid]
        makespan = clock()
        batch.close()
        lat = np.array([r.done - r.arrival for r in requests])
        work = float(sum(r.work for r in requests))
        return {
            "requests": len(requests),
            "particle_steps": work,
            "makespan_s": makespan,
            "throughput": work / makespan if makespan > 0 else 0.0,
            "p50_s": float(np.percentile(lat, 50)) if len(lat) else 0.0,
            "p99_s": float(np.percentile(lat, 99)) if len(lat) else 0.0,
            "chunks": chunks,
            "peak_resident": peak_resident,
            "peak_bytes": peak_bytes,
        }


def sequential_fifo(requests, service_time):
    """Latencies of a one-at-a-time FIFO server with the given per-request
    service times (seconds): the plain per-scene loop's queue."""
    t = 0.0
    lat = []
    for r in sorted(requests, key=lambda r: r.arrival):
        start = max(t, r.arrival)
        t = start + service_time(r)
        lat.append(t - r.arrival)
    lat = np.array(lat)
    work = float(sum(r.work for r in requests))
    return {"makespan_s": t, "throughput": work / t if t > 0 else 0.0,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99))}


def release(requests):
    for r in requests:
        if r.host is not None:
            free_data_cpu(r.host)
            r.host = None
