"""Served form: a request loop with continuous batching.

Requests (a scene and a substep count) arrive over time.  The server keeps
one :class:`~sph.batch.Batch` on the device.  Between chunks it admits
arrived requests first come, first served, while the batch stays within
the HBM budget and the resident-particle cap (enough particles to fill
the GPU; admitting more only makes everyone wait longer).  Each admitted
scene gets a substep quota equal to its request (`Batch.set_steps`), then
the whole batch advances by a chunk of up to `max_chunk` substeps: a scene
whose quota runs out inside the chunk goes idle on the device (every kernel
skips it) until the chunk ends, when its result is read back and its memory
freed for the next admissions.  Scenes that arrive while others run join at
the next chunk boundary and share their launches; a scene's result is the
same as when it runs alone (the batch kernels treat scenes independently).

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
        self.status = 0        # the scene's status word when it finished

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
    def __init__(self, budget_bytes=150e9, max_chunk=25, max_particles=8 << 20, keep_results=True, tune=None):
        self.budget = float(budget_bytes)
        self.max_chunk = int(max_chunk)
        self.max_particles = int(max_particles)
        self.keep = keep_results
        self.tune = tune

    def prepare(self, requests):
        """Builds each request's host store ahead of its arrival: the full
        store, or for a device-built lattice scene (scene.gen) only its
        conf values, the particles being made on the device at admission."""
        for r in requests:
            if r.host is None:
                r.host = Batch.lattice_store(r.scene) if r.scene.gen else Batch.host_store(r.scene)
                r.bytes = Batch.scene_bytes(r.scene, r.host)

    def _fits(self, batch, resident, r, active):
        if not active:
            return True  # a lone request always runs, whatever its size
        return batch.bytes + r.bytes <= self.budget and resident + r.scene.n <= self.max_particles

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
        resident = 0
        t0 = time.perf_counter()
        skew = 0.0

        def clock():
            return time.perf_counter() - t0 + skew

        chunks = 0
        substeps = 0
        log = []  # per chunk: resident particles, scenes, substeps, particle-steps advanced, seconds
        peak_resident = 0
        peak_particles = 0
        peak_bytes = 0
        busy = 0.0
        while pending or active:
            now = clock()
            while pending and pending[0].arrival <= now and self._fits(batch, resident, pending[0], active):
                r = pending.popleft()
                sid = batch.add_lattice(r.scene, ps=r.host) if r.scene.gen else batch.add(r.scene, ps=r.host)
                r.host = None  # owned by the batch now
                batch.set_steps(sid, r.remaining)
                r.admitted = clock()
                active[sid] = r
                resident += r.scene.n
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
            peak_particles = max(peak_particles, resident)
            peak_bytes = max(peak_bytes, batch.bytes)
            chunk = min(self.max_chunk, max(r.remaining for r in active.values()))
            advanced = sum(r.scene.n * min(chunk, r.remaining) for r in active.values())
            c0 = time.perf_counter()
            batch.step(chunk)
            batch.synchronize()
            dt = time.perf_counter() - c0
            busy += dt
            log.append((resident, len(active), chunk, advanced, dt))
            chunks += 1
            substeps += chunk
            for sid, r in list(active.items()):
                r.remaining -= min(chunk, r.remaining)
                if r.remaining == 0:
                    r.status = batch.status(sid)
                    if self.keep:
                        v = batch.read(sid)
                        r.result = {"position": np.array(v["position"][: r.scene.n]),
                                    "velocity": np.array(v["velocity"][: r.scene.n])}
                    batch.remove(sid)
                    r.done = clock()
                    resident -= r.scene.n
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
            "status_failed": sum(1 for r in requests if r.status),
            "chunks": chunks,
            "substeps": substeps,
            "gpu_busy_s": busy,
            # particle-steps/s while chunks ran (finished scenes idling in
            # their last chunk count as not advancing)
            "busy_throughput": sum(c[3] for c in log) / busy if busy > 0 else 0.0,
            "chunk_log": log,
            "peak_resident": peak_resident,
            "peak_particles": peak_particles,
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
