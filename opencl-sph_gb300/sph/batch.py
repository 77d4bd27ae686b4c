"""Batched form: many independent scenes advanced together on the GPU.

A :class:`Batch` keeps each scene's store resident on the device and
advances all of them with one CUDA graph per substep (libsph_gb300's
sph_batch_* entry points): every phase is one segment-aware launch over
all scenes, and the fluid / corotational / SVK material phases run as
parallel graph branches.  A scene's result does not depend on what else is
in the batch.
"""
import ctypes

import numpy as np

from . import bindings as bnd
from . import free_data_cpu, init_data_cpu


class Scene(object):
    """A scene resident in a batch: its host store and id."""

    def __init__(self, scene, ps, sid):
        self.scene = scene
        self.psdata = ps
        self.id = sid
        self.views = bnd.store_views(ps)


class Batch(object):
    def __init__(self):
        self.handle = bnd.sph_batch_create()
        if not self.handle:
            raise bnd.SphError(bnd.last_error())
        self.scenes = {}
        self._reads = None

    @staticmethod
    def host_store(scene):
        ps = init_data_cpu(scene.spec)
        v = bnd.store_views(ps)
        for k, val in scene.init.items():
            arr = np.asarray(val)
            if arr.size > 1:
                # fewer rows than the store's capacity fill its leading part
                v[k][tuple(slice(None, d) for d in arr.shape)] = arr
            else:
                v[k][...] = arr
        return ps

    @staticmethod
    def lattice_store(scene):
        """The host store of a device-built lattice scene: the conf's values
        and the small initial fields only (the particle arrays are made on
        the device)."""
        ps = init_data_cpu(scene.spec)
        v = bnd.store_views(ps)
        for k, val in scene.init.items():
            arr = np.asarray(val)
            if arr.nbytes <= 4096:
                v[k][...] = arr if arr.size == 1 else arr.reshape(v[k].shape)
        return ps

    @staticmethod
    def scene_bytes(scene, ps=None):
        own = ps is None
        ps = ps or Batch.host_store(scene)
        b = bnd.sph_scene_bytes(ctypes.byref(ps), scene.kernel_files)
        if own:
            free_data_cpu(ps)
        return int(b)

    def add(self, scene, ps=None):
        """Uploads `scene` (its initial values, or the given host store)."""
        ps = ps or self.host_store(scene)
        sid = bnd.sph_batch_add(self.handle, ctypes.byref(ps), scene.kernel_files)
        if sid < 0:
            free_data_cpu(ps)
            raise bnd.SphError(bnd.last_error())
        self.scenes[sid] = Scene(scene, ps, sid)
        return sid

    def add_lattice(self, scene, ps=None):
        """Adds a lattice scene built on the device (scene.gen, from a
        builder called with jitter_hash=True): no particle array is made or
        uploaded on the host.  The result equals add(scene)."""
        if not scene.gen:
            raise ValueError("%s has no device lattice (build it with jitter_hash=True)" % scene.name)
        g = scene.gen
        lat = bnd.sph_lattice(g["nx"], g["ny"], g["nz"], g["clamp_layers"], g["identity_rotation"], g["spacing"],
                              g["jitter"], (ctypes.c_double * 3)(*g["origin"]), g["seed"])
        ps = ps or self.lattice_store(scene)
        sid = bnd.sph_batch_add_lattice(self.handle, ctypes.byref(ps), scene.kernel_files, ctypes.byref(lat))
        if sid < 0:
            free_data_cpu(ps)
            raise bnd.SphError(bnd.last_error())
        self.scenes[sid] = Scene(scene, ps, sid)
        return sid

    def remove(self, sid):
        if bnd.sph_batch_remove(self.handle, sid) != 0:
            raise bnd.SphError(bnd.last_error())
        self._reads = None
        free_data_cpu(self.scenes.pop(sid).psdata)

    def step(self, steps=1):
        if bnd.sph_batch_step(self.handle, steps) != 0:
            raise bnd.SphError(bnd.last_error())

    UNLIMITED = 0xFFFFFFFF

    def set_steps(self, sid, steps):
        """Substep quota: the scene takes part in the next `steps` substeps
        and then stays idle (unchanged) until given a new quota."""
        if bnd.sph_batch_set_steps(self.handle, sid, int(steps)) != 0:
            raise bnd.SphError(bnd.last_error())

    def steps_left(self, sid):
        return int(bnd.sph_batch_steps_left(self.handle, sid))

    def synchronize(self):
        if bnd.sph_batch_synchronize(self.handle) != 0:
            raise bnd.SphError(bnd.last_error())

    def read(self, sid):
        """Copies scene `sid` back; returns its host views (name -> array)."""
        s = self.scenes[sid]
        if bnd.sph_batch_read(self.handle, sid, ctypes.byref(s.psdata)) != 0:
            raise bnd.SphError(bnd.last_error())
        return s.views

    def read_field(self, sid, name):
        """Copies one field of scene `sid` back; returns its host view."""
        s = self.scenes[sid]
        if bnd.sph_batch_read_field(self.handle, sid, name, ctypes.byref(s.psdata)) != 0:
            raise bnd.SphError(bnd.last_error())
        return s.views[name]

    def pin(self, sid):
        """Page-locks scene `sid`'s host store, so that read_fields writes it
        from one copy kernel; removing the scene or closing the batch ends
        it."""
        if bnd.sph_batch_pin_host(self.handle, sid, ctypes.byref(self.scenes[sid].psdata)) != 0:
            raise bnd.SphError(bnd.last_error())

    def unpin(self, sid):
        if bnd.sph_batch_unpin_host(self.handle, sid) != 0:
            raise bnd.SphError(bnd.last_error())

    def read_fields(self, sids, name):
        """Copies one field of several scenes back with a single wait (one
        kernel for the pinned stores); returns their host views (sid ->
        array)."""
        key, ids, outs = self._read_args(sids)
        if bnd.sph_batch_read_field_many(self.handle, ids, len(key), name, outs) != 0:
            raise bnd.SphError(bnd.last_error())
        return {sid: self.scenes[sid].views[name] for sid in key}

    def read_fields_async(self, sids, name):
        """Enqueues a read of one field of several pinned scenes: a device
        snapshot in stream order, written into their host stores while later
        substeps run.  Returns a ticket for wait_read()."""
        key, ids, outs = self._read_args(sids)
        t = bnd.sph_batch_read_field_many_async(self.handle, ids, len(key), name, outs)
        if t < 0:
            raise bnd.SphError(bnd.last_error())
        return t

    def write_fields_async(self, sids, *names):
        """Enqueues a write of the named fields of several scenes from their
        host stores (one host-to-device copy and one scatter kernel for all
        of them), in stream order before the substeps enqueued next; the
        host stores may change as soon as this returns."""
        if not names:
            raise ValueError("no field to write")
        key, ids, outs = self._read_args(sids)
        if len(names) == 1:
            rc = bnd.sph_batch_write_field_many_async(self.handle, ids, len(key), names[0], outs)
        else:
            arr = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
            rc = bnd.sph_batch_write_fields_many_async(self.handle, ids, len(key), len(names), arr, outs)
        if rc < 0:
            raise bnd.SphError(bnd.last_error())

    def wait_read(self, ticket):
        if bnd.sph_batch_wait_read(self.handle, ticket) != 0:
            raise bnd.SphError(bnd.last_error())

    def wait_reads(self):
        if bnd.sph_batch_wait_reads(self.handle) != 0:
            raise bnd.SphError(bnd.last_error())

    def _read_args(self, sids):
        key = tuple(sids)
        if self._reads is None or self._reads[0] != key:
            # the argument arrays, kept while the same scenes are read
            ids = (ctypes.c_int * len(key))(*key)
            outs = (ctypes.POINTER(bnd.psdata) * len(key))(*[ctypes.pointer(self.scenes[s].psdata) for s in key])
            self._reads = (key, ids, outs)
        return self._reads

    def profile(self, reps=3):
        """Mean device ms per phase of a substep (phases run one by one)."""
        ms = (ctypes.c_float * 16)()
        names = (ctypes.c_char_p * 16)()
        k = bnd.sph_batch_profile(self.handle, reps, ms, names, 16)
        if k < 0:
            raise bnd.SphError(bnd.last_error())
        return {names[i].decode(): float(ms[i]) for i in range(k)}

    def tune(self, block, pair_block, grid_cap):
        if bnd.sph_batch_tune(self.handle, block, pair_block, grid_cap) != 0:
            raise bnd.SphError(bnd.last_error())

    @property
    def bytes(self):
        return int(bnd.sph_batch_bytes(self.handle))

    @property
    def kernels_per_step(self):
        return int(bnd.sph_batch_kernel_count(self.handle))

    @property
    def stream(self):
        return bnd.sph_batch_stream(self.handle)

    def status(self, sid):
        return int(bnd.sph_batch_status(self.handle, sid))

    @property
    def particles(self):
        return sum(s.scene.n for s in self.scenes.values())

    def close(self):
        if self.handle:
            bnd.sph_batch_free(self.handle)
            self.handle = None
        for s in self.scenes.values():
            free_data_cpu(s.psdata)
        self.scenes = {}
        self._reads = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
