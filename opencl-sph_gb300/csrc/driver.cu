// driver.cu -- the drop-in device driver of libsph_gb300.so: the C ABI of
// src/opencl/particle_system_host.h re-implemented on CUDA streams, with
// the psdata blob mirrored as one device allocation and the reference's
// kernel names dispatched to the sm_103a kernels (launch.h).
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "launch.h"
#include "sph_gb300.h"
#include "sph_internal.h"
#include "store.h"

// ---------------------------------------------------------------------------
// errors

namespace {
std::mutex g_err_mu;
std::string g_error;
int g_abort_on_error = 1;
}  // namespace

void sph_set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_error = buf;
}

void sph_fail() {
    if (!g_abort_on_error) return;
    std::string msg;
    {
        std::lock_guard<std::mutex> lk(g_err_mu);
        msg = g_error;
    }
    fprintf(stderr, "sph: %s\n", msg.c_str());
    abort();
}

extern "C" const char *sph_last_error(void) {
    static thread_local std::string copy;
    std::lock_guard<std::mutex> lk(g_err_mu);
    copy = g_error;
    return copy.c_str();
}
extern "C" void sph_clear_error(void) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_error.clear();
}
extern "C" void sph_set_abort_on_error(int a) { g_abort_on_error = a; }

extern "C" const char *sph_version(void) {
    return "sph_gb300 1.0 (sm_103a; opencl-sph psdata ABI; FP32 pipeline, FP64 polar decomposition)";
}

// ---------------------------------------------------------------------------
// the per-store device state behind psdata_cuda.ps_prog

namespace {

struct Store {
    psdata host;                 // the host struct this store mirrors
    unsigned programs = 0;
    int material = -1;
    cudaStream_t stream = nullptr;
    Arena arena;                 // blob + scratch + tables
    char *d_blob = nullptr;
    size_t blob_size = 0;
    SceneDesc desc{};
    SceneDesc *d_desc = nullptr;
    Launch L{};
    cudaGraphExec_t step_graph = nullptr;
    unsigned graph_kernels = 0;
    std::vector<unsigned> rigid;   // rigid bodies (1-based), as last read from the host store
    RigidWork *d_rigid = nullptr;  // device list, room for every body
    unsigned rigid_room = 0;
    // device-resident recording (sph_record_*): one allocation holding the
    // counters, the field ranges and the ring
    char *rec_mem = nullptr;
    RecordPlan rec{};
    std::vector<std::string> rec_fields;
    // sph_pin_host: the host blob, page-locked by this store, and its
    // device-side address (mapped), or null
    void *pinned = nullptr;
    char *pinned_dev = nullptr;
    // calls through the store's entry points, and the call that recorded
    // the candidate masks in a named compute_density (0: none): a named
    // compute_forces_fluids that comes right after it, with no other call
    // between, finds the positions, velocities, densities and cell tables
    // the masks were recorded from, and walks them
    unsigned long long calls = 0, mask_call = 0;
    // the same for the solid recipe: the call of a named first solid pass
    // (which records its masks), and of a compute_stresses right after it
    // (which then writes the sorted stress copies): a compute_forces_solids
    // right after that walks the masks from the sorted copies
    unsigned long long solid_call = 0, stress_call = 0;
    // sph_read_fields_async: reads take turns over two snapshot buffers;
    // the stream `reads` copies a snapshot into the host store while later
    // substeps run on `stream`
    cudaStream_t reads = nullptr;
    cudaEvent_t snap_done[2] = {nullptr, nullptr}, read_done[2] = {nullptr, nullptr};
    char *snap[2] = {nullptr, nullptr};
    size_t snap_cap[2] = {0, 0};
    long long tickets = 0;  // reads enqueued so far
};

std::mutex g_stores_mu;
std::set<Store *> g_stores;

bool cuda_ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    sph_set_error("%s: %s", what, cudaGetErrorString(e));
    return false;
}

Store *store_of(const psdata_cuda &pso, const char *what) {
    Store *s = static_cast<Store *>(pso.ps_prog);
    std::lock_guard<std::mutex> lk(g_stores_mu);
    if (!s || !g_stores.count(s)) {
        sph_set_error("%s: not a live device store (created by create_psdata_cuda and not freed)", what);
        return nullptr;
    }
    ++s->calls;
    return s;
}

// Waits for every asynchronous read of the store.
bool drain_reads(Store *s, const char *what) {
    return !s->reads || cuda_ok(cudaStreamSynchronize(s->reads), what);
}

void destroy(Store *s) {
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->reads) {
        cudaStreamSynchronize(s->reads);
        for (int t = 0; t < 2; ++t) {
            if (s->snap[t]) cudaFree(s->snap[t]);
            if (s->snap_done[t]) cudaEventDestroy(s->snap_done[t]);
            if (s->read_done[t]) cudaEventDestroy(s->read_done[t]);
        }
        cudaStreamDestroy(s->reads);
    }
    if (s->pinned) cudaHostUnregister(s->pinned);
    if (s->rec_mem) cudaFree(s->rec_mem);
    if (s->step_graph) cudaGraphExecDestroy(s->step_graph);
    if (s->arena.base) cudaFree(s->arena.base);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

// Re-reads which bodies are rigid from the host store; a change of the
// list re-records the substep graph.
bool refresh_rigid(Store *s, const psdata &data) {
    std::vector<unsigned> now = sph_rigid_bodies(data, s->desc);
    if (now.size() > s->rigid_room) now.resize(s->rigid_room);
    if (now == s->rigid) return true;
    std::vector<RigidWork> w;
    for (unsigned b : now) w.push_back(RigidWork{0u, b});
    if (!w.empty() &&
        !cuda_ok(cudaMemcpyAsync(s->d_rigid, w.data(), w.size() * sizeof(RigidWork), cudaMemcpyHostToDevice,
                                 s->stream),
                 "rigid body list") )
        return false;
    // the list is read by launches already queued: let them finish first
    if (!cuda_ok(cudaStreamSynchronize(s->stream), "rigid body list")) return false;
    s->rigid = now;
    s->L.num_rigid = (unsigned)now.size();
    if (s->step_graph) cudaGraphExecDestroy(s->step_graph);
    s->step_graph = nullptr;
    s->graph_kernels = 0;
    return true;
}

// The grid resolution and the particle capacity size the device tables and
// block maps when the store is created, so an upload may not change them:
// the reference re-reads gridres on every launch (USE_FIELD), but its
// gridcount and celloffset fields keep the size the store was built with,
// and a larger gridres would index past them.  Checked before any copy.
bool shape_unchanged(const Store *s, const psdata &data, const char *what) {
    const int fr = get_field_psdata(data, "gridres"), fp = get_field_psdata(data, "pnum");
    if (fr < 0 || fp < 0) return true;
    const unsigned *res = (const unsigned *)((const char *)data.data + data.data_offsets[fr]);
    const unsigned pnum = *(const unsigned *)((const char *)data.data + data.data_offsets[fp]);
    if (res[0] == s->desc.gridres[0] && res[1] == s->desc.gridres[1] && res[2] == s->desc.gridres[2] &&
        pnum == s->desc.pnum)
        return true;
    sph_set_error("%s: gridres %ux%ux%u / pnum %u differ from the %ux%ux%u / %u the device store was created "
                  "with; the cell tables and block maps are sized at creation (create a new store instead)",
                  what, res[0], res[1], res[2], pnum, s->desc.gridres[0], s->desc.gridres[1], s->desc.gridres[2],
                  s->desc.pnum);
    return false;
}

bool names_shape(const char *const *names, size_t num) {
    for (size_t i = 0; i < num; ++i)
        if (names[i] && (!strcmp(names[i], "gridres") || !strcmp(names[i], "pnum"))) return true;
    return false;
}

// Fields the rigid bodies are set up from.
bool touches_rigid_setup(const char *name) {
    static const char *kNames[] = {"position", "velocity", "body_number", "body_dynamic", "body_count", "n"};
    for (const char *k : kNames)
        if (!strcmp(name, k)) return true;
    return false;
}

// Builds the device mirror of a host store.
Store *create_store(psdata *data, const char *file_list, std::string *err) {
    unsigned programs = sph_parse_programs(file_list, err);
    if (!programs) return nullptr;
    SceneDesc probe;
    if (!sph_resolve_scene(*data, nullptr, programs, &probe, err)) return nullptr;

    Store *s = new Store();
    s->host = *data;
    s->programs = programs;
    s->material = sph_material_of(programs);
    s->blob_size = psdata_data_size(*data);

    const unsigned block = 256, pair_block = 128;
    std::vector<SceneDesc> descs(1, probe);
    HostMaps maps;
    sph_build_maps(descs, {0u}, block, pair_block, &maps);

    size_t o_blob = 0;
    size_t o_scratch = o_blob + Arena::align(s->blob_size);
    size_t o_desc = o_scratch + Arena::align(sph_scratch_bytes(probe));
    size_t o_pm = o_desc + Arena::align(sizeof(SceneDesc));
    size_t o_ppm = o_pm + Arena::align(maps.particles.size() * sizeof(BlockWork));
    size_t o_cm = o_ppm + Arena::align(maps.pair_particles.size() * sizeof(BlockWork));
    size_t o_sm = o_cm + Arena::align(maps.cells.size() * sizeof(BlockWork));
    size_t o_rw = o_sm + Arena::align(maps.scan.size() * sizeof(BlockWork));
    s->rigid_room = std::min(probe.body_capacity, SPH_MAX_RIGID_WORK);
    size_t total = o_rw + Arena::align(s->rigid_room * sizeof(RigidWork));

    if (!cuda_ok(sph_prepare_kernels(), "kernel attributes") ||
        !cuda_ok(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaMalloc(&s->arena.base, total), "cudaMalloc(store)")) {
        *err = sph_last_error();
        destroy(s);
        return nullptr;
    }
    s->arena.size = total;
    char *b = s->arena.base;
    s->d_blob = b + o_blob;
    std::string e2;
    sph_resolve_scene(*data, s->d_blob, programs, &s->desc, &e2);
    sph_place_scratch(&s->desc, b + o_scratch);
    s->desc.steps_left = nullptr;  // a single store has no substep quota
    s->d_desc = reinterpret_cast<SceneDesc *>(b + o_desc);
    s->d_rigid = s->rigid_room ? reinterpret_cast<RigidWork *>(b + o_rw) : nullptr;
    auto up = [&](size_t off, const void *src, size_t bytes) {
        return bytes == 0 || cuda_ok(cudaMemcpyAsync(b + off, src, bytes, cudaMemcpyHostToDevice, s->stream),
                                     "cudaMemcpy(store)");
    };
    bool ok = up(o_blob, data->data, s->blob_size) && up(o_desc, &s->desc, sizeof(SceneDesc)) &&
              up(o_pm, maps.particles.data(), maps.particles.size() * sizeof(BlockWork)) &&
              up(o_ppm, maps.pair_particles.data(), maps.pair_particles.size() * sizeof(BlockWork)) &&
              up(o_cm, maps.cells.data(), maps.cells.size() * sizeof(BlockWork)) &&
              up(o_sm, maps.scan.data(), maps.scan.size() * sizeof(BlockWork)) &&
              cuda_ok(cudaMemsetAsync(s->desc.status, 0, 4, s->stream), "cudaMemset(status)") &&
              (!s->desc.rigid_state ||
               cuda_ok(cudaMemsetAsync(s->desc.rigid_state, 0, 8ull * s->desc.body_capacity * SPH_RIGID_STRIDE,
                                       s->stream),
                       "cudaMemset(rigid)")) &&
              cuda_ok(cudaStreamSynchronize(s->stream), "create_psdata_cuda");
    if (!ok) {
        *err = sph_last_error();
        destroy(s);
        return nullptr;
    }
    Launch &L = s->L;
    L.scenes = s->d_desc;
    L.num_scenes = 1;
    L.particles = {reinterpret_cast<BlockWork *>(b + o_pm), (unsigned)maps.particles.size()};
    L.pair_particles = {reinterpret_cast<BlockWork *>(b + o_ppm), (unsigned)maps.pair_particles.size()};
    L.cells = {reinterpret_cast<BlockWork *>(b + o_cm), (unsigned)maps.cells.size()};
    L.scan = {reinterpret_cast<BlockWork *>(b + o_sm), (unsigned)maps.scan.size()};
    L.block = block;
    L.pair_block = pair_block;
    L.grid_cap = 1u << 30;
    L.stream = s->stream;
    L.no_symmetry_planes = s->desc.num_symmetry_planes == 0;
    L.has_mixed = s->desc.phase != nullptr;
    L.all_mixed = L.has_mixed;  // one scene per store
    L.rigid = s->d_rigid;
    L.num_rigid = 0;
    if (!refresh_rigid(s, *data)) {
        *err = sph_last_error();
        destroy(s);
        return nullptr;
    }
    {
        std::lock_guard<std::mutex> lk(g_stores_mu);
        g_stores.insert(s);
    }
    return s;
}

// After enqueueing work: report launch errors (and, in the synchronous
// mode the reference's clFinish implies, execution errors).
bool finish(Store *s, const char *what, bool sync) {
    if (sph_check_launch(what) != cudaSuccess) return false;
    if (sync && !cuda_ok(cudaStreamSynchronize(s->stream), what)) return false;
    return true;
}

const char *kNeedsArgs[] = {"populate_position_cuboid", "rotate_particles", "set_body_position",
                            "set_body_rotation"};

// call_for_all_particles_device_opencl (particle_system_host.c:517-528):
// the reference's kernel names mapped onto launch sequences.  Pair kernels
// first refresh the cell-sorted copies from the current fields, so a named
// call sees exactly the fields the reference's kernel would read.
bool dispatch(Store *s, const char *name) {
    const Launch &L = s->L;
    const unsigned P = s->programs;
    auto need = [&](unsigned bits, const char *file) {
        if (P & bits) return true;
        sph_set_error("kernel '%s' is not in this store's program (needs %s.cl)", name, file);
        return false;
    };
    std::string k = name ? name : "";
    if (k == "find_particle_bins") { sph_launch_find_bins(L); return true; }
    if (k == "zero_gridcount") { sph_launch_zero_cells(L); return true; }
    if (k == "count_particles_in_bins") { sph_launch_count(L); return true; }
    if (k == "prefix_sum") { sph_launch_scan(L); return true; }
    // the arrival slots recorded by the count replace the backup cursor
    if (k == "copy_celloffset_to_backup") return true;
    if (k == "insert_particles_in_bin_array") { sph_launch_insert(L); return true; }
    if (k == "compute_density") {
        if ((P & PROG_FLUIDS) && !s->desc.phase && s->desc.nbmask) {
            // a fluid store: the masked pass (with the count), after a
            // gather of positions and velocities, so that the next call may
            // be the masked force pass
            sph_launch_gather(L, true, false);
            sph_launch_density(L, false, true, false, true);
            s->mask_call = s->calls;
            return true;
        }
        sph_launch_gather(L, false, false);
        sph_launch_density(L, false);
        return true;
    }
    if (k == "step_forward") {
        sph_launch_step_forward(L);
        sph_launch_rigid(L);  // rigid bodies (extension) take their step with the particles'
        return true;
    }
    if (k == "compute_forces_fluids") {
        if (!need(PROG_FLUIDS, "fluids")) return false;
        if (s->mask_call && s->calls == s->mask_call + 1) {
            // right after the masked compute_density: its sorted copies,
            // pressures, reciprocal densities and masks are current; the
            // walk gives the scan's bits (and the same neighbour count)
            sph_launch_forces_fluids(L, false, true);
            return true;
        }
        sph_launch_gather(L, true, true);
        sph_launch_forces_fluids(L, false);
        return true;
    }
    if (k == "init_original_position") {
        if (!need(PROG_SOLIDS, "solids")) return false;
        sph_launch_init_original_position(L);
        return true;
    }
    // a mixed fluid-solid store (extension): the solid kernels cover the
    // solid particles over their solid neighbours, and the fluid force pass
    // adds the fluid pair terms to the elastic forces (call it after
    // compute_forces_solids, as sph_update does)
    const bool mixed = s->desc.phase != nullptr;
    if (k == "compute_original_density") {
        if (!need(PROG_SOLIDS, "solids")) return false;
        sph_launch_gather(L, false, false);
        if (mixed) sph_launch_original_density_mixed(L);
        else sph_launch_density(L, true);
        return true;
    }
    if (mixed && k == "compute_deformations") {
        sph_launch_gather(L, false, false, true);
        sph_launch_deformations_mixed(L, false);
        return true;
    }
    if (mixed && k == "compute_forces_solids") {
        sph_launch_gather(L, false, false, true);
        sph_launch_forces_solids_mixed(L);
        return true;
    }
    if (k == "compute_rotations_and_strains") {
        if (!need(PROG_COROT, "solid_corotation")) return false;
        sph_launch_gather(L, false, false, true);
        sph_launch_rotations_and_strains(L);
        s->solid_call = s->desc.sstress ? s->calls : 0;
        return true;
    }
    if (k == "compute_deformations") {
        if (!need(PROG_SVK, "solid_svk")) return false;
        sph_launch_gather(L, false, false, true);
        sph_launch_deformations(L);
        s->solid_call = s->desc.sstress ? s->calls : 0;
        return true;
    }
    if (k == "compute_stresses") {
        if (!need(PROG_COROT | PROG_SVK, "solid_corotation or solid_svk")) return false;
        if (s->solid_call && s->calls == s->solid_call + 1) {
            // right after the first solid pass: the stress law writes the
            // sorted copies too (same field values), for the masked walk
            sph_launch_stresses(L, (P & PROG_COROT) != 0, true, false);
            s->stress_call = s->calls;
            return true;
        }
        sph_launch_stresses(L, (P & PROG_COROT) != 0);
        return true;
    }
    if (k == "compute_forces_solids") {
        if (!need(PROG_COROT | PROG_SVK, "solid_corotation or solid_svk")) return false;
        if (s->stress_call && s->calls == s->stress_call + 1) {
            // right after that compute_stresses: the positions, velocities,
            // rest positions and masks of the first pass and the sorted
            // stresses are current; the walk gives the scan's bits (scenes
            // with symmetry planes scan, as in a fused substep)
            sph_launch_forces_solids(L, (P & PROG_COROT) != 0, true, false);
            return true;
        }
        sph_launch_gather(L, false, false);
        sph_launch_forces_solids(L, (P & PROG_COROT) != 0);
        return true;
    }
    if (k == "apply_plane_constraints") {
        if (!need(PROG_CONSTRAINTS, "constraints")) return false;
        sph_launch_plane_constraints(L);
        return true;
    }
    for (const char *a : kNeedsArgs)
        if (k == a) {
            sph_set_error("kernel '%s' takes arguments; call its own entry point", name);
            return false;
        }
    sph_set_error("no kernel named '%s'", name);
    return false;
}

template <typename F>
void with_store(const psdata_cuda &pso, const char *what, bool sync, F &&body) {
    Store *s = store_of(pso, what);
    if (!s) { sph_fail(); return; }
    if (!body(s) || !finish(s, what, sync)) sph_fail();
}

bool copy_field(Store *s, const psdata &data, const char *name, bool to_device) {
    int f = get_field_psdata(data, name);
    if (f < 0) {
        note(1, "Field %s not found.\n", name);
        return true;  // the reference logs and skips (particle_system_host.c:819-822)
    }
    size_t off = data.data_offsets[f], sz = data.data_sizes[f];
    if (off + sz > s->blob_size) {
        sph_set_error("field %s lies outside the device store", name);
        return false;
    }
    char *host = (char *)data.data + off;
    char *dev = s->d_blob + off;
    return cuda_ok(to_device ? cudaMemcpyAsync(dev, host, sz, cudaMemcpyHostToDevice, s->stream)
                             : cudaMemcpyAsync(host, dev, sz, cudaMemcpyDeviceToHost, s->stream),
                   "field copy");
}

}  // namespace

// ---------------------------------------------------------------------------
// ABI

extern "C" void init_cuda(void) {
    if (!cuda_ok(cudaFree(nullptr), "init_cuda")) sph_fail();
}
extern "C" void terminate_cuda(void) {
    if (!cuda_ok(cudaDeviceSynchronize(), "terminate_cuda")) sph_fail();
}

extern "C" psdata_cuda create_psdata_cuda(psdata *data, const char *file_list) {
    psdata_cuda pso;
    memset(&pso, 0, sizeof(pso));
    std::string err;
    Store *s = data ? create_store(data, file_list, &err) : nullptr;
    if (!s) {
        sph_set_error("create_psdata_cuda: %s", data ? err.c_str() : "null store");
        sph_fail();
        return pso;
    }
    pso.host_psdata = *data;
    pso.num_fields = data->num_fields;
    pso.data = s->d_blob;
    pso.block_totals = s->desc.scan_sums;
    pso.backup_prefix_sum = s->desc.slot;
    pso.ps_prog = s;
    pso.num_grid_cells = s->desc.num_cells;
    // the reference's work-group bookkeeping (particle_system_host.c:661-674)
    pso.po2_workgroup_size = 256;
    pso.num_blocks = (s->desc.num_cells - 1) / 512 + 1;
    return pso;
}

extern "C" void free_psdata_cuda(psdata_cuda *pso) {
    if (!pso) return;
    Store *s = store_of(*pso, "free_psdata_cuda");
    if (!s) { sph_fail(); return; }
    {
        std::lock_guard<std::mutex> lk(g_stores_mu);
        g_stores.erase(s);
    }
    destroy(s);
    pso->ps_prog = nullptr;
    pso->data = nullptr;
    pso->block_totals = nullptr;
    pso->backup_prefix_sum = nullptr;
}

// particle_system_host.c:837-841
extern "C" void sync_psdata_device_to_host(psdata data, psdata_cuda pso) {
    with_store(pso, "sync_psdata_device_to_host", true, [&](Store *s) {
        if (!drain_reads(s, "sync_psdata_device_to_host")) return false;
        size_t sz = psdata_data_size(data);
        if (sz > s->blob_size) {
            sph_set_error("store layout differs from the device copy");
            return false;
        }
        return cuda_ok(cudaMemcpyAsync(data.data, s->d_blob, sz, cudaMemcpyDeviceToHost, s->stream), "sync");
    });
}

// particle_system_host.c:780-809; the layout tables never change on the
// device (field offsets are resolved once), so `full` has nothing more to
// upload.
extern "C" void sync_psdata_host_to_device(psdata data, psdata_cuda pso, int full) {
    (void)full;
    with_store(pso, "sync_psdata_host_to_device", true, [&](Store *s) {
        if (!drain_reads(s, "sync_psdata_host_to_device")) return false;
        size_t sz = psdata_data_size(data);
        if (sz > s->blob_size) {
            sph_set_error("store layout differs from the device copy");
            return false;
        }
        if (!shape_unchanged(s, data, "sync_psdata_host_to_device")) return false;
        if (!cuda_ok(cudaMemcpyAsync(s->d_blob, data.data, sz, cudaMemcpyHostToDevice, s->stream), "sync") ||
            !refresh_rigid(s, data))
            return false;
        if (s->desc.rigid_state) sph_launch_rigid_reset(s->L);
        return true;
    });
}

// particle_system_host.c:812-829
extern "C" void sync_psdata_fields_host_to_device(psdata data, psdata_cuda pso, size_t num_fields,
                                                  const char *const *names) {
    with_store(pso, "sync_psdata_fields_host_to_device", true, [&](Store *s) {
        if (!drain_reads(s, "sync_psdata_fields_host_to_device")) return false;
        if (names_shape(names, num_fields) && !shape_unchanged(s, data, "sync_psdata_fields_host_to_device"))
            return false;
        bool rigid = false;
        for (size_t i = 0; i < num_fields; ++i) {
            if (names[i] && !copy_field(s, data, names[i], true)) return false;
            rigid = rigid || (names[i] && touches_rigid_setup(names[i]));
        }
        if (rigid && s->desc.rigid_state) {
            if (!refresh_rigid(s, data)) return false;
            sph_launch_rigid_reset(s->L);
        }
        return true;
    });
}

// particle_system_host.c:843-858
extern "C" void sync_psdata_fields_device_to_host(psdata data, psdata_cuda pso, size_t num_fields,
                                                  const char *const *names) {
    with_store(pso, "sync_psdata_fields_device_to_host", true, [&](Store *s) {
        if (!drain_reads(s, "sync_psdata_fields_device_to_host")) return false;
        for (size_t i = 0; i < num_fields; ++i)
            if (names[i] && !copy_field(s, data, names[i], false)) return false;
        return true;
    });
}

extern "C" void call_for_all_particles_device_cuda(psdata_cuda pso, const char *kernel_name) {
    with_store(pso, kernel_name ? kernel_name : "call_for_all_particles", false,
               [&](Store *s) { return dispatch(s, kernel_name); });
}

// particle_system_host.c:448-454
extern "C" void compute_particle_bins_device_cuda(psdata_cuda pso) {
    with_store(pso, "compute_particle_bins", false, [&](Store *s) {
        sph_launch_bins(s->L);
        return true;
    });
}

extern "C" void compute_density_device_cuda(psdata_cuda pso) {
    call_for_all_particles_device_cuda(pso, "compute_density");
}

// particle_system_host.c:477-495 launches a kernel named "compute_forces",
// which no reference program defines; here it is the store's force pass.
extern "C" void compute_forces_device_cuda(psdata_cuda pso) {
    Store *s = store_of(pso, "compute_forces");
    if (!s) { sph_fail(); return; }
    if (s->desc.phase) {  // a mixed store: the elastic forces, then the fluid pair terms
        call_for_all_particles_device_cuda(pso, "compute_forces_solids");
        call_for_all_particles_device_cuda(pso, "compute_forces_fluids");
        return;
    }
    call_for_all_particles_device_cuda(pso, (s->programs & (PROG_COROT | PROG_SVK)) ? "compute_forces_solids"
                                                                                     : "compute_forces_fluids");
}

extern "C" void step_forward_device_cuda(psdata_cuda pso) { call_for_all_particles_device_cuda(pso, "step_forward"); }

extern "C" void populate_position_cuboid_device_cuda(psdata_cuda pso, float x1, float y1, float z1, float x2,
                                                     float y2, float z2, unsigned xs, unsigned ys, unsigned zs) {
    with_store(pso, "populate_position_cuboid", false, [&](Store *s) {
        const float c1[3] = {x1, y1, z1}, c2[3] = {x2, y2, z2};
        const unsigned sz[3] = {xs, ys, zs};
        if (xs == 0 || ys == 0 || zs == 0) return true;
        sph_launch_populate_cuboid(s->L, c1, c2, sz);
        if (s->desc.rigid_state) sph_launch_rigid_reset(s->L);
        return true;
    });
}

extern "C" void rotate_particles_device_cuda(psdata_cuda pso, float ax, float ay, float az) {
    with_store(pso, "rotate_particles", false, [&](Store *s) {
        sph_launch_rotate_particles(s->L, ax, ay, az);
        if (s->desc.rigid_state) sph_launch_rigid_reset(s->L);
        return true;
    });
}

static bool body_ok(Store *s, unsigned body, const char *what) {
    if (!(s->programs & PROG_RIGIDBODY)) {
        sph_set_error("%s: the store's program lacks rigidbody.cl", what);
        return false;
    }
    if (body >= s->desc.body_capacity) {
        sph_set_error("%s: body %u beyond the store's %u bodies", what, body, s->desc.body_capacity);
        return false;
    }
    return true;
}

// particle_system_host.c:562-574
extern "C" void set_body_position_device_cuda(psdata_cuda pso, unsigned body, float *position) {
    with_store(pso, "set_body_position", false, [&](Store *s) {
        if (!body_ok(s, body, "set_body_position")) return false;
        sph_launch_set_body_position(s->L, body, position);
        return true;
    });
}

// particle_system_host.c:576-588
extern "C" void set_body_rotation_device_cuda(psdata_cuda pso, unsigned body, float *euler) {
    with_store(pso, "set_body_rotation", false, [&](Store *s) {
        if (!body_ok(s, body, "set_body_rotation")) return false;
        sph_launch_set_body_rotation(s->L, body, euler);
        return true;
    });
}

extern "C" int sph_synchronize(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_synchronize");
    if (!s) return -1;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && s->reads) e = cudaStreamSynchronize(s->reads);
    if (e != cudaSuccess) sph_set_error("sph_synchronize: %s", cudaGetErrorString(e));
    return (int)e;
}

extern "C" int sph_pin_host(psdata data, psdata_cuda pso) {
    const char *what = "sph_pin_host";
    Store *s = store_of(pso, what);
    if (!s) return -1;
    if (psdata_data_size(data) != s->blob_size || !data.data) {
        sph_set_error("%s: store layout differs from the device copy", what);
        return -1;
    }
    if (s->pinned == data.data) return 0;
    if (s->pinned) {
        sph_set_error("%s: another host store is pinned for this device store (sph_unpin_host first)", what);
        return -1;
    }
    // mapped, so that small writes can be read in place by a kernel; a
    // device that cannot map host memory gets the plain page-locking
    if (cudaHostRegister(data.data, s->blob_size, cudaHostRegisterMapped) != cudaSuccess) {
        cudaGetLastError();
        if (!cuda_ok(cudaHostRegister(data.data, s->blob_size, cudaHostRegisterDefault), what)) return -1;
    }
    s->pinned = data.data;
    void *dev = nullptr;
    s->pinned_dev = cudaHostGetDevicePointer(&dev, data.data, 0) == cudaSuccess ? static_cast<char *>(dev) : nullptr;
    cudaGetLastError();  // a store without a device-side address keeps the copy-engine writes
    return 0;
}

extern "C" int sph_unpin_host(psdata_cuda pso) {
    const char *what = "sph_unpin_host";
    Store *s = store_of(pso, what);
    if (!s) return -1;
    if (!s->pinned) return 0;
    // copies into or out of the blob must end before it is unlocked
    if (!cuda_ok(cudaStreamSynchronize(s->stream), what) || !drain_reads(s, what)) return -1;
    void *p = s->pinned;
    s->pinned = nullptr;
    s->pinned_dev = nullptr;
    return cuda_ok(cudaHostUnregister(p), what) ? 0 : -1;
}

extern "C" int sph_write_fields_async(psdata data, psdata_cuda pso, size_t num_fields, const char *const *names) {
    const char *what = "sph_write_fields_async";
    Store *s = store_of(pso, what);
    if (!s) return -1;
    if (num_fields && !names) {
        sph_set_error("%s: no field names", what);
        return -1;
    }
    if (names_shape(names, num_fields) && !shape_unchanged(s, data, what)) return -1;
    bool rigid = false;
    // a pinned store's few small fields go by one copy kernel reading the
    // mapped host store (no copy engine: see InlineSegs), others by copies
    InlineSegs inl{};
    size_t inl_bytes = 0;
    const bool inline_ok = s->pinned == data.data && s->pinned_dev && num_fields <= SPH_INLINE_SEGS;
    for (size_t i = 0; i < num_fields; ++i) {
        if (!names[i]) continue;
        rigid = rigid || touches_rigid_setup(names[i]);
        const int f = get_field_psdata(data, names[i]);
        if (inline_ok && f >= 0 && data.data_offsets[f] + data.data_sizes[f] <= s->blob_size &&
            inl_bytes + data.data_sizes[f] <= 65536) {
            const size_t off = data.data_offsets[f], sz = data.data_sizes[f];
            inl.seg[inl.count++] = CopySeg{s->pinned_dev + off, s->d_blob + off, (unsigned long long)sz};
            inl_bytes += sz;
            continue;
        }
        if (!copy_field(s, data, names[i], true)) return -1;
    }
    if (inl.count) {
        sph_launch_copy_inline(inl, s->stream);
        if (sph_check_launch(what) != cudaSuccess) return -1;
    }
    if (rigid && s->desc.rigid_state) {
        if (!refresh_rigid(s, data)) return -1;
        sph_launch_rigid_reset(s->L);
    }
    return finish(s, what, false) ? 0 : -1;
}

extern "C" long long sph_read_fields_async(psdata data, psdata_cuda pso, size_t num_fields,
                                           const char *const *names) {
    const char *what = "sph_read_fields_async";
    Store *s = store_of(pso, what);
    if (!s) return -1;
    if (psdata_data_size(data) != s->blob_size || !data.data) {
        sph_set_error("%s: store layout differs from the device copy", what);
        return -1;
    }
    if (num_fields && !names) {
        sph_set_error("%s: no field names", what);
        return -1;
    }
    if (!s->reads) {
        bool good = cuda_ok(cudaStreamCreateWithFlags(&s->reads, cudaStreamNonBlocking), what);
        for (int t = 0; good && t < 2; ++t)
            good = cuda_ok(cudaEventCreateWithFlags(&s->snap_done[t], cudaEventDisableTiming), what) &&
                   cuda_ok(cudaEventCreateWithFlags(&s->read_done[t], cudaEventDisableTiming), what);
        if (!good) return -1;
    }
    struct Part {
        size_t off, at, bytes;
    };
    std::vector<Part> parts;
    size_t total = 0;
    for (size_t i = 0; i < num_fields; ++i) {
        const int f = names[i] ? get_field_psdata(data, names[i]) : -1;
        if (f < 0) {
            sph_set_error("%s: no field '%s'", what, names[i] ? names[i] : "");
            return -1;
        }
        parts.push_back(Part{data.data_offsets[f], total, data.data_sizes[f]});
        total += (data.data_sizes[f] + 15) / 16 * 16;
    }
    const int t = (int)(s->tickets & 1);
    // turn t's snapshot is free once the read two tickets back has written
    // the host store (an event never recorded counts as complete)
    if (!cuda_ok(cudaStreamWaitEvent(s->stream, s->read_done[t], 0), what)) return -1;
    if (total > s->snap_cap[t]) {
        if (s->snap[t] && !cuda_ok(cudaStreamSynchronize(s->reads), what)) return -1;
        if (s->snap[t]) cudaFree(s->snap[t]);
        s->snap[t] = nullptr;
        s->snap_cap[t] = 0;
        if (!cuda_ok(cudaMalloc(&s->snap[t], total), what)) return -1;
        s->snap_cap[t] = total;
    }
    // the snapshot, in stream order after the substeps enqueued so far
    for (const Part &p : parts)
        if (!cuda_ok(cudaMemcpyAsync(s->snap[t] + p.at, s->d_blob + p.off, p.bytes, cudaMemcpyDeviceToDevice,
                                     s->stream),
                     what))
            return -1;
    if (!cuda_ok(cudaEventRecord(s->snap_done[t], s->stream), what) ||
        !cuda_ok(cudaStreamWaitEvent(s->reads, s->snap_done[t], 0), what))
        return -1;
    // the host store, written by the copy engines beside later substeps
    char *host = static_cast<char *>(data.data);
    for (const Part &p : parts)
        if (!cuda_ok(cudaMemcpyAsync(host + p.off, s->snap[t] + p.at, p.bytes, cudaMemcpyDeviceToHost, s->reads),
                     what))
            return -1;
    if (!cuda_ok(cudaEventRecord(s->read_done[t], s->reads), what)) return -1;
    return s->tickets++;
}

extern "C" int sph_wait_read(psdata_cuda pso, long long ticket) {
    Store *s = store_of(pso, "sph_wait_read");
    if (!s) return -1;
    if (ticket < 0 || ticket >= s->tickets) {
        sph_set_error("sph_wait_read: no such read");
        return -1;
    }
    // the turn's event covers this read or a later one of the same turn,
    // which the stream ordered after it
    return cuda_ok(cudaEventSynchronize(s->read_done[ticket & 1]), "sph_wait_read") ? 0 : -1;
}

extern "C" int sph_wait_reads(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_wait_reads");
    if (!s) return -1;
    return drain_reads(s, "sph_wait_reads") ? 0 : -1;
}

extern "C" int sph_update(psdata_cuda pso, unsigned num_steps) {
    Store *s = store_of(pso, "sph_update");
    if (!s) return -1;
    if (s->material < 0) {
        sph_set_error("sph_update: the store's program has no substep recipe (needs fluids, "
                      "solid_corotation or solid_svk)");
        return -1;
    }
    if (!s->step_graph) {
        cudaGraph_t g = nullptr;
        if (!cuda_ok(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "capture")) return -1;
        sph_launch_substep(s->L, (SphMaterial)s->material);
        if (s->rec_mem) sph_launch_record(s->rec, s->stream);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
        if (le != cudaSuccess || ce != cudaSuccess) {
            sph_set_error("sph_update capture: %s", cudaGetErrorString(le != cudaSuccess ? le : ce));
            if (g) cudaGraphDestroy(g);
            return -1;
        }
        size_t nn = 0;
        cudaGraphGetNodes(g, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
        s->graph_kernels = 0;
        for (size_t k = 0; k < nn; ++k) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++s->graph_kernels;
        }
        cudaError_t ie = cudaGraphInstantiate(&s->step_graph, g, 0);
        cudaGraphDestroy(g);
        if (!cuda_ok(ie, "cudaGraphInstantiate")) {
            s->step_graph = nullptr;
            return -1;
        }
    }
    for (unsigned k = 0; k < num_steps; ++k)
        if (!cuda_ok(cudaGraphLaunch(s->step_graph, s->stream), "cudaGraphLaunch")) return -1;
    return 0;
}

namespace {
struct ProfileCtx {
    cudaStream_t stream;
    std::vector<cudaEvent_t> events;
    std::vector<const char *> names;
    bool ok = true;
};
void profile_mark(void *p, const char *name) {
    ProfileCtx *c = static_cast<ProfileCtx *>(p);
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) { c->ok = false; return; }
    cudaEventRecord(e, c->stream);
    c->events.push_back(e);
    c->names.push_back(name);
}
}  // namespace

extern "C" int sph_profile_substep(psdata_cuda pso, unsigned reps, float *phase_ms, const char **phase_names,
                                   unsigned max_phases) {
    Store *s = store_of(pso, "sph_profile_substep");
    if (!s) return -1;
    if (s->material < 0) {
        sph_set_error("sph_profile_substep: no substep recipe for this store's program");
        return -1;
    }
    std::vector<double> acc;
    std::vector<const char *> names;
    for (unsigned r = 0; r < reps; ++r) {
        ProfileCtx c;
        c.stream = s->stream;
        sph_launch_substep(s->L, (SphMaterial)s->material, profile_mark, &c);
        bool ok = c.ok && sph_check_launch("sph_profile_substep") == cudaSuccess &&
                  cuda_ok(cudaStreamSynchronize(s->stream), "sph_profile_substep");
        if (ok && acc.empty()) {
            acc.assign(c.events.size() - 1, 0.0);
            names.assign(c.names.begin(), c.names.end() - 1);
        }
        for (size_t k = 0; ok && k + 1 < c.events.size(); ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, c.events[k], c.events[k + 1]);
            acc[k] += ms;
        }
        for (cudaEvent_t e : c.events) cudaEventDestroy(e);
        if (!ok) return -1;
    }
    unsigned np = (unsigned)acc.size() < max_phases ? (unsigned)acc.size() : max_phases;
    for (unsigned k = 0; k < np; ++k) {
        phase_ms[k] = reps ? (float)(acc[k] / reps) : 0.f;
        if (phase_names) phase_names[k] = names[k];
    }
    return (int)np;
}

// ---- device-resident recording ------------------------------------------------

static void drop_graph(Store *s) {
    if (s->step_graph) cudaGraphExecDestroy(s->step_graph);
    s->step_graph = nullptr;
    s->graph_kernels = 0;
}

extern "C" int sph_record_stop(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_record_stop");
    if (!s) return -1;
    if (!cuda_ok(cudaStreamSynchronize(s->stream), "sph_record_stop")) return -1;
    if (s->rec_mem) cudaFree(s->rec_mem);
    s->rec_mem = nullptr;
    s->rec = RecordPlan{};
    s->rec_fields.clear();
    drop_graph(s);
    return 0;
}

extern "C" int sph_record_start(psdata_cuda pso, size_t num_fields, const char *const *names, unsigned every,
                                unsigned frames) {
    Store *s = store_of(pso, "sph_record_start");
    if (!s) return -1;
    if (!num_fields || !names || !every || !frames) {
        sph_set_error("sph_record_start: needs at least one field, every >= 1 and frames >= 1");
        return -1;
    }
    std::vector<uint2> ranges;
    std::vector<std::string> fields;
    size_t words = 0;
    for (size_t k = 0; k < num_fields; ++k) {
        const int f = names[k] ? get_field_psdata(s->host, names[k]) : -1;
        if (f < 0) {
            sph_set_error("sph_record_start: no field '%s' in the store", names[k] ? names[k] : "");
            return -1;
        }
        const size_t off = s->host.data_offsets[f], sz = s->host.data_sizes[f];
        if (off % 4 || sz % 4) {
            sph_set_error("sph_record_start: field '%s' is not word-aligned", names[k]);
            return -1;
        }
        ranges.push_back(make_uint2((unsigned)(off / 4), (unsigned)(sz / 4)));
        fields.push_back(names[k]);
        words += sz / 4;
    }
    const size_t ring_bytes = (size_t)frames * words * 4;
    if (words > 0xffffffffu || ring_bytes / frames / 4 != words) {
        sph_set_error("sph_record_start: frame too large");
        return -1;
    }
    if (sph_record_stop(pso) != 0) return -1;
    const size_t o_ranges = 256, o_ring = Arena::align(o_ranges + ranges.size() * sizeof(uint2));
    char *mem = nullptr;
    if (!cuda_ok(cudaMalloc(&mem, o_ring + ring_bytes), "sph_record_start")) return -1;
    if (!cuda_ok(cudaMemsetAsync(mem, 0, 256, s->stream), "sph_record_start") ||
        !cuda_ok(cudaMemcpyAsync(mem + o_ranges, ranges.data(), ranges.size() * sizeof(uint2),
                                 cudaMemcpyHostToDevice, s->stream),
                 "sph_record_start") ||
        !cuda_ok(cudaStreamSynchronize(s->stream), "sph_record_start")) {
        cudaFree(mem);
        return -1;
    }
    s->rec_mem = mem;
    s->rec.counters = reinterpret_cast<unsigned long long *>(mem);
    s->rec.ranges = reinterpret_cast<const uint2 *>(mem + o_ranges);
    s->rec.num_ranges = (unsigned)ranges.size();
    s->rec.frame_words = (unsigned)words;
    s->rec.blob = reinterpret_cast<const unsigned *>(s->d_blob);
    s->rec.ring = reinterpret_cast<unsigned *>(mem + o_ring);
    s->rec.frames = frames;
    s->rec.every = every;
    s->rec_fields = fields;
    drop_graph(s);
    return 0;
}

extern "C" unsigned long long sph_record_count(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_record_count");
    unsigned long long c[2] = {0, 0};
    if (!s || !s->rec_mem) return 0;
    if (!cuda_ok(cudaMemcpyAsync(c, s->rec.counters, sizeof(c), cudaMemcpyDeviceToHost, s->stream),
                 "sph_record_count") ||
        !cuda_ok(cudaStreamSynchronize(s->stream), "sph_record_count"))
        return 0;
    return c[1];
}

extern "C" size_t sph_record_frame_bytes(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_record_frame_bytes");
    return s && s->rec_mem ? (size_t)s->rec.frame_words * 4 : 0;
}

extern "C" int sph_record_read(psdata_cuda pso, void *host, unsigned long long first, unsigned count) {
    Store *s = store_of(pso, "sph_record_read");
    if (!s) return -1;
    if (!s->rec_mem) {
        sph_set_error("sph_record_read: not recording");
        return -1;
    }
    const unsigned long long recorded = sph_record_count(pso);
    const unsigned long long kept = recorded < s->rec.frames ? recorded : s->rec.frames;
    if (first < recorded - kept || first + count > recorded) {
        sph_set_error("sph_record_read: frames [%llu, %llu) not held (the ring holds [%llu, %llu))", first,
                      first + count, recorded - kept, recorded);
        return -1;
    }
    const size_t fb = (size_t)s->rec.frame_words * 4;
    for (unsigned k = 0; k < count; ++k) {
        const size_t slot = (size_t)((first + k) % s->rec.frames);
        if (!cuda_ok(cudaMemcpyAsync(static_cast<char *>(host) + k * fb, s->rec.ring + slot * s->rec.frame_words, fb,
                                     cudaMemcpyDeviceToHost, s->stream),
                     "sph_record_read"))
            return -1;
    }
    return cuda_ok(cudaStreamSynchronize(s->stream), "sph_record_read") ? 0 : -1;
}

extern "C" void *sph_stream(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_stream");
    return s ? (void *)s->stream : nullptr;
}

extern "C" unsigned sph_graph_kernel_count(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_graph_kernel_count");
    return s ? s->graph_kernels : 0u;
}

extern "C" unsigned sph_status(psdata_cuda pso) {
    Store *s = store_of(pso, "sph_status");
    if (!s) return 0xFFFFFFFFu;
    unsigned v = 0;
    if (!cuda_ok(cudaMemcpyAsync(&v, s->desc.status, 4, cudaMemcpyDeviceToHost, s->stream), "sph_status") ||
        !cuda_ok(cudaStreamSynchronize(s->stream), "sph_status"))
        return 0xFFFFFFFFu;
    return v;
}

extern "C" void sph_clear_status(psdata_cuda pso) {
    with_store(pso, "sph_clear_status", false, [&](Store *s) {
        return cuda_ok(cudaMemsetAsync(s->desc.status, 0, 4, s->stream), "sph_clear_status");
    });
}

// ---- the reference's names -------------------------------------------------

extern "C" void init_opencl(void) { init_cuda(); }
extern "C" void terminate_opencl(void) { terminate_cuda(); }
extern "C" psdata_opencl create_psdata_opencl(psdata *data, const char *file_list) {
    return create_psdata_cuda(data, file_list);
}
extern "C" void free_psdata_opencl(psdata_opencl *pso) { free_psdata_cuda(pso); }
extern "C" void populate_position_cuboid_device_opencl(psdata_opencl pso, float x1, float y1, float z1, float x2,
                                                       float y2, float z2, unsigned xs, unsigned ys, unsigned zs) {
    populate_position_cuboid_device_cuda(pso, x1, y1, z1, x2, y2, z2, xs, ys, zs);
}
extern "C" void rotate_particles_device_opencl(psdata_opencl pso, float ax, float ay, float az) {
    rotate_particles_device_cuda(pso, ax, ay, az);
}
extern "C" void call_for_all_particles_device_opencl(psdata_opencl pso, const char *kernel_name) {
    call_for_all_particles_device_cuda(pso, kernel_name);
}
extern "C" void compute_particle_bins_device_opencl(psdata_opencl pso) { compute_particle_bins_device_cuda(pso); }
extern "C" void compute_density_device_opencl(psdata_opencl pso) { compute_density_device_cuda(pso); }
extern "C" void compute_forces_device_opencl(psdata_opencl pso) { compute_forces_device_cuda(pso); }
extern "C" void step_forward_device_opencl(psdata_opencl pso) { step_forward_device_cuda(pso); }
extern "C" void set_body_position_device_opencl(psdata_opencl pso, unsigned body, float *position) {
    set_body_position_device_cuda(pso, body, position);
}
extern "C" void set_body_rotation_device_opencl(psdata_opencl pso, unsigned body, float *euler) {
    set_body_rotation_device_cuda(pso, body, euler);
}
