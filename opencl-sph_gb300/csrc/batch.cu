// batch.cu -- the batched form: many independent scenes resident on the
// device, advanced together by segment-aware launches captured in one
// CUDA graph per substep (see the sph_batch_* declarations in sph_gb300.h).
//
// Memory is stream-ordered (allocations from the batch's own pool and
// cudaFreeAsync on the batch's stream), so adding or retiring a scene never
// synchronises the device and work already queued keeps running: this is
// what lets the serving loop admit requests while others are on the GPU.
// The pool keeps what retired scenes freed for the next admissions (its
// release threshold is unbounded): the default pool releases its memory at
// every synchronisation and would map it again for the next scene.
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "launch.h"
#include "sph_gb300.h"
#include "sph_internal.h"
#include "store.h"

namespace {

struct BatchScene {
    unsigned programs = 0;
    int material = -1;
    std::vector<unsigned> rigid;  // rigid bodies (1-based), from the host store at add
    char *mem = nullptr;     // blob followed by scratch
    size_t bytes = 0;
    size_t blob_size = 0;
    SceneDesc desc{};
    // the host store page-locked by sph_batch_pin_host, and its device
    // address (written by sph_batch_read_field_many's copy kernel)
    char *host = nullptr;
    char *host_dev = nullptr;
    bool host_owned = false;  // registered here (else by the caller)
};

bool ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    sph_set_error("%s: %s", what, cudaGetErrorString(e));
    return false;
}

struct GroupLaunch {
    Launch L{};
    bool present = false;
};

}  // namespace


struct sph_batch {
    cudaMemPool_t pool = nullptr;  // every device allocation of the batch
    cudaStream_t stream = nullptr;
    cudaStream_t side[2] = {nullptr, nullptr};

    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    std::vector<BatchScene *> slots;
    bool dirty = true;
    char *tables = nullptr;  // scene table + block maps
    size_t table_bytes = 0;
    Launch all{};
    GroupLaunch group[3];    // by SphMaterial
    cudaGraphExec_t graph = nullptr;
    unsigned graph_kernels = 0;
    unsigned block = 256, pair_block = 128, grid_cap = 0;
    size_t bytes = 0;
    CopySeg *copy_segs = nullptr;  // device table of sph_batch_read_field_many
    unsigned copy_cap = 0;
    // sph_batch_read_field_many_async: reads take turns over two snapshot
    // buffers and segment tables; the stream `reads` copies a snapshot into
    // the pinned host stores while later substeps run on `stream`
    cudaStream_t reads = nullptr;
    cudaEvent_t snap_done[2] = {nullptr, nullptr}, read_done[2] = {nullptr, nullptr};
    char *snap[2] = {nullptr, nullptr};
    size_t snap_cap[2] = {0, 0};
    CopySeg *snap_segs[2] = {nullptr, nullptr};
    unsigned snap_seg_cap[2] = {0, 0};
    CopySeg *seg_host[2] = {nullptr, nullptr};  // pinned: the upload must not wait for the stream
    size_t seg_host_cap[2] = {0, 0};
    unsigned seg_count[2] = {0, 0};             // segments in turn t's device table (0: none)
    long long tickets = 0;  // reads enqueued so far
    // sph_batch_write_field_many_async: writes take turns over two pinned
    // staging buffers (segment table, then the fields' bytes), each copied
    // to a device buffer of its turn and scattered into the scenes by one
    // copy kernel; write_done[t] marks the staging buffer's copy finished
    char *wstage_host[2] = {nullptr, nullptr};
    size_t wstage_host_cap[2] = {0, 0};
    char *wstage_dev[2] = {nullptr, nullptr};
    size_t wstage_dev_cap[2] = {0, 0};
    cudaEvent_t write_done[2] = {nullptr, nullptr};
    long long wtickets = 0;  // writes enqueued so far
};

// A stream-ordered allocation from the batch's pool.
static bool balloc(sph_batch *b, void **p, size_t bytes, cudaStream_t stream, const char *what) {
    return ok(cudaMallocFromPoolAsync(p, bytes, b->pool, stream), what);
}

namespace {

unsigned cap_of(const sph_batch *b) { return b->grid_cap ? b->grid_cap : (1u << 30); }

// Uploads a table of scenes and its maps into one stream-ordered buffer.
struct TableBuild {
    std::vector<char> host;
    size_t add(const void *p, size_t n) {
        const size_t o = host.size();
        host.resize(o + Arena::align(n), 0);
        const char *src = static_cast<const char *>(p);
        std::copy(src, src + n, host.begin() + o);
        return o;
    }
};

BlockMap map_at(char *base, size_t off, const std::vector<BlockWork> &v) {
    return {reinterpret_cast<const BlockWork *>(base + off), (unsigned)v.size()};
}

void release_graph(sph_batch *b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_kernels = 0;
}

// Runs the solid setup (init_original_position, compute_particle_bins,
// compute_original_density) for one freshly added scene.
bool solid_setup(sph_batch *b, BatchScene *sc) {
    std::vector<SceneDesc> one(1, sc->desc);
    HostMaps m;
    sph_build_maps(one, {0u}, b->block, b->pair_block, &m);
    TableBuild t;
    size_t o_d = t.add(&sc->desc, sizeof(SceneDesc));
    size_t o_p = t.add(m.particles.data(), m.particles.size() * sizeof(BlockWork));
    size_t o_pp = t.add(m.pair_particles.data(), m.pair_particles.size() * sizeof(BlockWork));
    size_t o_c = t.add(m.cells.data(), m.cells.size() * sizeof(BlockWork));
    size_t o_s = t.add(m.scan.data(), m.scan.size() * sizeof(BlockWork));
    char *d = nullptr;
    if (!balloc(b, (void **)&d, t.host.size(), b->stream, "scene setup tables")) return false;
    if (!ok(cudaMemcpyAsync(d, t.host.data(), t.host.size(), cudaMemcpyHostToDevice, b->stream), "setup upload"))
        return false;
    Launch L{};
    L.scenes = reinterpret_cast<SceneDesc *>(d + o_d);
    L.num_scenes = 1;
    L.particles = map_at(d, o_p, m.particles);
    L.pair_particles = map_at(d, o_pp, m.pair_particles);
    L.cells = map_at(d, o_c, m.cells);
    L.scan = map_at(d, o_s, m.scan);
    L.block = b->block;
    L.pair_block = b->pair_block;
    L.grid_cap = cap_of(b);
    L.stream = b->stream;
    L.no_symmetry_planes = sc->desc.num_symmetry_planes == 0;
    sph_launch_init_original_position(L);
    sph_launch_bins(L);
    sph_launch_gather(L, false, false);
    sph_launch_density(L, true);
    bool good = sph_check_launch("sph_batch_add(setup)") == cudaSuccess;
    // the host copy must outlive the asynchronous upload
    good = ok(cudaStreamSynchronize(b->stream), "sph_batch_add(setup)") && good;
    cudaFreeAsync(d, b->stream);
    return good;
}

bool rebuild(sph_batch *b) {
    // the previous graph may still be running: let it finish before its
    // executable and tables go away
    if (b->graph && !ok(cudaStreamSynchronize(b->stream), "batch rebuild")) return false;
    release_graph(b);
    std::vector<unsigned> ids;
    std::vector<SceneDesc> descs;
    for (unsigned i = 0; i < b->slots.size(); ++i)
        if (b->slots[i]) {
            ids.push_back(i);
            descs.push_back(b->slots[i]->desc);
        }
    if (b->tables) cudaFreeAsync(b->tables, b->stream);
    b->tables = nullptr;
    b->table_bytes = 0;
    b->dirty = false;
    if (descs.empty()) return true;
    std::vector<unsigned> idx(descs.size()), by_mat[3];
    for (unsigned k = 0; k < descs.size(); ++k) {
        idx[k] = k;
        by_mat[b->slots[ids[k]]->material].push_back(k);
    }
    HostMaps all, g[3];
    sph_build_maps(descs, idx, b->block, b->pair_block, &all);
    for (int m = 0; m < 3; ++m) sph_build_maps(descs, by_mat[m], b->block, b->pair_block, &g[m]);
    TableBuild t;
    size_t o_d = t.add(descs.data(), descs.size() * sizeof(SceneDesc));
    size_t o_p = t.add(all.particles.data(), all.particles.size() * sizeof(BlockWork));
    size_t o_pp = t.add(all.pair_particles.data(), all.pair_particles.size() * sizeof(BlockWork));
    size_t o_c = t.add(all.cells.data(), all.cells.size() * sizeof(BlockWork));
    size_t o_s = t.add(all.scan.data(), all.scan.size() * sizeof(BlockWork));
    std::vector<RigidWork> rigid;
    for (unsigned k = 0; k < descs.size(); ++k)
        for (unsigned body : b->slots[ids[k]]->rigid)
            if (rigid.size() < SPH_MAX_RIGID_WORK) rigid.push_back(RigidWork{k, body});
    size_t o_rw = t.add(rigid.data(), rigid.size() * sizeof(RigidWork));
    size_t o_gp[3], o_gpp[3];
    for (int m = 0; m < 3; ++m) {
        o_gp[m] = t.add(g[m].particles.data(), g[m].particles.size() * sizeof(BlockWork));
        o_gpp[m] = t.add(g[m].pair_particles.data(), g[m].pair_particles.size() * sizeof(BlockWork));
    }
    if (!balloc(b, (void **)&b->tables, t.host.size(), b->stream, "batch tables")) return false;
    b->table_bytes = t.host.size();
    if (!ok(cudaMemcpyAsync(b->tables, t.host.data(), t.host.size(), cudaMemcpyHostToDevice, b->stream),
            "batch tables upload") ||
        !ok(cudaStreamSynchronize(b->stream), "batch tables upload"))
        return false;
    char *d = b->tables;
    Launch &A = b->all;
    A = Launch{};
    A.scenes = reinterpret_cast<SceneDesc *>(d + o_d);
    A.num_scenes = (unsigned)descs.size();
    A.particles = map_at(d, o_p, all.particles);
    A.pair_particles = map_at(d, o_pp, all.pair_particles);
    A.cells = map_at(d, o_c, all.cells);
    A.scan = map_at(d, o_s, all.scan);
    A.block = b->block;
    A.pair_block = b->pair_block;
    A.grid_cap = cap_of(b);
    A.stream = b->stream;
    A.rigid = rigid.empty() ? nullptr : reinterpret_cast<const RigidWork *>(d + o_rw);
    A.num_rigid = (unsigned)rigid.size();
    A.no_symmetry_planes = std::all_of(descs.begin(), descs.end(),
                                       [](const SceneDesc &d) { return d.num_symmetry_planes == 0; });
    cudaStream_t streams[3] = {b->stream, b->side[0], b->side[1]};
    for (int m = 0; m < 3; ++m) {
        GroupLaunch &G = b->group[m];
        G.present = !by_mat[m].empty();
        G.L = A;
        G.L.particles = map_at(d, o_gp[m], g[m].particles);
        G.L.pair_particles = map_at(d, o_gpp[m], g[m].pair_particles);
        G.L.stream = streams[m];
    }
    // capture one substep: shared phases on the batch stream, then one
    // branch per material present, joined back
    cudaGraph_t graph = nullptr;
    if (!ok(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "batch capture")) return false;
    sph_launch_bins(A);
    sph_launch_gather(A, true, false, true);
    // masks for the fluid scenes only; the plane-free solid scenes' blocks
    // are not launched at all
    sph_launch_density_fused(A, b->group[MAT_FLUID].present ? &b->group[MAT_FLUID].L : nullptr);
    cudaEventRecord(b->fork, b->stream);
    for (int m = 0; m < 3; ++m) {
        GroupLaunch &G = b->group[m];
        if (!G.present) continue;
        if (m > 0) cudaStreamWaitEvent(G.L.stream, b->fork, 0);
        if (m == MAT_FLUID) {
            sph_launch_forces_fluids(G.L, true, true);
        } else {
            sph_launch_solid_passes(G.L, m == MAT_COROT);
        }
        if (m > 0) {
            cudaEventRecord(b->join[m - 1], G.L.stream);
            cudaStreamWaitEvent(b->stream, b->join[m - 1], 0);
        }
    }
    sph_launch_rigid(A);
    sph_launch_count_down(A);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
    if (le != cudaSuccess || ce != cudaSuccess) {
        sph_set_error("batch capture: %s", cudaGetErrorString(le != cudaSuccess ? le : ce));
        if (graph) cudaGraphDestroy(graph);
        return false;
    }
    size_t nn = 0;
    cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(graph, nodes.data(), &nn);
    for (size_t k = 0; k < nn; ++k) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nodes[k], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ++b->graph_kernels;
    }
    cudaError_t ie = cudaGraphInstantiate(&b->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (!ok(ie, "batch graph instantiate")) {
        b->graph = nullptr;
        return false;
    }
    return true;
}

BatchScene *scene_of(sph_batch *b, int id, const char *what) {
    if (!b || id < 0 || (size_t)id >= b->slots.size() || !b->slots[id]) {
        sph_set_error("%s: no scene %d in the batch", what, id);
        return nullptr;
    }
    return b->slots[id];
}

}  // namespace

extern "C" sph_batch *sph_batch_create(void) {
    sph_batch *b = new sph_batch();
    int dev = 0;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    const unsigned long long keep = ~0ull;
    bool good = ok(cudaGetDevice(&dev), "sph_batch_create");
    props.location.id = dev;
    good = good && ok(cudaMemPoolCreate(&b->pool, &props), "sph_batch_create (memory pool)") &&
           ok(cudaMemPoolSetAttribute(b->pool, cudaMemPoolAttrReleaseThreshold, (void *)&keep),
              "sph_batch_create (memory pool)");
    good = good && ok(sph_prepare_kernels(), "sph_batch_create") &&
                ok(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "sph_batch_create") &&
                ok(cudaStreamCreateWithFlags(&b->side[0], cudaStreamNonBlocking), "sph_batch_create") &&
                ok(cudaStreamCreateWithFlags(&b->side[1], cudaStreamNonBlocking), "sph_batch_create") &&
                ok(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "sph_batch_create") &&
                ok(cudaEventCreateWithFlags(&b->join[0], cudaEventDisableTiming), "sph_batch_create") &&
                ok(cudaEventCreateWithFlags(&b->join[1], cudaEventDisableTiming), "sph_batch_create");
    if (!good) {
        sph_batch_free(b);
        return nullptr;
    }
    return b;
}

// Waits for the asynchronous reads in flight (they write host stores).
static bool drain_reads(sph_batch *b, const char *what) {
    return !b->reads || ok(cudaStreamSynchronize(b->reads), what);
}

// Ends sph_batch_pin_host's registration (after the streams' work).
static void unpin_host(sph_batch *b, BatchScene *s) {
    if (!s->host) return;
    drain_reads(b, "unpin");
    cudaStreamSynchronize(b->stream);
    if (s->host_owned) cudaHostUnregister(s->host);
    s->host = s->host_dev = nullptr;
    s->host_owned = false;
}

extern "C" void sph_batch_free(sph_batch *b) {
    if (!b) return;
    drain_reads(b, "sph_batch_free");
    if (b->stream) cudaStreamSynchronize(b->stream);
    release_graph(b);
    for (BatchScene *s : b->slots)
        if (s) {
            unpin_host(b, s);
            if (s->mem) cudaFreeAsync(s->mem, b->stream);
            delete s;
        }
    if (b->tables) cudaFreeAsync(b->tables, b->stream);
    if (b->copy_segs) cudaFreeAsync(b->copy_segs, b->stream);
    for (int t = 0; t < 2; ++t) {
        if (b->snap[t]) cudaFreeAsync(b->snap[t], b->stream);
        if (b->snap_segs[t]) cudaFreeAsync(b->snap_segs[t], b->stream);
    }
    for (int t = 0; t < 2; ++t)
        if (b->wstage_dev[t]) cudaFreeAsync(b->wstage_dev[t], b->stream);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (int t = 0; t < 2; ++t) {
        if (b->seg_host[t]) cudaFreeHost(b->seg_host[t]);
        if (b->wstage_host[t]) cudaFreeHost(b->wstage_host[t]);
    }
    for (cudaEvent_t e : {b->fork, b->join[0], b->join[1], b->snap_done[0], b->snap_done[1], b->read_done[0],
                          b->read_done[1], b->write_done[0], b->write_done[1]})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t s : {b->stream, b->side[0], b->side[1], b->reads})
        if (s) cudaStreamDestroy(s);
    if (b->pool) cudaMemPoolDestroy(b->pool);
    delete b;
}

extern "C" size_t sph_scene_bytes(psdata *scene, const char *file_list) {
    std::string err;
    unsigned programs = scene ? sph_parse_programs(file_list, &err) : 0;
    SceneDesc d;
    if (!programs || !sph_resolve_scene(*scene, nullptr, programs, &d, &err)) {
        sph_set_error("sph_scene_bytes: %s", err.c_str());
        return 0;
    }
    return Arena::align(psdata_data_size(*scene)) + sph_scratch_bytes(d);
}

// sph_batch_add and sph_batch_add_lattice: the scene's device memory from
// the host store (all of it, or with `gen` its small fields and a lattice).
static int add_scene(sph_batch *b, psdata *scene, const char *file_list, const sph_lattice *gen) {
    if (!b || !scene) {
        sph_set_error("sph_batch_add: null batch or scene");
        return -1;
    }
    std::string err;
    unsigned programs = sph_parse_programs(file_list, &err);
    SceneDesc probe;
    if (!programs || !sph_resolve_scene(*scene, nullptr, programs, &probe, &err)) {
        sph_set_error("sph_batch_add: %s", err.c_str());
        return -1;
    }
    int material = sph_material_of(programs);
    if (material < 0) {
        sph_set_error("sph_batch_add: the program has no substep recipe (needs fluids, solid_corotation or solid_svk)");
        return -1;
    }
    if (material == MAT_MIXED) {
        sph_set_error("sph_batch_add: a mixed fluid-solid scene runs as a store of its own (create_psdata_cuda)");
        return -1;
    }
    BatchScene *sc = new BatchScene();
    sc->programs = programs;
    sc->material = material;
    sc->blob_size = psdata_data_size(*scene);
    size_t o_scratch = Arena::align(sc->blob_size);
    sc->bytes = o_scratch + sph_scratch_bytes(probe);
    if (!balloc(b, (void **)&sc->mem, sc->bytes, b->stream, "scene memory")) {
        delete sc;
        return -1;
    }
    sph_resolve_scene(*scene, sc->mem, programs, &sc->desc, &err);
    sph_place_scratch(&sc->desc, sc->mem + o_scratch);
    bool good = true;
    if (gen) {
        const unsigned long long count = (unsigned long long)gen->nx * gen->ny * gen->nz;
        if (count == 0 || count > sc->desc.pnum || !sc->desc.position || !sc->desc.n) {
            sph_set_error("sph_batch_add_lattice: %llu lattice points for a store of %u particles", count,
                          sc->desc.pnum);
            good = false;
        }
        good = good && ok(cudaMemsetAsync(sc->mem, 0, sc->blob_size, b->stream), "sph_batch_add_lattice");
        for (unsigned f = 0; good && f < scene->num_fields; ++f)
            if (scene->data_sizes[f] && scene->data_sizes[f] <= 4096)
                good = ok(cudaMemcpyAsync(sc->mem + scene->data_offsets[f],
                                          static_cast<const char *>(scene->data) + scene->data_offsets[f],
                                          scene->data_sizes[f], cudaMemcpyHostToDevice, b->stream),
                          "sph_batch_add_lattice");
        if (good) {
            LatticeGen g{gen->nx, gen->ny, gen->nz, gen->clamp_layers, gen->identity_rotation, gen->spacing,
                         gen->jitter, {gen->origin[0], gen->origin[1], gen->origin[2]}, gen->seed};
            sph_launch_lattice(sc->desc, g, b->stream);
            good = sph_check_launch("sph_batch_add_lattice") == cudaSuccess;
        }
    } else {
        good = ok(cudaMemcpyAsync(sc->mem, scene->data, sc->blob_size, cudaMemcpyHostToDevice, b->stream),
                  "sph_batch_add upload");
    }
    good = good && ok(cudaMemsetAsync(sc->desc.status, 0, 4, b->stream), "sph_batch_add") &&
                (!sc->desc.rigid_state ||
                 ok(cudaMemsetAsync(sc->desc.rigid_state, 0, 8ull * sc->desc.body_capacity * SPH_RIGID_STRIDE,
                                    b->stream),
                    "sph_batch_add")) &&
                ok((sph_launch_set_steps(sc->desc.steps_left, SPH_STEPS_UNLIMITED, b->stream), cudaGetLastError()),
                   "sph_batch_add") &&
                ok(cudaStreamSynchronize(b->stream), "sph_batch_add upload");
    if (good && material != MAT_FLUID) good = solid_setup(b, sc);
    if (good) sc->rigid = sph_rigid_bodies(*scene, sc->desc);
    if (!good) {
        cudaFreeAsync(sc->mem, b->stream);
        delete sc;
        return -1;
    }
    int id = -1;
    for (size_t i = 0; i < b->slots.size(); ++i)
        if (!b->slots[i]) {
            id = (int)i;
            break;
        }
    if (id < 0) {
        id = (int)b->slots.size();
        b->slots.push_back(nullptr);
    }
    b->slots[id] = sc;
    b->bytes += sc->bytes;
    b->dirty = true;
    return id;
}

extern "C" int sph_batch_add(sph_batch *b, psdata *scene, const char *file_list) {
    return add_scene(b, scene, file_list, nullptr);
}

extern "C" int sph_batch_add_lattice(sph_batch *b, psdata *scene, const char *file_list, const sph_lattice *gen) {
    if (!gen) {
        sph_set_error("sph_batch_add_lattice: no lattice");
        return -1;
    }
    return add_scene(b, scene, file_list, gen);
}

extern "C" int sph_batch_remove(sph_batch *b, int id) {
    BatchScene *sc = scene_of(b, id, "sph_batch_remove");
    if (!sc) return -1;
    unpin_host(b, sc);
    cudaFreeAsync(sc->mem, b->stream);
    b->bytes -= sc->bytes;
    delete sc;
    b->slots[id] = nullptr;
    b->dirty = true;
    return 0;
}

extern "C" int sph_batch_set_steps(sph_batch *b, int id, unsigned int steps) {
    BatchScene *sc = scene_of(b, id, "sph_batch_set_steps");
    if (!sc) return -1;
    sph_launch_set_steps(sc->desc.steps_left, steps, b->stream);
    return sph_check_launch("sph_batch_set_steps") == cudaSuccess ? 0 : -1;
}

extern "C" unsigned int sph_batch_steps_left(sph_batch *b, int id) {
    BatchScene *sc = scene_of(b, id, "sph_batch_steps_left");
    unsigned v = 0;
    if (!sc || !ok(cudaMemcpyAsync(&v, sc->desc.steps_left, 4, cudaMemcpyDeviceToHost, b->stream),
                   "sph_batch_steps_left") ||
        !ok(cudaStreamSynchronize(b->stream), "sph_batch_steps_left"))
        return 0;
    return v;
}

extern "C" int sph_batch_step(sph_batch *b, unsigned num_steps) {
    if (!b) return -1;
    if (b->dirty && !rebuild(b)) return -1;
    if (!b->graph) return 0;  // empty batch
    for (unsigned k = 0; k < num_steps; ++k)
        if (!ok(cudaGraphLaunch(b->graph, b->stream), "sph_batch_step")) return -1;
    return 0;
}

extern "C" int sph_batch_read(sph_batch *b, int id, psdata *out) {
    BatchScene *sc = scene_of(b, id, "sph_batch_read");
    if (!sc) return -1;
    if (!out || psdata_data_size(*out) != sc->blob_size) {
        sph_set_error("sph_batch_read: the host store's layout differs from the scene's");
        return -1;
    }
    if (!drain_reads(b, "sph_batch_read") ||
        !ok(cudaMemcpyAsync(out->data, sc->mem, sc->blob_size, cudaMemcpyDeviceToHost, b->stream), "sph_batch_read") ||
        !ok(cudaStreamSynchronize(b->stream), "sph_batch_read"))
        return -1;
    return 0;
}

static int read_field(sph_batch *b, int id, const char *field, psdata *out, bool wait, const char *what) {
    BatchScene *sc = scene_of(b, id, what);
    if (!sc) return -1;
    int f = out && field ? get_field_psdata(*out, field) : -1;
    if (f < 0 || psdata_data_size(*out) != sc->blob_size) {
        sph_set_error("%s: no field '%s' in a store of the scene's layout", what, field ? field : "");
        return -1;
    }
    size_t off = out->data_offsets[f], sz = out->data_sizes[f];
    if (!drain_reads(b, what) ||
        !ok(cudaMemcpyAsync((char *)out->data + off, sc->mem + off, sz, cudaMemcpyDeviceToHost, b->stream), what))
        return -1;
    return !wait || ok(cudaStreamSynchronize(b->stream), what) ? 0 : -1;
}

extern "C" int sph_batch_read_field(sph_batch *b, int id, const char *field, psdata *out) {
    return read_field(b, id, field, out, true, "sph_batch_read_field");
}

extern "C" int sph_batch_read_field_async(sph_batch *b, int id, const char *field, psdata *out) {
    return read_field(b, id, field, out, false, "sph_batch_read_field_async");
}

extern "C" int sph_batch_pin_host(sph_batch *b, int id, psdata *store) {
    const char *what = "sph_batch_pin_host";
    BatchScene *sc = scene_of(b, id, what);
    if (!sc) return -1;
    if (!store || !store->data || psdata_data_size(*store) != sc->blob_size) {
        sph_set_error("%s: the host store's layout differs from the scene's", what);
        return -1;
    }
    char *host = static_cast<char *>(store->data);
    if (sc->host == host) return 0;
    unpin_host(b, sc);
    bool owned = true;
    cudaError_t e = cudaHostRegister(host, sc->blob_size, cudaHostRegisterMapped);
    if (e == cudaErrorHostMemoryAlreadyRegistered) {
        cudaGetLastError();  // registered by the caller: use it, leave it registered
        owned = false;
    } else if (!ok(e, what)) {
        cudaGetLastError();
        return -1;
    }
    void *dev = nullptr;
    e = cudaHostGetDevicePointer(&dev, host, 0);
    if (e != cudaSuccess || !dev) {
        cudaGetLastError();
        if (owned) cudaHostUnregister(host);
        sph_set_error("%s: no device address for the host store (%s)", what, cudaGetErrorString(e));
        return -1;
    }
    sc->host = host;
    sc->host_dev = static_cast<char *>(dev);
    sc->host_owned = owned;
    return 0;
}

extern "C" int sph_batch_unpin_host(sph_batch *b, int id) {
    BatchScene *sc = scene_of(b, id, "sph_batch_unpin_host");
    if (!sc) return -1;
    unpin_host(b, sc);
    return 0;
}

extern "C" int sph_batch_read_field_many(sph_batch *b, const int *ids, unsigned int count, const char *field,
                                         psdata *const *outs) {
    const char *what = "sph_batch_read_field_many";
    if (!b || (count && (!ids || !outs))) {
        sph_set_error("%s: no batch, ids or stores", what);
        return -1;
    }
    if (!drain_reads(b, what)) return -1;
    std::vector<CopySeg> segs;
    unsigned long long max_bytes = 0;
    for (unsigned k = 0; k < count; ++k) {
        BatchScene *sc = scene_of(b, ids[k], what);
        if (!sc) return -1;
        psdata *out = outs[k];
        const int f = out && field ? get_field_psdata(*out, field) : -1;
        if (f < 0 || psdata_data_size(*out) != sc->blob_size) {
            sph_set_error("%s: no field '%s' in a store of the scene's layout", what, field ? field : "");
            return -1;
        }
        const size_t off = out->data_offsets[f], sz = out->data_sizes[f];
        if (sc->host && sc->host == static_cast<char *>(out->data)) {
            segs.push_back(CopySeg{sc->mem + off, sc->host_dev + off, (unsigned long long)sz});
            if (sz > max_bytes) max_bytes = sz;
        } else if (!ok(cudaMemcpyAsync((char *)out->data + off, sc->mem + off, sz, cudaMemcpyDeviceToHost,
                                       b->stream),
                       what)) {
            return -1;
        }
    }
    if (!segs.empty()) {
        if (segs.size() > b->copy_cap) {
            if (b->copy_segs) cudaFreeAsync(b->copy_segs, b->stream);
            b->copy_segs = nullptr;
            b->copy_cap = 0;
            const unsigned cap = (unsigned)segs.size() * 2;
            if (!balloc(b, (void **)&b->copy_segs, cap * sizeof(CopySeg), b->stream, what)) return -1;
            b->copy_cap = cap;
        }
        if (!ok(cudaMemcpyAsync(b->copy_segs, segs.data(), segs.size() * sizeof(CopySeg), cudaMemcpyHostToDevice,
                                b->stream),
                what))
            return -1;
        sph_launch_copy_segments(b->copy_segs, (unsigned)segs.size(), max_bytes, b->stream);
        if (sph_check_launch(what) != cudaSuccess) return -1;
    }
    return ok(cudaStreamSynchronize(b->stream), what) ? 0 : -1;
}

// Grows a stream-ordered buffer (on `stream`, after what it ordered).
template <class T>
static bool grow(sph_batch *b, T **p, size_t *cap, size_t want, cudaStream_t stream, const char *what) {
    if (want <= *cap) return true;
    if (*p) cudaFreeAsync(*p, stream);
    *p = nullptr;
    *cap = 0;
    const size_t c = want + want / 2;
    if (!balloc(b, (void **)p, c * sizeof(T), stream, what)) return false;
    *cap = c;
    return true;
}

extern "C" long long sph_batch_read_field_many_async(sph_batch *b, const int *ids, unsigned int count,
                                                     const char *field, psdata *const *outs) {
    const char *what = "sph_batch_read_field_many_async";
    if (!b || !count || !ids || !outs) {
        sph_set_error("%s: no batch, ids or stores", what);
        return -1;
    }
    if (!b->reads) {
        bool good = ok(cudaStreamCreateWithFlags(&b->reads, cudaStreamNonBlocking), what);
        for (int t = 0; good && t < 2; ++t)
            good = ok(cudaEventCreateWithFlags(&b->snap_done[t], cudaEventDisableTiming), what) &&
                   ok(cudaEventCreateWithFlags(&b->read_done[t], cudaEventDisableTiming), what);
        if (!good) return -1;
    }
    std::vector<CopySeg> segs(count);
    std::vector<size_t> at(count);
    std::vector<char *> dst(count);
    size_t total = 0;
    unsigned long long max_bytes = 0;
    for (unsigned k = 0; k < count; ++k) {
        BatchScene *sc = scene_of(b, ids[k], what);
        if (!sc) return -1;
        psdata *out = outs[k];
        const int f = out && field ? get_field_psdata(*out, field) : -1;
        if (f < 0 || psdata_data_size(*out) != sc->blob_size) {
            sph_set_error("%s: no field '%s' in a store of the scene's layout", what, field ? field : "");
            return -1;
        }
        if (!sc->host || sc->host != static_cast<char *>(out->data)) {
            sph_set_error("%s: scene %d's store is not pinned (sph_batch_pin_host)", what, ids[k]);
            return -1;
        }
        const size_t off = out->data_offsets[f], sz = out->data_sizes[f];
        segs[k] = CopySeg{sc->mem + off, nullptr, (unsigned long long)sz};
        dst[k] = sc->host + off;
        // the snapshot copy at the field's offset within 16 bytes, so that
        // the copy kernel moves 16-byte words (the buffer is 256-aligned)
        at[k] = total + ((uintptr_t)(sc->mem + off) & 15u);
        total = (at[k] + sz + 15) / 16 * 16;
        if (sz > max_bytes) max_bytes = sz;
    }
    const int t = (int)(b->tickets & 1);
    // turn t's buffers are free once the read two tickets back has written
    // the host stores (an event never recorded counts as complete)
    if (!ok(cudaStreamWaitEvent(b->stream, b->read_done[t], 0), what)) return -1;
    size_t seg_cap = b->snap_seg_cap[t];
    if (!grow(b, &b->snap[t], &b->snap_cap[t], total ? total : 16, b->stream, what) ||
        !grow(b, &b->snap_segs[t], &seg_cap, segs.size(), b->stream, what))
        return -1;
    b->snap_seg_cap[t] = (unsigned)seg_cap;
    for (unsigned k = 0; k < count; ++k) segs[k].dst = b->snap[t] + at[k];
    // a frame loop reads the same field of the same scenes every time: the
    // turn's device table is then current and is not uploaded again (the
    // pinned copy holds what was uploaded, and `grow` kept the table)
    const bool same = b->seg_count[t] == count && b->snap_segs[t] && b->seg_host[t] &&
                      std::equal(segs.begin(), segs.end(), b->seg_host[t], [](const CopySeg &x, const CopySeg &y) {
                          return x.src == y.src && x.dst == y.dst && x.bytes == y.bytes;
                      });
    if (!same) {
        // turn t's pinned table was last uploaded before the snapshot two
        // tickets back
        if (!ok(cudaEventSynchronize(b->snap_done[t]), what)) return -1;
        b->seg_count[t] = 0;
        if (segs.size() > b->seg_host_cap[t]) {
            if (b->seg_host[t]) cudaFreeHost(b->seg_host[t]);
            b->seg_host[t] = nullptr;
            b->seg_host_cap[t] = 0;
            const size_t c = segs.size() * 2;
            if (!ok(cudaMallocHost((void **)&b->seg_host[t], c * sizeof(CopySeg)), what)) return -1;
            b->seg_host_cap[t] = c;
        }
        std::copy(segs.begin(), segs.end(), b->seg_host[t]);
        if (!ok(cudaMemcpyAsync(b->snap_segs[t], b->seg_host[t], segs.size() * sizeof(CopySeg),
                                cudaMemcpyHostToDevice, b->stream),
                what))
            return -1;
        b->seg_count[t] = count;
    }
    // the snapshot, in stream order after the substeps enqueued so far
    sph_launch_copy_segments(b->snap_segs[t], count, max_bytes, b->stream);
    if (!ok(cudaEventRecord(b->snap_done[t], b->stream), what) ||
        !ok(cudaStreamWaitEvent(b->reads, b->snap_done[t], 0), what))
        return -1;
    // the host stores, written by the copy engines beside later substeps
    // (a copy kernel's slow writes to host memory would hold SM slots the
    // substeps need)
    for (unsigned k = 0; k < count; ++k)
        if (!ok(cudaMemcpyAsync(dst[k], b->snap[t] + at[k], segs[k].bytes, cudaMemcpyDeviceToHost, b->reads), what))
            return -1;
    if (!ok(cudaEventRecord(b->read_done[t], b->reads), what) || sph_check_launch(what) != cudaSuccess) return -1;
    return b->tickets++;
}

// Fields a write may not touch: the shape the scene's tables were sized
// for, and (in a scene with rigid bodies) what the bodies are set up from.
static bool write_allowed(const BatchScene *sc, const char *field, const char *what, int id) {
    static const char *kShape[] = {"pnum", "gridres"};
    static const char *kRigid[] = {"position", "velocity", "body_number", "body_dynamic", "body_count", "n"};
    for (const char *k : kShape)
        if (!strcmp(field, k)) {
            sph_set_error("%s: '%s' sizes scene %d's device tables and cannot be written", what, field, id);
            return false;
        }
    if (!sc->rigid.empty())
        for (const char *k : kRigid)
            if (!strcmp(field, k)) {
                sph_set_error("%s: scene %d has rigid bodies, which are set up from '%s'; add it anew instead",
                              what, id, field);
                return false;
            }
    return true;
}

// Writes fields[0 .. nfields) of the scenes ids[0 .. count) from their host
// stores: one staging buffer, one host-to-device copy and one scatter for
// all of them.
static int write_many(sph_batch *b, const int *ids, unsigned count, const char *const *fields, unsigned nfields,
                      psdata *const *ins, const char *what) {
    if (!b || !count || !ids || !ins || !fields || !nfields) {
        sph_set_error("%s: no batch, ids, stores or fields", what);
        return -1;
    }
    if (!b->write_done[0]) {
        for (int t = 0; t < 2; ++t)
            if (!ok(cudaEventCreateWithFlags(&b->write_done[t], cudaEventDisableTiming), what)) return -1;
    }
    // layout of a turn's staging buffer: the segment table, then each
    // scene's bytes of each field at a 16-byte aligned offset
    const size_t nseg = (size_t)count * nfields;
    std::vector<CopySeg> segs(nseg);
    std::vector<const char *> src(nseg);
    std::vector<size_t> at(nseg);
    const size_t table = (nseg * sizeof(CopySeg) + 255) / 256 * 256;
    size_t total = table;
    unsigned long long max_bytes = 0;
    for (unsigned q = 0; q < nfields; ++q) {
        const char *field = fields[q];
        if (!field) {
            sph_set_error("%s: no field name", what);
            return -1;
        }
        for (unsigned k = 0; k < count; ++k) {
            BatchScene *sc = scene_of(b, ids[k], what);
            if (!sc) return -1;
            const psdata *in = ins[k];
            const int f = in ? get_field_psdata(*in, field) : -1;
            if (f < 0 || psdata_data_size(*in) != sc->blob_size) {
                sph_set_error("%s: no field '%s' in a store of the scene's layout", what, field);
                return -1;
            }
            if (!write_allowed(sc, field, what, ids[k])) return -1;
            const size_t off = in->data_offsets[f], sz = in->data_sizes[f];
            const size_t j = (size_t)q * count + k;
            segs[j] = CopySeg{nullptr, sc->mem + off, (unsigned long long)sz};
            src[j] = static_cast<const char *>(in->data) + off;
            at[j] = total;
            total += (sz + 15) / 16 * 16;
            if (sz > max_bytes) max_bytes = sz;
        }
    }
    const int t = (int)(b->wtickets & 1);
    // turn t's staging buffer is free once its copy two writes back is done
    if (!ok(cudaEventSynchronize(b->write_done[t]), what)) return -1;
    if (total > b->wstage_host_cap[t]) {
        if (b->wstage_host[t]) cudaFreeHost(b->wstage_host[t]);
        b->wstage_host[t] = nullptr;
        b->wstage_host_cap[t] = 0;
        const size_t c = total + total / 2;
        if (!ok(cudaMallocHost((void **)&b->wstage_host[t], c), what)) return -1;
        b->wstage_host_cap[t] = c;
    }
    // the scatter reads the page-locked staging buffer where it lies (its
    // device-side address), so the write takes no copy engine and does not
    // queue behind the device-to-host copies of reads in flight; without
    // such an address, one host-to-device copy into a device buffer first
    void *mapped = nullptr;
    char *dev = cudaHostGetDevicePointer(&mapped, b->wstage_host[t], 0) == cudaSuccess
                    ? static_cast<char *>(mapped)
                    : nullptr;
    cudaGetLastError();
    const bool zero_copy = dev != nullptr;
    if (!zero_copy) {
        if (!grow(b, &b->wstage_dev[t], &b->wstage_dev_cap[t], total, b->stream, what)) return -1;
        dev = b->wstage_dev[t];
    }
    for (size_t j = 0; j < nseg; ++j) {
        segs[j].src = dev + at[j];
        memcpy(b->wstage_host[t] + at[j], src[j], (size_t)segs[j].bytes);
    }
    memcpy(b->wstage_host[t], segs.data(), nseg * sizeof(CopySeg));
    // in stream order before the substeps enqueued after this call
    if (!zero_copy && !ok(cudaMemcpyAsync(dev, b->wstage_host[t], total, cudaMemcpyHostToDevice, b->stream), what))
        return -1;
    sph_launch_copy_segments(reinterpret_cast<const CopySeg *>(dev), (unsigned)nseg, max_bytes, b->stream);
    // the staging buffer is free again once the scatter (or the copy) has
    // read it
    if (sph_check_launch(what) != cudaSuccess || !ok(cudaEventRecord(b->write_done[t], b->stream), what)) return -1;
    return (int)(b->wtickets++ & 0x7fffffff);
}

extern "C" int sph_batch_write_field_many_async(sph_batch *b, const int *ids, unsigned int count, const char *field,
                                                psdata *const *ins) {
    return write_many(b, ids, count, &field, 1, ins, "sph_batch_write_field_many_async");
}

extern "C" int sph_batch_write_fields_many_async(sph_batch *b, const int *ids, unsigned int count,
                                                 unsigned int nfields, const char *const *fields,
                                                 psdata *const *ins) {
    return write_many(b, ids, count, fields, nfields, ins, "sph_batch_write_fields_many_async");
}

extern "C" int sph_batch_wait_read(sph_batch *b, long long ticket) {
    if (!b || ticket < 0 || ticket >= b->tickets) {
        sph_set_error("sph_batch_wait_read: no such read");
        return -1;
    }
    // the turn's event covers this read or a later one of the same turn,
    // which the stream ordered after it
    return ok(cudaEventSynchronize(b->read_done[ticket & 1]), "sph_batch_wait_read") ? 0 : -1;
}

extern "C" int sph_batch_wait_reads(sph_batch *b) {
    if (!b) return -1;
    return drain_reads(b, "sph_batch_wait_reads") ? 0 : -1;
}

namespace {
struct PhaseLog {
    cudaStream_t stream;
    std::vector<cudaEvent_t> events;
    std::vector<const char *> names;
    void mark(const char *name) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        cudaEventRecord(e, stream);
        events.push_back(e);
        names.push_back(name);
    }
};
}  // namespace

// Phase names of the batched solid passes, by material: the first pass
// goes under the material's name already marked.
struct SolidMarks {
    PhaseLog *log;
    bool corot;
    int seen;
};
static void solid_mark(void *ctx, const char *name) {
    SolidMarks *m = static_cast<SolidMarks *>(ctx);
    if (m->seen++ == 0 || !name) return;
    static const char *kCorot[][2] = {{"stresses", "corotational stresses"},
                                      {"forces_solids+step", "corotational forces+step"},
                                      {"step_forward", "corotational step (planes)"}};
    static const char *kSvk[][2] = {{"stresses", "svk stresses"},
                                    {"forces_solids+step", "svk forces+step"},
                                    {"step_forward", "svk step (planes)"}};
    const char *(*names)[2] = m->corot ? kCorot : kSvk;
    for (int k = 0; k < 3; ++k)
        if (!strcmp(names[k][0], name)) m->log->mark(names[k][1]);
}

extern "C" int sph_batch_profile(sph_batch *b, unsigned reps, float *phase_ms, const char **phase_names,
                                 unsigned max_phases) {
    if (!b) return -1;
    if (b->dirty && !rebuild(b)) return -1;
    if (!b->graph) return 0;
    static const char *kMat[3] = {"fluid forces+step", "corotational rotations", "svk deformations"};
    std::vector<double> acc;
    std::vector<const char *> names;
    for (unsigned r = 0; r < reps; ++r) {
        PhaseLog log{b->stream};
        Launch A = b->all;
        log.mark("bin_count");
        sph_launch_bin_count(A);
        log.mark("scan");
        sph_launch_scan(A, true);
        log.mark("insert");
        sph_launch_insert(A);
        log.mark("gather");
        sph_launch_gather(A, true, false, true);
        log.mark("density");
        sph_launch_density_fused(A, b->group[MAT_FLUID].present ? &b->group[MAT_FLUID].L : nullptr);
        for (int m = 0; m < 3; ++m) {
            if (!b->group[m].present) continue;
            Launch G = b->group[m].L;
            G.stream = b->stream;
            log.mark(kMat[m]);
            if (m == MAT_FLUID) {
                sph_launch_forces_fluids(G, true, true);
            } else {
                const bool corot = m == MAT_COROT;
                // the first phase is named by kMat; the others by the material
                SolidMarks sm{&log, corot, 0};
                sph_launch_solid_passes(G, corot, solid_mark, &sm);
            }
        }
        if (A.num_rigid) {
            log.mark("rigid bodies");
            sph_launch_rigid(A);
        }
        sph_launch_count_down(A);
        log.mark(nullptr);
        bool good = sph_check_launch("sph_batch_profile") == cudaSuccess &&
                    ok(cudaStreamSynchronize(b->stream), "sph_batch_profile");
        if (good && acc.empty()) {
            acc.assign(log.events.size() - 1, 0.0);
            names.assign(log.names.begin(), log.names.end() - 1);
        }
        for (size_t k = 0; good && k + 1 < log.events.size() && k < acc.size(); ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, log.events[k], log.events[k + 1]);
            acc[k] += ms;
        }
        for (cudaEvent_t e : log.events) cudaEventDestroy(e);
        if (!good) return -1;
    }
    unsigned np = (unsigned)acc.size() < max_phases ? (unsigned)acc.size() : max_phases;
    for (unsigned k = 0; k < np; ++k) {
        phase_ms[k] = reps ? (float)(acc[k] / reps) : 0.f;
        if (phase_names) phase_names[k] = names[k];
    }
    return (int)np;
}

extern "C" int sph_batch_synchronize(sph_batch *b) {
    if (!b) return -1;
    return ok(cudaStreamSynchronize(b->stream), "sph_batch_synchronize") ? 0 : -1;
}

extern "C" size_t sph_batch_bytes(sph_batch *b) { return b ? b->bytes + b->table_bytes : 0; }

extern "C" unsigned sph_batch_size(sph_batch *b) {
    if (!b) return 0;
    unsigned n = 0;
    for (BatchScene *s : b->slots) n += s != nullptr;
    return n;
}

extern "C" int sph_batch_tune(sph_batch *b, unsigned block, unsigned pair_block, unsigned grid_cap) {
    if (!b) return -1;
    auto valid = [](unsigned t, unsigned hi) { return t >= 32 && t <= hi && t % 32 == 0; };
    if (!valid(block, 1024) || !valid(pair_block, 512)) {
        sph_set_error("sph_batch_tune: block sizes must be multiples of 32, at most 1024 (512 for pair kernels)");
        return -1;
    }
    b->block = block;
    b->pair_block = pair_block;
    b->grid_cap = grid_cap;
    b->dirty = true;
    return 0;
}

extern "C" unsigned sph_batch_kernel_count(sph_batch *b) {
    if (!b) return 0;
    if (b->dirty && !rebuild(b)) return 0;
    return b->graph_kernels;
}

extern "C" void *sph_batch_stream(sph_batch *b) { return b ? (void *)b->stream : nullptr; }

extern "C" unsigned sph_batch_status(sph_batch *b, int id) {
    BatchScene *sc = scene_of(b, id, "sph_batch_status");
    if (!sc) return 0xFFFFFFFFu;
    unsigned v = 0;
    if (!ok(cudaMemcpyAsync(&v, sc->desc.status, 4, cudaMemcpyDeviceToHost, b->stream), "sph_batch_status") ||
        !ok(cudaStreamSynchronize(b->stream), "sph_batch_status"))
        return 0xFFFFFFFFu;
    return v;
}
