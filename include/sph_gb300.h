/*
 * sph_gb300.h -- C ABI of libsph_gb300.so, the GB300 (sm_103a) implementation
 * of the opencl-sph per-substep particle pipeline.
 *
 * Every declaration below either replaces one function of the reference's
 * libSPH.so (its header and line are cited beside it) or is an addition
 * marked NEW.  Types and struct layouts are those of the reference, so the
 * reference's ctypes bindings (scripts/sph/bindings.py) and its Python
 * driver code can load this library unchanged; the `_opencl` names are kept
 * as aliases of the `_cuda` ones.  No torch or CUDA type appears here: the
 * device side is reached only through the opaque handle below.
 *
 * Error behaviour follows the reference: void functions that fail record a
 * message (sph_last_error) and, unless sph_set_abort_on_error(0) was called,
 * abort the process as the reference's ASSERT/HANDLE_CL_ERROR do; int
 * functions return non-zero.  Kernel launches are asynchronous on the
 * handle's CUDA stream; every sync_* call, sph_synchronize and the
 * free/terminate calls wait for the stream, so host views of the psdata
 * blob are current after a device-to-host sync exactly as in the reference.
 */
#ifndef SPH_GB300_H_
#define SPH_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- store types ---------------------------------------------------------- */

/* src/datatypes.h:7-14 */
typedef enum { T_CHAR, T_UINT, T_INT, T_FLOAT32, T_FLOAT64, TYPE_COUNT } FieldType;

/* src/datatypes.h:16-26 */
typedef struct {
    FieldType type;
    union {
        char *c;
        uint32_t *u;
        int32_t *i;
        float *f4;
        double *f8;
        void *ptr;
    };
} DataPtr;

/* src/particle_system.h:18-48: a flat, self-describing particle store.
 * Field f occupies data_sizes[f] bytes at data + data_offsets[f]; its shape
 * is dimensions[dimensions_offsets[f] .. + num_dimensions[f]] (first
 * dimension fastest). */
typedef struct {
    unsigned int num_fields;
    const char *names;
    unsigned int *names_offsets;
    unsigned int *dimensions;
    unsigned int *num_dimensions;
    unsigned int *dimensions_offsets;
    unsigned int *entry_sizes;

    void *data;
    unsigned int *data_sizes;
    unsigned int *data_offsets;

    DataPtr *data_ptrs;

    unsigned int num_host_fields;
    char **host_names;
    void **host_data;
    unsigned int *host_data_size;
} psdata;

/* src/opencl/particle_system_host.h:7-47, same member layout.  Each cl_mem
 * slot holds a CUDA device pointer (or NULL), the kernel slots are unused,
 * and ps_prog holds the opaque per-store device state (stream, resolved
 * field table, material pipeline, scratch, CUDA graph).  The struct is
 * passed by value, like the reference's; copies share the device state. */
typedef struct {
    psdata host_psdata;

    unsigned int num_fields;
    void *names;
    void *names_offsets;
    void *dimensions;
    void *num_dimensions;
    void *dimensions_offsets;
    void *field_types;
    void *entry_sizes;

    void *data;              /* device copy of the whole psdata blob */
    void *data_sizes;
    void *data_offsets;

    void *block_totals;      /* device scratch: scan partial sums */
    void *backup_prefix_sum; /* device scratch: per-particle slot in its cell */

    size_t num_kernels;
    const char *const *kernel_names;
    const void *kernels;

    void *ps_prog;           /* opaque device state */

    unsigned int num_grid_cells;
    size_t po2_workgroup_size;
    unsigned int num_blocks;
} psdata_cuda;

typedef psdata_cuda psdata_opencl;

/* ---- host store: src/build_psdata.h, src/particle_system.h --------------- */

void build_psdata_from_string(psdata *data, const char *string);   /* build_psdata.h:6 */
void build_psdata(psdata *data, const char *path);                  /* build_psdata.h:7 */
void display_psdata(psdata data, const char *const *mask);          /* particle_system.h:56 */
int get_field_psdata(psdata data, const char *name);                /* particle_system.h:61 */
void set_field_psdata(psdata *data, const char *name, void *field,  /* particle_system.h:62 */
                      unsigned int size, unsigned int offset);
unsigned int psdata_names_size(psdata data);                        /* particle_system.h:64 */
unsigned int psdata_dimensions_size(psdata data);                   /* particle_system.h:65 */
unsigned int psdata_data_size(psdata data);                         /* particle_system.h:66 */
int create_host_field_psdata(psdata *data, const char *name,        /* particle_system.h:68 */
                             void *field, unsigned int size);
int get_host_field_psdata(psdata *data, const char *name);          /* particle_system.h:69 */
void free_psdata(psdata *data);                                     /* particle_system.h:77 */

/* ---- config and logging: src/config.h, src/note.h ------------------------ */

int load_config(const char *relative_path);                         /* config.h:4 */
const char *get_config_section(const char *heading);                /* config.h:5 */
void unload_config(void);                                           /* config.h:6 */
void set_log_level(unsigned int loglevel);                          /* note.h:4 */
void note(unsigned int level, const char *fmt, ...);                /* note.h:5 */

/* ---- device driver: src/opencl/particle_system_host.h -------------------- */

void init_cuda(void);                                               /* :55 init_opencl */
void terminate_cuda(void);                                          /* :60 terminate_opencl */
psdata_cuda create_psdata_cuda(psdata *data, const char *file_list);/* :56 create_psdata_opencl */
void free_psdata_cuda(psdata_cuda *pso);                            /* :59 free_psdata_opencl */

void sync_psdata_device_to_host(psdata data, psdata_cuda pso);      /* :62 */
void sync_psdata_fields_device_to_host(psdata data, psdata_cuda pso,/* :63 */
                                       size_t num_fields, const char *const *field_names);
void sync_psdata_host_to_device(psdata data, psdata_cuda pso, int full);              /* :64 */
void sync_psdata_fields_host_to_device(psdata data, psdata_cuda pso,/* :65 */
                                       size_t num_fields, const char *const *field_names);

void populate_position_cuboid_device_cuda(psdata_cuda pso,          /* :67-72 */
                                          float x1, float y1, float z1,
                                          float x2, float y2, float z2,
                                          unsigned int xsize, unsigned int ysize,
                                          unsigned int zsize);
void rotate_particles_device_cuda(psdata_cuda pso, float angle_x,   /* :73 */
                                  float angle_y, float angle_z);
void call_for_all_particles_device_cuda(psdata_cuda pso,            /* :74 */
                                        const char *kernel_name);
void compute_particle_bins_device_cuda(psdata_cuda pso);            /* :76 */
void compute_density_device_cuda(psdata_cuda pso);                  /* :78 */
void compute_forces_device_cuda(psdata_cuda pso);                   /* :79 */
void step_forward_device_cuda(psdata_cuda pso);                     /* :80 */
/* particle_system_host.c:562-588 (defined but not declared there) */
void set_body_position_device_cuda(psdata_cuda pso, unsigned int body, float *position);
void set_body_rotation_device_cuda(psdata_cuda pso, unsigned int body, float *euler_angles);

/* the reference's own names, aliases of the above */
void init_opencl(void);
void terminate_opencl(void);
psdata_opencl create_psdata_opencl(psdata *data, const char *file_list);
void free_psdata_opencl(psdata_opencl *pso);
void populate_position_cuboid_device_opencl(psdata_opencl pso, float x1, float y1, float z1,
                                            float x2, float y2, float z2, unsigned int xsize,
                                            unsigned int ysize, unsigned int zsize);
void rotate_particles_device_opencl(psdata_opencl pso, float angle_x, float angle_y, float angle_z);
void call_for_all_particles_device_opencl(psdata_opencl pso, const char *kernel_name);
void compute_particle_bins_device_opencl(psdata_opencl pso);
void compute_density_device_opencl(psdata_opencl pso);
void compute_forces_device_opencl(psdata_opencl pso);
void step_forward_device_opencl(psdata_opencl pso);
void set_body_position_device_opencl(psdata_opencl pso, unsigned int body, float *position);
void set_body_rotation_device_opencl(psdata_opencl pso, unsigned int body, float *euler_angles);

/* ---- NEW: errors, streams, whole substeps -------------------------------- */

/* Message of the last failure in this process ("" if none). */
const char *sph_last_error(void);
void sph_clear_error(void);
/* 1 (default, the reference's behaviour): a failing void call aborts.
 * 0: it records the error and returns. */
void sph_set_abort_on_error(int abort_on_error);
/* Waits for the store's stream and its reads (sph_read_fields_async);
 * returns 0 or a non-zero CUDA error. */
int sph_synchronize(psdata_cuda pso);
/* Page-locks the host store `data` (the psdata the device store mirrors) so
 * that copies to and from it run on the copy engines without a staging
 * copy; the library ends the registration on sph_unpin_host or
 * free_psdata_cuda, which must come before the blob is freed.  One host
 * store per device store.  Returns 0 or -1. */
int sph_pin_host(psdata data, psdata_cuda pso);
int sph_unpin_host(psdata_cuda pso);
/* sync_psdata_fields_host_to_device (particle_system_host.c:812-829)
 * without the wait: the copies are enqueued on the store's stream, so the
 * named fields of `data` must stay unchanged until the stream has passed
 * them (a later blocking call or sph_synchronize).  An unknown name is
 * logged and skipped, as in the blocking sync.  Returns 0 or -1. */
int sph_write_fields_async(psdata data, psdata_cuda pso, size_t num_fields, const char *const *names);
/* sync_psdata_fields_device_to_host (particle_system_host.c:843-858)
 * without the wait: the fields are copied to a device snapshot in stream
 * order (after the substeps enqueued so far), and a side stream copies the
 * snapshot into `data` (one cudaMemcpyAsync per field) while later
 * substeps run.  Returns a ticket (>= 0), or -1.  `data` holds the
 * snapshot after sph_wait_read(ticket); its named fields must not be used
 * until then, and a later read writes them again, so enqueue it after the
 * previous snapshot has been used.  Two reads are in flight at most: a
 * third waits, on the device, for the first to finish.  Every blocking
 * sync_* call first waits for the reads in flight. */
long long sph_read_fields_async(psdata data, psdata_cuda pso, size_t num_fields, const char *const *names);
int sph_wait_read(psdata_cuda pso, long long ticket);
/* Waits for every read enqueued so far. */
int sph_wait_reads(psdata_cuda pso);
/* Runs `num_steps` substeps of the store's material recipe (the sequence a
 * reference driver issues through call_for_all_particles:
 * scripts/sph/systems.py:194-204 for corotational solids, :225-235 for SVK,
 * src/mex/simstep_fluid.c:18-23 for fluids), as one CUDA graph per substep
 * captured on first use.  Returns 0 or non-zero on failure. */
int sph_update(psdata_cuda pso, unsigned int num_steps);
/* Device status word accumulated since the last sph_clear_status():
 * bit 0 = a NaN/Inf position was written, bit 1 = a particle was binned
 * outside the grid bounds (and clamped into an edge cell). */
unsigned int sph_status(psdata_cuda pso);
void sph_clear_status(psdata_cuda pso);
/* The store's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events with the store's kernels. */
void *sph_stream(psdata_cuda pso);
/* Kernel launches in one sph_update substep of this store (the kernel
 * nodes of its CUDA graph; 0 before the first sph_update). */
unsigned int sph_graph_kernel_count(psdata_cuda pso);
/* Runs `reps` substeps of the store's recipe as individual launches (the
 * kernels sph_update's graph holds) with CUDA events between phases, and
 * writes each phase's mean device time in ms and its name.  Returns the
 * number of phases (at most max_phases), or -1 on failure. */
int sph_profile_substep(psdata_cuda pso, unsigned int reps, float *phase_ms, const char **phase_names,
                        unsigned int max_phases);
/* ---- NEW: device-resident recording --------------------------------------
 * Replaces the reference drivers' per-substep host copy of the whole store
 * (scripts/straintest.py:183-198 syncs every field to the host and appends
 * it to .npy memmaps; scripts/sph/systems.py:89-99).  sph_record_start
 * makes every later sph_update substep copy the named fields, on every
 * `every`-th substep, into a ring of `frames` frames in device memory;
 * the copy is part of the substep graph, so recording adds no host work or
 * synchronisation.  A frame is the fields' bytes concatenated in the given
 * order.  Frames are numbered from 0 in recording order; the ring holds
 * the last `frames` of them.  Returns 0, or -1 with sph_last_error set. */
int sph_record_start(psdata_cuda pso, size_t num_fields, const char *const *names, unsigned int every,
                     unsigned int frames);
int sph_record_stop(psdata_cuda pso);
/* Frames recorded so far (waits for the store's stream). */
unsigned long long sph_record_count(psdata_cuda pso);
size_t sph_record_frame_bytes(psdata_cuda pso);
/* Copies frames [first, first + count) into `host` (count x frame bytes). */
int sph_record_read(psdata_cuda pso, void *host, unsigned long long first, unsigned int count);

/* ---- NEW: batched and served forms ---------------------------------------
 * A batch holds many independent scenes resident on the device and
 * advances all of them together: every phase of the substep is one
 * segment-aware launch over all scenes (blocks map to (scene, first item)),
 * the material phases of fluid, corotational and SVK scenes run as
 * parallel branches, and the whole substep is one CUDA graph, recaptured
 * only when scenes are added or removed.  Scenes keep the psdata layout of
 * their host store; each scene's result is independent of the others in
 * the batch (the same kernels, order and arithmetic as alone). */
typedef struct sph_batch sph_batch;
sph_batch *sph_batch_create(void);
void sph_batch_free(sph_batch *batch);
/* Device bytes a scene will hold once added (blob + scratch). */
size_t sph_scene_bytes(psdata *scene, const char *file_list);
/* Uploads a scene (its current host values) and, for solids, runs the
 * setup of scripts/sph/systems.py:185-192.  Returns its id (>= 0) or -1. */
int sph_batch_add(sph_batch *batch, psdata *scene, const char *file_list);
/* A jittered lattice scene built on the device.  Particle p sits at
 * lattice point (p % nx, p / nx % ny, p / (nx ny)) * spacing + origin, each
 * coordinate plus jitter * (2u - 1) with u = splitmix64(seed * 2^32 + 3p +
 * axis) / 2^64 (its top 53 bits), computed in IEEE double and rounded to
 * float; sph/scenes.py's lattice(hash_seed=...) gives the same floats on
 * the host.  The first clamp_layers * nx * ny particles get body_number 1
 * (where the field exists); identity_rotation sets every rotation to I. */
typedef struct {
    unsigned int nx, ny, nz;
    unsigned int clamp_layers;
    unsigned int identity_rotation;
    double spacing, jitter;
    double origin[3];
    unsigned long long seed;
} sph_lattice;
/* sph_batch_add for a lattice scene built on the device: `scene` is a
 * freshly built host store (build_psdata) of at least nx ny nz particles.
 * Its fields of at most 4096 bytes (the conf's scalars and small arrays,
 * n, body_dynamic) are copied; the larger fields start at zero, as in a
 * freshly built store, except position, n (and body_number, rotation),
 * which `gen` writes.  The large host fields are never read or uploaded. */
int sph_batch_add_lattice(sph_batch *batch, psdata *scene, const char *file_list, const sph_lattice *gen);
/* Releases a scene's device memory (stream-ordered). */
int sph_batch_remove(sph_batch *batch, int id);
/* Advances every scene of the batch by num_steps substeps. */
int sph_batch_step(sph_batch *batch, unsigned int num_steps);
/* Substep quotas, for serving: a scene given a quota of `steps` takes part
 * in the next `steps` substeps of the batch and then stays idle -- every
 * kernel skips it, its store keeps its values -- until it gets a new
 * quota.  Scenes are added with SPH_BATCH_STEPS_UNLIMITED (never idle).
 * The write is stream-ordered after the work already enqueued. */
#define SPH_BATCH_STEPS_UNLIMITED 0xffffffffu
int sph_batch_set_steps(sph_batch *batch, int id, unsigned int steps);
/* The scene's remaining quota (waits for the batch's stream). */
unsigned int sph_batch_steps_left(sph_batch *batch, int id);
/* Copies a scene's device store into `out` (same layout as when added). */
int sph_batch_read(sph_batch *batch, int id, psdata *out);
/* Copies one named field of a scene into the same field of `out`. */
int sph_batch_read_field(sph_batch *batch, int id, const char *field, psdata *out);
/* The same copy enqueued on the batch's stream without waiting: `out` is
 * current after sph_batch_synchronize (and asynchronous only when its
 * blob is pinned, e.g. by cudaHostRegister). */
int sph_batch_read_field_async(sph_batch *batch, int id, const char *field, psdata *out);
/* Page-locks the host store `store` (of the scene's layout) for reads of
 * scene `id` (cudaHostRegister, mapped; a store the caller registered
 * already is used as it is).  Reads into it by sph_batch_read_field_many
 * then go through one copy kernel that writes the store directly.  The
 * registration ends with sph_batch_unpin_host, sph_batch_remove or
 * sph_batch_free, which must come before the store is freed. */
int sph_batch_pin_host(sph_batch *batch, int id, psdata *store);
int sph_batch_unpin_host(sph_batch *batch, int id);
/* Copies one named field of `count` scenes into the same field of their
 * stores outs[k] and waits: one kernel launch for all stores pinned with
 * sph_batch_pin_host, one cudaMemcpyAsync for each other store. */
int sph_batch_read_field_many(sph_batch *batch, const int *ids, unsigned int count, const char *field,
                              psdata *const *outs);
/* The same read without waiting, for stores pinned with sph_batch_pin_host:
 * the field is copied to a device snapshot in stream order (after the
 * substeps enqueued so far), and a side stream copies the snapshot into the
 * stores (one cudaMemcpyAsync each) while later substeps run.  Returns a ticket (>= 0), or -1.  The
 * stores hold the snapshot after sph_batch_wait_read(ticket); a later read
 * overwrites them.  Two reads are in flight at most: a third waits, on the
 * device, for the first to finish. */
long long sph_batch_read_field_many_async(sph_batch *batch, const int *ids, unsigned int count, const char *field,
                                          psdata *const *outs);
int sph_batch_wait_read(sph_batch *batch, long long ticket);
/* The write direction (the per-substep inputs a host controller sets, such
 * as each scene's time step or gravity): the named field of each host
 * store ins[k] is copied into scene ids[k], in stream order before the
 * substeps enqueued after this call.  The bytes are taken from the stores
 * during the call (into a page-locked staging buffer), so the stores may
 * change as soon as it returns; one scatter kernel, reading the staging
 * buffer over the host link, carries every scene's bytes.  gridres and pnum cannot be written
 * (they size the scene's tables), nor, in a scene with rigid bodies, the
 * fields the bodies are set up from (position, velocity, n, body tables).
 * Returns a non-negative count of writes so far, or -1. */
int sph_batch_write_field_many_async(sph_batch *batch, const int *ids, unsigned int count, const char *field,
                                     psdata *const *ins);
/* The same for fields[0 .. nfields) at once: one staging buffer, one
 * host-to-device copy and one scatter kernel for every field of every
 * scene (a controller's per-substep inputs, e.g. time step and gravity). */
int sph_batch_write_fields_many_async(sph_batch *batch, const int *ids, unsigned int count, unsigned int nfields,
                                      const char *const *fields, psdata *const *ins);
/* Waits for every read enqueued so far. */
int sph_batch_wait_reads(sph_batch *batch);
/* Runs `reps` substeps of the batch as individual launches with CUDA events
 * between phases (material branches one after another) and writes each
 * phase's mean device time in ms and its name; returns the phase count. */
int sph_batch_profile(sph_batch *batch, unsigned int reps, float *phase_ms, const char **phase_names,
                      unsigned int max_phases);
int sph_batch_synchronize(sph_batch *batch);
/* Device bytes held by the batch's scenes and tables. */
size_t sph_batch_bytes(sph_batch *batch);
unsigned int sph_batch_size(sph_batch *batch);
/* Launch shape: threads per block for particle/cell kernels (32..1024) and
 * for pair kernels (32..512), multiples of 32, and the persistent-grid cap
 * (0: one block per work item). */
int sph_batch_tune(sph_batch *batch, unsigned int block, unsigned int pair_block, unsigned int grid_cap);
unsigned int sph_batch_kernel_count(sph_batch *batch);
void *sph_batch_stream(sph_batch *batch);
unsigned int sph_batch_status(sph_batch *batch, int id);

/* ---- NEW: neighbour grid without allocation -------------------------------
 * No counterpart in the reference.  compute_particle_bins for callers that
 * cannot allocate device memory: engines and plugin hosts whose own pool
 * owns all device memory and forbids other allocations in their frame
 * loop, and real-time loops that cannot afford the implicit device
 * synchronisation of cudaMalloc/cudaFree.  The caller passes device
 * buffers: positions (AoS float[3] x n), gridbounds (6 floats), and the
 * outputs gridcell[n], gridcount[rx*ry*rz], celloffset[rx*ry*rz],
 * cellparticles[n], with the meanings and layout of the store fields of the
 * same names.  `status`, when not NULL, is a device word into which the
 * call ORs its status bits (those of sph_status: bit 1 = a particle lay
 * outside gridbounds and was clamped into an edge cell); NULL drops them.
 * The scratch is a fixed file-scope device array (about 12.3 MB, held by
 * every GPU that loads the library until the process exits), so
 * n <= SPH_NOALLOC_MAX_PARTICLES and rx*ry*rz <= SPH_NOALLOC_MAX_CELLS;
 * larger sizes return -1 with an error message.  The call allocates
 * nothing, enqueues on `stream` (a cudaStream_t, NULL for the default
 * stream) and returns 0.  Calls share the array and each starts by
 * clearing what must start at zero: calls that overlap on the GPU race, so
 * order them on one stream.  The first call on a device looks up the
 * array's address with that device current; make it before any stream
 * capture.  The address is looked up again on every call whose stream is
 * not capturing, so a context made anew (after cudaDeviceReset) is served;
 * one context per device is assumed. */
#define SPH_NOALLOC_MAX_PARTICLES (1u << 20)
#define SPH_NOALLOC_MAX_CELLS (1u << 22)
int sph_compute_particle_bins_noalloc(const float *position, unsigned int n, const float *gridbounds,
                                      unsigned int rx, unsigned int ry, unsigned int rz,
                                      unsigned int *gridcell, unsigned int *gridcount,
                                      unsigned int *celloffset, unsigned int *cellparticles,
                                      unsigned int *status, void *stream);

/* Library and device description (static string). */
const char *sph_version(void);

#ifdef __cplusplus
}
#endif

#endif
