// store.h -- what a scene needs on the device, shared by the drop-in store
// (driver.cu) and the batched/served forms (batch.cu): the program list,
// field resolution against the reference's per-file field sets, the
// scratch arena and the segment-aware block maps.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "launch.h"
#include "sph_gb300.h"
#include "sph_internal.h"

// Parses a $opencl_kernel_files list ("common, fluids", ...).  Returns the
// SphProgram bits, or 0 with *err set.
unsigned sph_parse_programs(const char *file_list, std::string *err);

// Checks that the store holds every field the listed programs use, with
// the right element type and enough entries (the reference's program build
// fails when a field is missing), and fills desc's field pointers relative
// to the device blob `d_blob` (which may be null while only checking).
bool sph_resolve_scene(const psdata &host, char *d_blob, unsigned programs, SceneDesc *desc, std::string *err);

// Material recipe of a program set, or -1 when it has none.
int sph_material_of(unsigned programs);

// Byte sizes of a scene's scratch (sorted copies, slots, scan sums, queue,
// status) given its shape; `place` lays them out from `base`.
size_t sph_scratch_bytes(const SceneDesc &d);
void sph_place_scratch(SceneDesc *d, char *base);

// Rigid bodies of a host store (extension): the 1-based numbers of the
// bodies whose body_dynamic is SPH_BODY_RIGID, among the first body_count.
std::vector<unsigned> sph_rigid_bodies(const psdata &h, const SceneDesc &d);

// Block maps for a table of scenes (host vectors; BlockWork entries).
struct HostMaps {
    std::vector<BlockWork> particles, pair_particles, cells, scan;
};
void sph_build_maps(const std::vector<SceneDesc> &descs, const std::vector<unsigned> &scene_ids, unsigned block,
                    unsigned pair_block, HostMaps *out);

// A single cudaMalloc carved into 256-byte aligned pieces.
struct Arena {
    char *base = nullptr;
    size_t size = 0;
    static size_t align(size_t x) { return (x + 255) & ~(size_t)255; }
};

// Number of SMs of the current device (for persistent grid caps).
unsigned sph_sm_count();
