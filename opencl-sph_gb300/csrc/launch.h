// launch.h -- host-side entry points that enqueue the sm_103a kernels of
// the pipeline on a stream.  Every function works on a table of scenes
// (one for the drop-in store, many for a batch) through segment-aware
// block maps; none allocates memory or synchronises.
#pragma once

#include <cuda_runtime.h>

#include "sph_internal.h"

struct Launch {
    const SceneDesc *scenes;  // device table
    unsigned num_scenes;
    BlockMap particles;       // `block` items per entry
    BlockMap cells;           // `block` cells per entry
    BlockMap scan;            // SPH_SCAN_TILE cells per entry
    unsigned block;           // threads per block for particle/cell kernels
    unsigned pair_block;      // threads per block for the pair kernels
    BlockMap pair_particles;  // `pair_block` items per entry
    unsigned grid_cap;        // upper bound on blocks per launch (persistent loop)
    cudaStream_t stream;
    // no scene of the table has symmetry planes: the density pass's plane
    // variant is not launched (false is always safe)
    bool no_symmetry_planes;
    // rigid bodies of the table (device list; none when num_rigid is 0)
    const RigidWork *rigid;
    unsigned num_rigid;
    // some scene of the table is a mixed fluid-solid scene (its phase
    // field is set): the mixed kernels are launched too
    bool has_mixed;
    // every scene of the table is mixed: the plain-fluid instantiations,
    // which skip mixed scenes, are not launched (false is always safe)
    bool all_mixed;
};

// At most this many rigid bodies per launch (the reduction grid's y extent).
#define SPH_MAX_RIGID_WORK 65535u

// MAT_MIXED: fluid and St. Venant-Kirchhoff particles in one scene, told
// apart by the `phase` field (extension; plain stores only)
enum SphMaterial { MAT_FLUID = 0, MAT_COROT = 1, MAT_SVK = 2, MAT_MIXED = 3 };

// Neighbour grid, the reference's kernels one by one.
void sph_launch_find_bins(const Launch &L);
void sph_launch_zero_cells(const Launch &L);
void sph_launch_count(const Launch &L);
// sums_ready: k_bin_count has added up the tiles' totals (a fused binning);
// otherwise a pass over the counts does (prefix_sum called by name)
void sph_launch_scan(const Launch &L, bool sums_ready = false);
void sph_launch_insert(const Launch &L);  // scatter + per-cell ordering
// zero_gridcount + find_particle_bins + count_particles_in_bins in one
// pass, recording each particle's arrival slot
void sph_launch_bin_count(const Launch &L);
// All of compute_particle_bins: zero, bin+count, scan, insert.
void sph_launch_bins(const Launch &L);
// Cell-sorted copies (positions; velocities and densities on request).
void sph_launch_gather(const Launch &L, bool vel, bool dens, bool solid = false);

// skip_solids: a fused substep, where a plane-free solid's first solid pass
// sums its density
// mask: record the candidate masks (fused substeps); count: count
// num_neighbours in the masked pass too (a named compute_density)
void sph_launch_density(const Launch &L, bool original, bool mask = false, bool skip_solids = false,
                        bool count = false);
// The fused batched density: the plane-free instantiation over `fluids`'
// pair map only (plane-free solids sum their density in their first solid
// pass), the plane instantiation over every scene of L when some has
// planes.  `fluids` is null when the batch has no fluid scene.
void sph_launch_density_fused(const Launch &L, const Launch *fluids);
void sph_launch_forces_fluids(const Launch &L, bool fuse_step, bool masked = false);
// planes_only: skip plane-free scenes (a fused substep's solid force pass
// stepped them)
void sph_launch_step_forward(const Launch &L, bool planes_only = false);
void sph_launch_plane_constraints(const Launch &L);
void sph_launch_init_original_position(const Launch &L);
// with_density: also the density pass's sums (fused substeps); with_stress:
// also the stress law and the sorted stress copies of plane-free scenes
// (fused substeps, with_density too)
void sph_launch_rotations_and_strains(const Launch &L, bool with_density = false, bool with_stress = false);
// sorted: a fused substep's stress pass, which also fills the sorted copy;
// planes_only: only scenes with symmetry planes (the first pass stored the
// others' stresses)
void sph_launch_stresses(const Launch &L, bool corot, bool sorted = false, bool planes_only = false);
void sph_launch_deformations(const Launch &L, bool with_density = false, bool with_stress = false);
// masked: a fused substep's force pass over the first pair pass's masks;
// fuse_step: also step_forward for the plane-free scenes it covers
void sph_launch_forces_solids(const Launch &L, bool corot, bool masked = false, bool fuse_step = false);

// Mixed fluid-solid scenes: rest density, deformation gradient and the
// elastic pair forces of the solid particles over their solid neighbours
// (the force pass of fluids.cl then adds the fluid-solid pair terms).
void sph_launch_original_density_mixed(const Launch &L);
void sph_launch_deformations_mixed(const Launch &L, bool masked);
void sph_launch_forces_solids_mixed(const Launch &L);

void sph_launch_set_body_position(const Launch &L, unsigned body, const float pos[3]);
void sph_launch_set_body_rotation(const Launch &L, unsigned body, const float euler[3]);
void sph_launch_populate_cuboid(const Launch &L, const float c1[3], const float c2[3], const unsigned size[3]);
void sph_launch_rotate_particles(const Launch &L, float ax, float ay, float az);
// Device-resident recording: on every `every`-th substep the fields' word
// ranges of the store's blob are copied into the ring's next frame.  The
// counters live on the device, so the two launches sit in the substep graph.
struct RecordPlan {
    const uint2 *ranges;           // (word offset in the blob, word count) per field
    unsigned num_ranges;
    unsigned frame_words;
    const unsigned *blob;
    unsigned *ring;                // frames x frame_words
    unsigned frames, every;
    unsigned long long *counters;  // [0] substeps seen, [1] frames recorded
};
void sph_launch_record(const RecordPlan &p, cudaStream_t stream);

// Rigid bodies: force/torque sums, body substep and particle placement
// (after the material's step), and the reset that sets bodies up again
// from their particles' current state.
void sph_launch_rigid(const Launch &L);
void sph_launch_rigid_reset(const Launch &L);
// Batched form: the end-of-substep quota count-down over all scenes, and a
// stream-ordered write of one scene's quota.
void sph_launch_count_down(const Launch &L);
void sph_launch_set_steps(unsigned *steps_left, unsigned steps, cudaStream_t stream);

// A jittered lattice written into a scene on the device (the device form
// of the lattice scene builders): particle p sits at lattice point
// (p % nx, p / nx % ny, p / (nx ny)) * spacing + origin, each coordinate
// plus jitter * (2u - 1), u = splitmix64(seed * 2^32 + 3p + axis) / 2^64
// (53 bits), in IEEE double, rounded to float.  The first clamp_layers
// nx ny particles get body_number 1; identity_rotation sets rotation = I.
struct LatticeGen {
    unsigned nx, ny, nz, clamp_layers, identity_rotation;
    double spacing, jitter, origin[3];
    unsigned long long seed;
};
void sph_launch_lattice(const SceneDesc &d, const LatticeGen &g, cudaStream_t stream);

// One byte range to copy (device to device or to mapped host memory).
struct CopySeg {
    const char *src;
    char *dst;
    unsigned long long bytes;
};
// A few segments passed by value (no table to upload first): a store's
// small per-substep writes, read by the kernel from the mapped pinned host
// store, so they take no copy engine (a host-to-device copy would queue
// behind the device-to-host copies of the reads in flight).
#define SPH_INLINE_SEGS 8
struct InlineSegs {
    CopySeg seg[SPH_INLINE_SEGS];
    unsigned count;
};
void sph_launch_copy_inline(const InlineSegs &segs, cudaStream_t stream);
// Copies segs[0 .. count) (a device table) in one launch per 65,535
// segments; `max_bytes` is the largest segment.
void sph_launch_copy_segments(const CopySeg *segs, unsigned count, unsigned long long max_bytes,
                              cudaStream_t stream);

// One substep of a material's recipe for every scene of the launch.  All
// scenes of L must share the material (batches launch one Launch per
// material group).  `mark`, when given, is called with each phase's name
// before the phase is enqueued and with nullptr after the last one.
typedef void (*PhaseMark)(void *ctx, const char *phase);
void sph_launch_substep(const Launch &L, SphMaterial mat, PhaseMark mark = nullptr, void *ctx = nullptr);
// A fused substep's solid passes after the density pass: the first pass
// (with the density sums and the stresses), the forces with the step, and
// the separate stress and step passes for scenes with symmetry planes.
// `mark` names each phase.
void sph_launch_solid_passes(const Launch &L, bool corot, PhaseMark mark = nullptr, void *ctx = nullptr);

// One-time kernel attributes (call outside any stream capture).
cudaError_t sph_prepare_kernels();

// cudaGetLastError() after the enqueues above; records and returns it.
cudaError_t sph_check_launch(const char *what);
