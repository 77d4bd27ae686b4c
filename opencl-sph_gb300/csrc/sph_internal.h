// sph_internal.h -- definitions shared by the host driver and the CUDA
// kernels of libsph_gb300.so (not part of the public ABI).
#pragma once

#include <stdint.h>

#include <vector_types.h>  // float4 (CUDA runtime headers)

// ---- errors ---------------------------------------------------------------

// Records a message for sph_last_error() (printf-style).
void sph_set_error(const char *fmt, ...);
// Aborts when abort-on-error is on (the reference's ASSERT behaviour).
void sph_fail();

// ---- materials ------------------------------------------------------------

// Kernel files named in a conf's $opencl_kernel_files list
// (src/opencl/particle_system_host.c:221-272 loads kernels/<name>.cl).
enum SphProgram : unsigned {
    PROG_COMMON = 1u << 0,            // kernels/common.cl
    PROG_FLUIDS = 1u << 1,            // kernels/fluids.cl
    PROG_SOLIDS = 1u << 2,            // kernels/solids.cl
    PROG_COROT = 1u << 3,             // kernels/solid_corotation.cl
    PROG_SVK = 1u << 4,               // kernels/solid_svk.cl
    PROG_CONSTRAINTS = 1u << 5,       // kernels/constraints.cl
    PROG_RIGIDBODY = 1u << 6,         // kernels/rigidbody.cl
};

// Device status word bits (sph_status()).
enum SphStatus : unsigned {
    STATUS_NONFINITE = 1u << 0,       // a non-finite position was written
    STATUS_OUTSIDE_GRID = 1u << 1,    // a particle was binned outside gridbounds
};

// Cells with more particles than this are ordered by the block-wide
// fallback sort instead of the per-cell insertion sort.
#define SPH_SMALL_CELL 32

// ---- one scene on the device ----------------------------------------------
//
// Pointers into the scene's device copy of its psdata blob (fields the
// program does not use may be null) plus the scratch the GB300 pipeline
// keeps beside it.  Scalars are read through their device pointers at run
// time, as the reference's USE_FIELD_FIRST_VALUE does, so a host-to-device
// sync of a scalar takes effect at the next launch.
struct SceneDesc {
    // scalars (device pointers)
    const unsigned *n;
    const float *mass, *timestep, *h, *restdens, *stiffness, *viscosity;
    const float *youngs_modulus, *poisson;
    const float *gravity, *gridbounds;
    const float *wallbounds;  // optional reflective box (extension)
    // particle fields
    float *position, *velocity, *acceleration, *force;
    float *density, *density0, *originalpos;
    float *rotation, *strain, *stress, *apq_temp, *intermediate, *deformation;
    float *cutoff_force, *force_elastic, *force_viscous;
    unsigned *num_neighbours;
    // neighbour grid fields
    unsigned *gridcell, *gridcount, *celloffset, *cellparticles;
    // planes and bodies
    const float *symmetry_planes, *plane_constraints;
    const unsigned *plane_constraints_particles;
    const unsigned *body_number, *body_dynamic, *body_count;
    float *body_position, *body_euler_rotation;
    // mixed fluid-solid scenes (extension; null otherwise): per particle 0
    // = fluid (fluids.cl's law), 1 = elastic solid (solid_svk.cl's law),
    // and the solids' own viscosity (the store's `viscosity` when absent)
    const unsigned *phase;
    const float *solid_viscosity;
    // shape, fixed when the store is created
    unsigned pnum;
    unsigned gridres[3];
    unsigned num_cells;
    unsigned num_symmetry_planes;
    unsigned num_plane_constraints;
    unsigned body_capacity;
    unsigned programs;        // SphProgram bits
    unsigned jacobi_guard;    // 1: Givens angle 0 when the pivot is exactly 0
    // scratch (device)
    unsigned *slot;           // per particle: arrival slot within its cell
    float4 *spos;             // cell-sorted (x, y, z, 0) positions
    float4 *svel;             // cell-sorted velocities
    float *sdens;             // cell-sorted densities
    unsigned *scan_sums;      // this scene's scan partial sums
    unsigned num_scan_blocks;
    unsigned *big_cells;      // [0] = count, [1..] = cells above SPH_SMALL_CELL
    unsigned *status;         // SphStatus bits
    // candidate masks (fluids, fused substep): bit t of stencil row r's
    // 64-bit mask of sorted particle k is set when the row's t-th candidate
    // lies within h; low word at nbmask[(2r) * pnum + k], high word at
    // nbmask[(2r+1) * pnum + k] (written only for rows of more than 32
    // candidates); ncand[k] = candidate count, or SPH_NCAND_SCAN when a row
    // exceeds 64 and the force pass must scan
    unsigned *nbmask;
    unsigned *ncand;
    // solids: cell-sorted copies for the fused substep's pair passes --
    // rest position (w: body_number bits), stress (6 floats, then
    // mass/density), rotation (3 rows of 4 floats); the velocity copy
    // carries 1/density0 in w
    float4 *spos0, *sstress, *srot;
    // batched form only (null otherwise): substeps this scene still takes;
    // at 0 every kernel skips the scene, SPH_STEPS_UNLIMITED never expires
    unsigned *steps_left;
    // rigid bodies (extension; present when the store has body fields):
    // per body SPH_RIGID_STRIDE doubles of state, the reduction's per-block
    // partial sums, and each rigid particle's offset from its body's centre
    // in the body frame
    double *rigid_state;
    double *rigid_partial;
    float4 *rigid_offset;
};

// body_dynamic value that makes a body rigid (extension): its particles
// move with the body's rigid motion, driven by the sum of their forces.
// 0 (fixed) and any other value (free particles) keep the reference's
// meaning.
#define SPH_BODY_RIGID 2u
// In a mixed fluid-solid scene (extension) the sorted rest-position copy's
// w lane holds the body number's bits with this bit set for a solid-phase
// particle.
#define SPH_SOLID_PHASE_BIT 0x80000000u
#define SPH_RIGID_BLOCKS 32     // reduction blocks per body
#define SPH_RIGID_THREADS 256
#define SPH_RIGID_Q 24          // reduced quantities per body
#define SPH_RIGID_STRIDE 64     // doubles of state per body

// One rigid body of one scene (body is 1-based, as body_number).
struct RigidWork {
    unsigned scene;
    unsigned body;
};

#define SPH_STEPS_UNLIMITED 0xffffffffu

// Candidate masks: two words for each of the 9 stencil rows.
#define SPH_MASK_WORDS 18
#define SPH_NCAND_SCAN 0xffffffffu

// Block map entry: block b of a launch works on `scene`, items
// [first, first + block size).
struct BlockWork {
    unsigned scene;
    unsigned first;
};

struct BlockMap {
    const BlockWork *work;
    unsigned num;
};

#define SPH_SCAN_TILE 2048      // cells per scan block (256 threads x 8)
#define SPH_SCAN_THREADS 256
