// kernels.cu -- the sm_103a kernels of the per-substep particle pipeline
// and the host functions that enqueue them (see launch.h).
#include <stdio.h>

#include "kernels_fluid.cuh"
#include "kernels_grid.cuh"
#include "kernels_mixed.cuh"
#include "kernels_rigid.cuh"
#include "kernels_solid.cuh"
#include "launch.h"

static inline unsigned grid_for(const BlockMap &m, unsigned cap) {
    unsigned g = m.num < cap ? m.num : cap;
    return g ? g : 1;
}

cudaError_t sph_prepare_kernels() {
    // the staged density pass may use more than the default 48 KB of
    // dynamic shared memory for large pair blocks
    int dev = 0, max_optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    size_t want = density_smem_bytes(1024);
    if (max_optin > 0 && want > (size_t)max_optin) want = (size_t)max_optin;
    cudaError_t e = cudaFuncSetAttribute(k_density<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_density<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_density<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_density<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want);
    return e;
}

cudaError_t sph_check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) sph_set_error("%s: %s", what, cudaGetErrorString(e));
    return e;
}

void sph_launch_find_bins(const Launch &L) {
    k_bin_count<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles, 0);
}

void sph_launch_zero_cells(const Launch &L) {
    k_zero_cells<<<grid_for(L.scan, L.grid_cap), SPH_SCAN_THREADS, 0, L.stream>>>(L.scenes, L.scan);
}

void sph_launch_count(const Launch &L) {
    k_count_only<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles);
}

void sph_launch_scan(const Launch &L, bool sums_ready) {
    if (!sums_ready)
        k_scan_reduce<<<grid_for(L.scan, L.grid_cap), SPH_SCAN_THREADS, 0, L.stream>>>(L.scenes, L.scan);
    k_scan_down<<<grid_for(L.scan, L.grid_cap), SPH_SCAN_THREADS, 0, L.stream>>>(L.scenes, L.scan);
}

void sph_launch_insert(const Launch &L) {
    k_scatter<<<wide_grid(L.particles.num, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles);
    k_rank_cells<<<wide_grid(L.particles.num, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles);
    // crowded cells are rare: a few blocks per scene walk its queue
    const unsigned gy = L.num_scenes < 65535u ? (L.num_scenes ? L.num_scenes : 1u) : 65535u;
    // (a batch: 4 blocks of 256 per scene, most of which find no queue)
    if (L.num_scenes > 1)
        k_sort_big_cells<<<dim3(4, gy), 256, 0, L.stream>>>(L.scenes, L.num_scenes);
    else
        k_sort_big_cells<<<dim3(32, gy), 1024, 0, L.stream>>>(L.scenes, L.num_scenes);
}

void sph_launch_bin_count(const Launch &L) {
    sph_launch_zero_cells(L);
    k_bin_count<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles, 1);
}

void sph_launch_bins(const Launch &L) {
    sph_launch_bin_count(L);
    sph_launch_scan(L, true);
    sph_launch_insert(L);
}

void sph_launch_gather(const Launch &L, bool vel, bool dens, bool solid) {
    k_gather<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles, vel ? 1 : 0,
                                                                          dens ? 1 : 0, solid ? 1 : 0);
}

void sph_launch_density(const Launch &L, bool original, bool mask, bool skip_solids, bool count) {
    const size_t smem = density_smem_bytes(L.pair_block);
    const unsigned g = grid_for(L.pair_particles, L.grid_cap);
    const int o = original ? 1 : 0, m = mask ? 1 : 0, sk = skip_solids ? 1 : 0;
    if (mask && count) {
        k_density<false, true><<<g, L.pair_block, smem, L.stream>>>(L.scenes, L.pair_particles, o, m, sk);
        if (!L.no_symmetry_planes)
            k_density<true, true><<<g, L.pair_block, smem, L.stream>>>(L.scenes, L.pair_particles, o, m, 0);
        return;
    }
    k_density<false><<<g, L.pair_block, smem, L.stream>>>(L.scenes, L.pair_particles, o, m, sk);
    if (!L.no_symmetry_planes) k_density<true><<<g, L.pair_block, smem, L.stream>>>(L.scenes, L.pair_particles, o, m, 0);
}

void sph_launch_density_fused(const Launch &L, const Launch *fluids) {
    const size_t smem = density_smem_bytes(L.pair_block);
    if (fluids && fluids->pair_particles.num)
        k_density<false><<<grid_for(fluids->pair_particles, L.grid_cap), L.pair_block, smem, L.stream>>>(
            L.scenes, fluids->pair_particles, 0, 1, 1);
    if (!L.no_symmetry_planes)
        k_density<true><<<grid_for(L.pair_particles, L.grid_cap), L.pair_block, smem, L.stream>>>(
            L.scenes, L.pair_particles, 0, 1, 0);
}

void sph_launch_forces_fluids(const Launch &L, bool fuse_step, bool masked) {
    const unsigned g = grid_for(L.pair_particles, L.grid_cap);
    const int step = fuse_step ? 1 : 0;
    if (masked) {
        if (!L.all_mixed)
            k_forces_fluids_masked<false><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, step);
        if (L.has_mixed)
            k_forces_fluids_masked<true><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, step);
    } else {
        if (!L.all_mixed) k_forces_fluids<false><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, step);
        if (L.has_mixed) k_forces_fluids<true><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, step);
    }
}

void sph_launch_original_density_mixed(const Launch &L) {
    k_original_density_mixed<<<grid_for(L.pair_particles, L.grid_cap), L.pair_block, 0, L.stream>>>(
        L.scenes, L.pair_particles);
}

void sph_launch_deformations_mixed(const Launch &L, bool masked) {
    k_deformations_mixed<<<grid_for(L.pair_particles, L.grid_cap), L.pair_block, 0, L.stream>>>(
        L.scenes, L.pair_particles, masked ? 1 : 0);
}

void sph_launch_forces_solids_mixed(const Launch &L) {
    k_forces_solids_mixed<<<grid_for(L.pair_particles, L.grid_cap), L.pair_block, 0, L.stream>>>(
        L.scenes, L.pair_particles);
}

void sph_launch_step_forward(const Launch &L, bool planes_only) {
    k_step_forward<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles,
                                                                                planes_only ? 1 : 0);
}

void sph_launch_plane_constraints(const Launch &L) {
    k_plane_constraints<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles);
}

void sph_launch_init_original_position(const Launch &L) {
    k_init_original_position<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles);
}

void sph_launch_rotations_and_strains(const Launch &L, bool with_density, bool with_stress) {
    const unsigned g = grid_for(L.pair_particles, L.grid_cap);
    k_rotations_and_strains<<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, with_density ? 1 : 0,
                                                              with_density && with_stress ? 1 : 0);
    if (!L.no_symmetry_planes)
        k_rotations_and_strains_planes<<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles);
}

void sph_launch_stresses(const Launch &L, bool corot, bool sorted, bool planes_only) {
    const unsigned g = grid_for(L.particles, L.grid_cap);
    if (sorted) {
        if (corot) k_stresses_sorted<true><<<g, L.block, 0, L.stream>>>(L.scenes, L.particles, planes_only ? 1 : 0);
        else k_stresses_sorted<false><<<g, L.block, 0, L.stream>>>(L.scenes, L.particles, planes_only ? 1 : 0);
    } else {
        if (corot) k_stresses_corot<<<g, L.block, 0, L.stream>>>(L.scenes, L.particles);
        else k_stresses_svk<<<g, L.block, 0, L.stream>>>(L.scenes, L.particles);
    }
}

void sph_launch_deformations(const Launch &L, bool with_density, bool with_stress) {
    const unsigned g = grid_for(L.pair_particles, L.grid_cap);
    k_deformations<<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, with_density ? 1 : 0,
                                                     with_density && with_stress ? 1 : 0);
    if (!L.no_symmetry_planes) k_deformations_planes<<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles);
}

void sph_launch_forces_solids(const Launch &L, bool corot, bool masked, bool fuse_step) {
    const unsigned g = grid_for(L.pair_particles, L.grid_cap);
    const int step = masked && fuse_step ? 1 : 0;
    if (corot) {
        if (masked) k_forces_solids<true, true><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, step);
        else k_forces_solids<true, false><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, 0);
        if (!L.no_symmetry_planes)
            k_forces_solids_planes<true><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles);
    } else {
        if (masked) k_forces_solids<false, true><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, step);
        else k_forces_solids<false, false><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles, 0);
        if (!L.no_symmetry_planes)
            k_forces_solids_planes<false><<<g, L.pair_block, 0, L.stream>>>(L.scenes, L.pair_particles);
    }
}

void sph_launch_solid_passes(const Launch &L, bool corot, PhaseMark mark, void *ctx) {
    auto phase = [&](const char *name) {
        if (mark) mark(ctx, name);
    };
    const bool planes = !L.no_symmetry_planes;
    phase(corot ? "rotations_and_strains" : "deformations");
    if (corot) sph_launch_rotations_and_strains(L, true, true);
    else sph_launch_deformations(L, true, true);
    if (planes) {
        phase("stresses");
        sph_launch_stresses(L, corot, true, true);
    }
    phase("forces_solids+step");
    sph_launch_forces_solids(L, corot, true, true);
    if (planes) {
        phase("step_forward");
        sph_launch_step_forward(L, true);
    }
}

void sph_launch_set_body_position(const Launch &L, unsigned body, const float pos[3]) {
    float3 p = make_float3(pos[0], pos[1], pos[2]);
    k_set_body_position<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles, body, p);
    k_store_body_vec<<<1, 32, 0, L.stream>>>(L.scenes, 0, body, p);
}

void sph_launch_set_body_rotation(const Launch &L, unsigned body, const float euler[3]) {
    float3 e = make_float3(euler[0], euler[1], euler[2]);
    k_set_body_rotation<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles, body);
    k_store_body_vec<<<1, 32, 0, L.stream>>>(L.scenes, 1, body, e);
}

void sph_launch_populate_cuboid(const Launch &L, const float c1[3], const float c2[3], const unsigned size[3]) {
    dim3 block(8, 8, 4);
    dim3 grid((size[0] + 7) / 8, (size[1] + 7) / 8, (size[2] + 3) / 4);
    k_populate_cuboid<<<grid, block, 0, L.stream>>>(L.scenes, make_float3(c1[0], c1[1], c1[2]),
                                                    make_float3(c2[0], c2[1], c2[2]), make_uint3(size[0], size[1], size[2]));
}

void sph_launch_rotate_particles(const Launch &L, float ax, float ay, float az) {
    k_rotate_particles<<<grid_for(L.particles, L.grid_cap), L.block, 0, L.stream>>>(L.scenes, L.particles, ax, ay, az);
}

// The substep recipes a reference driver issues by name:
//   fluids: compute_particle_bins, compute_density, compute_forces_fluids,
//           step_forward (src/mex/simstep_fluid.c:18-23)
//   corotational solid: bins, compute_density,
//           compute_rotations_and_strains, compute_stresses,
//           compute_forces_solids, step_forward (scripts/sph/systems.py:194-204)
//   SVK solid: the same with compute_deformations (systems.py:225-235)
// Positions do not move between the bins and the integrator, so the sorted
// copies are gathered once, the force pass walks the candidate masks the
// density pass recorded, and for fluids the integrator is fused into the
// force pass.
void sph_launch_substep(const Launch &L, SphMaterial mat, PhaseMark mark, void *ctx) {
    auto phase = [&](const char *name) {
        if (mark) mark(ctx, name);
    };
    phase("bin_count");
    sph_launch_bin_count(L);
    phase("scan");
    sph_launch_scan(L, true);
    phase("insert");
    sph_launch_insert(L);
    if (mat == MAT_MIXED) {
        // fluid and solid particles in one scene (extension): the fluid
        // recipe, with the solids' elastic passes before the force pass,
        // which adds the fluid-solid pair terms and steps every particle
        phase("gather");
        sph_launch_gather(L, true, false, true);
        phase("density");
        sph_launch_density(L, false, true, false);
        phase("deformations (solid phase)");
        sph_launch_deformations_mixed(L, true);
        phase("stresses (solid phase)");
        sph_launch_stresses(L, false);
        phase("forces_solids (solid phase)");
        sph_launch_forces_solids_mixed(L);
        phase("forces_fluids+step");
        sph_launch_forces_fluids(L, true, true);
        if (L.num_rigid) {
            phase("rigid_bodies");
            sph_launch_rigid(L);
        }
        phase(nullptr);
        return;
    }
    phase("gather");
    sph_launch_gather(L, mat == MAT_FLUID, false, mat != MAT_FLUID);
    if (mat == MAT_FLUID || !L.no_symmetry_planes) {
        // a plane-free solid's density is summed by its first solid pass
        phase("density");
        sph_launch_density(L, false, mat == MAT_FLUID, mat != MAT_FLUID);
    }
    if (mat == MAT_FLUID) {
        phase("forces_fluids+step");
        sph_launch_forces_fluids(L, true, true);
        if (L.num_rigid) {
            phase("rigid_bodies");
            sph_launch_rigid(L);
        }
        phase(nullptr);
        return;
    }
    sph_launch_solid_passes(L, mat == MAT_COROT, mark, ctx);
    if (L.num_rigid) {
        phase("rigid_bodies");
        sph_launch_rigid(L);
    }
    phase(nullptr);
}

void sph_launch_rigid(const Launch &L) {
    if (!L.num_rigid || !L.rigid) return;
    const dim3 grid(SPH_RIGID_BLOCKS, L.num_rigid);
    k_rigid_reduce<<<grid, SPH_RIGID_THREADS, 0, L.stream>>>(L.scenes, L.rigid);
    k_rigid_integrate<<<L.num_rigid, 32, 0, L.stream>>>(L.scenes, L.rigid, L.num_rigid);
    k_rigid_scatter<<<grid, SPH_RIGID_THREADS, 0, L.stream>>>(L.scenes, L.rigid);
}

void sph_launch_rigid_reset(const Launch &L) {
    const unsigned g = L.num_scenes < 1024 ? L.num_scenes : 1024;
    k_rigid_reset<<<g ? g : 1, 64, 0, L.stream>>>(L.scenes, L.num_scenes);
}

// End of a batched substep: each scene with a finite quota left uses one.
__global__ void k_count_down(const SceneDesc *__restrict__ scenes, unsigned num_scenes) {
    for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < num_scenes; s += gridDim.x * blockDim.x) {
        unsigned *q = scenes[s].steps_left;
        if (!q) continue;
        const unsigned v = *q;
        if (v != 0u && v != SPH_STEPS_UNLIMITED) *q = v - 1u;
    }
}

__global__ void k_set_steps(unsigned *steps_left, unsigned steps) { *steps_left = steps; }

void sph_launch_count_down(const Launch &L) {
    unsigned g = (L.num_scenes + 255) / 256;
    k_count_down<<<g ? g : 1, 256, 0, L.stream>>>(L.scenes, L.num_scenes);
}

void sph_launch_set_steps(unsigned *steps_left, unsigned steps, cudaStream_t stream) {
    k_set_steps<<<1, 1, 0, stream>>>(steps_left, steps);
}

// Recording: the copy reads the counters, the tick (one thread, after the
// copy in stream order) advances them.
__global__ void k_record_copy(RecordPlan p) {
    const unsigned long long step = p.counters[0];
    if ((step + 1) % p.every) return;
    unsigned *dst = p.ring + (size_t)(p.counters[1] % p.frames) * p.frame_words;
    size_t base = 0;
    for (unsigned r = 0; r < p.num_ranges; ++r) {
        const uint2 rg = p.ranges[r];
        for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < rg.y; w += (size_t)gridDim.x * blockDim.x)
            dst[base + w] = p.blob[rg.x + w];
        base += rg.y;
    }
}

__global__ void k_record_tick(RecordPlan p) {
    const unsigned long long step = p.counters[0] + 1;
    p.counters[0] = step;
    if (step % p.every == 0) p.counters[1] += 1;
}

void sph_launch_record(const RecordPlan &p, cudaStream_t stream) {
    unsigned g = (p.frame_words + 255) / 256;
    if (g > 1024) g = 1024;
    k_record_copy<<<g ? g : 1, 256, 0, stream>>>(p);
    k_record_tick<<<1, 1, 0, stream>>>(p);
}

// Segment copy: block row y copies segment y, in 16-byte words where both
// ends allow, else 4-byte words, else bytes (a grid-stride loop each).
__global__ void k_copy_segments(const CopySeg *__restrict__ segs, unsigned first) {
    const CopySeg g = segs[first + blockIdx.y];
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uintptr_t align = (uintptr_t)g.src | (uintptr_t)g.dst;
    size_t done = 0;
    if ((((uintptr_t)g.src ^ (uintptr_t)g.dst) & 15u) == 0) {
        // source and destination at the same offset within 16 bytes: the
        // bytes up to the first 16-byte boundary, 16-byte words, the tail
        size_t head = (16u - ((uintptr_t)g.src & 15u)) & 15u;
        if (head > g.bytes) head = g.bytes;
        for (size_t c = t0; c < head; c += stride) g.dst[c] = g.src[c];
        const size_t n = (g.bytes - head) / 16;
        const uint4 *s = reinterpret_cast<const uint4 *>(g.src + head);
        uint4 *d = reinterpret_cast<uint4 *>(g.dst + head);
#pragma unroll 4
        for (size_t w = t0; w < n; w += stride) d[w] = s[w];
        done = head + n * 16;
    } else if (align % 4 == 0) {
        const size_t n = g.bytes / 4;
        const unsigned *s = reinterpret_cast<const unsigned *>(g.src);
        unsigned *d = reinterpret_cast<unsigned *>(g.dst);
        for (size_t w = t0; w < n; w += stride) d[w] = s[w];
        done = n * 4;
    }
    for (size_t c = done + t0; c < g.bytes; c += stride) g.dst[c] = g.src[c];
}

// One block copies a few small segments, in 4-byte words where both ends
// are 4-byte aligned, else bytes.
__global__ void k_copy_inline(InlineSegs segs) {
    for (unsigned q = 0; q < segs.count && q < SPH_INLINE_SEGS; ++q) {
        const CopySeg g = segs.seg[q];
        if ((((uintptr_t)g.src | (uintptr_t)g.dst | (uintptr_t)g.bytes) & 3u) == 0) {
            const unsigned *s = reinterpret_cast<const unsigned *>(g.src);
            unsigned *d = reinterpret_cast<unsigned *>(g.dst);
            for (size_t w = threadIdx.x; w < g.bytes / 4; w += blockDim.x) d[w] = s[w];
        } else {
            for (size_t c = threadIdx.x; c < g.bytes; c += blockDim.x) g.dst[c] = g.src[c];
        }
    }
}

void sph_launch_copy_inline(const InlineSegs &segs, cudaStream_t stream) {
    k_copy_inline<<<1, 256, 0, stream>>>(segs);
}

void sph_launch_copy_segments(const CopySeg *segs, unsigned count, unsigned long long max_bytes,
                              cudaStream_t stream) {
    // 64 KB per block (sixteen 16-byte words per thread, four in flight):
    // a segment's blocks share gridDim.x, so the large segments' count
    // sets it and the small segments' extra blocks exit at once
    const unsigned long long per_block = 256ull * 16 * 16;
    unsigned gx = (unsigned)((max_bytes + per_block - 1) / per_block);
    gx = gx < 1 ? 1 : gx > 256 ? 256 : gx;
    for (unsigned first = 0; first < count; first += 65535u) {
        const unsigned gy = count - first < 65535u ? count - first : 65535u;
        k_copy_segments<<<dim3(gx, gy), 256, 0, stream>>>(segs, first);
    }
}

// splitmix64 (Steele, Lea and Flood, 2014; the finaliser of Vigna's
// xorshift generators): a 64-bit counter-based mix.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    unsigned long long z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_lattice(SceneDesc S, LatticeGen g, unsigned count) {
    for (unsigned p = blockIdx.x * blockDim.x + threadIdx.x; p < count; p += gridDim.x * blockDim.x) {
        const unsigned q[3] = {p % g.nx, p / g.nx % g.ny, p / (g.nx * g.ny)};
        for (int a = 0; a < 3; ++a) {
            const unsigned long long z = splitmix64(g.seed * 0x100000000ull + 3ull * p + (unsigned long long)a);
            const double u = (double)(z >> 11) * 0x1.0p-53;
            const double off = __dmul_rn(g.jitter, __dsub_rn(__dmul_rn(2.0, u), 1.0));
            const double x = __dadd_rn(__dadd_rn(__dmul_rn((double)q[a], g.spacing), g.origin[a]), off);
            S.position[3 * (size_t)p + a] = __double2float_rn(x);
        }
        if (S.body_number)
            const_cast<unsigned *>(S.body_number)[p] = p < g.clamp_layers * g.nx * g.ny ? 1u : 0u;
        if (g.identity_rotation && S.rotation)
            for (int c = 0; c < 9; ++c) S.rotation[9 * (size_t)p + c] = (c % 4 == 0) ? 1.f : 0.f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *const_cast<unsigned *>(S.n) = count;
}

void sph_launch_lattice(const SceneDesc &d, const LatticeGen &g, cudaStream_t stream) {
    const unsigned count = g.nx * g.ny * g.nz;
    unsigned grid = (count + 255) / 256;
    grid = grid < 1 ? 1 : grid > 4096 ? 4096 : grid;
    k_lattice<<<grid, 256, 0, stream>>>(d, g, count);
}
