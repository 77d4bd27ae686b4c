// kernels_grid.cuh -- neighbour grid on sm_103a: cell hash, counting sort
// with warp-aggregated atomics, segmented exclusive scan, scatter and a
// deterministic per-cell order (ascending particle index), plus the gathers
// that build the cell-sorted float4 copies the pair kernels stream.
//
// Replaces find_particle_bins, zero_gridcount, count_particles_in_bins,
// prefix_sum, copy_celloffset_to_backup and insert_particles_in_bin_array
// (kernels/common.cl:372-529).  Output fields gridcell, gridcount,
// celloffset and cellparticles have the reference's meaning and layout; the
// order inside a cell is ascending particle index (the reference's is the
// atomic race order).
#pragma once

#include "kernels_common.cuh"

// The scatter and the per-cell ranking are chains of dependent loads (work
// entry -> scene -> gridcell -> celloffset -> the cell's entries), so each
// of their blocks takes SPH_WIDE consecutive work entries per pass and runs
// their chains side by side: the loads of all entries are issued before any
// result is used, and a launch needs a quarter of the blocks.
#define SPH_WIDE 4

struct WideItem {
    const SceneDesc *S;  // null: no entry, or the scene idles
    unsigned item;
    bool valid;          // item < the scene's active count
};

__device__ __forceinline__ void wide_items(const SceneDesc *__restrict__ scenes, const BlockMap &map, unsigned v0,
                                           WideItem (&w)[SPH_WIDE]) {
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j) {
        w[j].S = nullptr;
        w[j].item = 0u;
        w[j].valid = false;
        const unsigned v = v0 + j;
        if (v < map.num) {
            const BlockWork bw = map.work[v];
            const SceneDesc *S = scenes + bw.scene;
            if (!scene_idle(*S)) {
                w[j].S = S;
                w[j].item = bw.first + threadIdx.x;
                w[j].valid = w[j].item < active_count(*S);
            }
        }
    }
}

#define SPH_FOR_WIDE(map)                                                                       \
    for (unsigned v0_ = blockIdx.x * SPH_WIDE; v0_ < (map).num; v0_ += gridDim.x * SPH_WIDE) { \
        WideItem W[SPH_WIDE];                                                                   \
        wide_items(scenes, map, v0_, W);
#define SPH_END_WIDE }

// Blocks for a wide launch over `map`, at most `cap`.
__host__ __device__ inline unsigned wide_grid(unsigned num, unsigned cap) {
    const unsigned g = (num + SPH_WIDE - 1) / SPH_WIDE;
    const unsigned c = g < cap ? g : cap;
    return c ? c : 1u;
}

// find_particle_bins' cell coordinate (common.cl:372-391): clamp((uint)((p
// - b0)/(b1 - b0)*R), 0, R-1) with each float operation individually
// rounded and a saturating conversion; *outside is set for a particle
// outside gridbounds.
__device__ __forceinline__ unsigned cell_of(const SceneDesc &S, float3 p, bool *outside) {
    const float *gb = S.gridbounds;
    const float q[3] = {p.x, p.y, p.z};
    unsigned c[3];
    bool out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float lo = gb[2 * a], hi = gb[2 * a + 1];
        const float r = (float)S.gridres[a];
        const float v = __fmul_rn(__fdiv_rn(__fsub_rn(q[a], lo), __fsub_rn(hi, lo)), r);
        unsigned u = __float2uint_rz(v);  // saturating: negative and NaN -> 0
        if (u > S.gridres[a] - 1) u = S.gridres[a] - 1;
        out |= !(v >= 0.f && v < r);
        c[a] = u;
    }
    *outside = out;
    return c[2] * S.gridres[0] * S.gridres[1] + c[1] * S.gridres[0] + c[0];
}

// find_particle_bins (common.cl:372-391) fused with count_particles_in_bins
// (:401-408).  Lanes of a warp that hit the same cell combine into one
// atomicAdd; each particle keeps its arrival slot within the cell.  (One
// work entry per block: the wide form measured slower here.)
__global__ void k_bin_count(const SceneDesc *__restrict__ scenes, BlockMap map, int do_count) {
    SPH_FOR_WORK(map)
    const unsigned n = active_count(S);
    const bool valid = item < n;
    const unsigned lanes = __ballot_sync(SPH_FULL_MASK, valid);
    if (valid) {
        bool outside;
        const unsigned cell = cell_of(S, ld3(S.position, item), &outside);
        S.gridcell[item] = cell;
        if (outside) atomicOr(S.status, (unsigned)STATUS_OUTSIDE_GRID);
        if (do_count) {
            const unsigned peers = __match_any_sync(lanes, cell);
            const unsigned lane = threadIdx.x & 31u;
            const unsigned leader = __ffs(peers) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(S.gridcount + cell, (unsigned)__popc(peers));
            base = __shfl_sync(peers, base, leader);
            S.slot[item] = base + __popc(peers & ((1u << lane) - 1u));
            // the scan tile's total (k_scan_down reads these)
            const unsigned tile = cell / SPH_SCAN_TILE;
            const unsigned tpeers = __match_any_sync(lanes, tile);
            if (lane == (unsigned)(__ffs(tpeers) - 1)) atomicAdd(S.scan_sums + tile, (unsigned)__popc(tpeers));
        }
    }
    SPH_END_WORK
}

// zero_gridcount (common.cl:392-400) for every scene of the launch, one
// block per scan tile of SPH_SCAN_TILE cells: the counts, the tile's total
// (which k_bin_count accumulates) and, once per scene, the crowded-cell
// queue counter.
__global__ void __launch_bounds__(SPH_SCAN_THREADS) k_zero_cells(const SceneDesc *__restrict__ scenes, BlockMap map) {
    for (unsigned vb = blockIdx.x; vb < map.num; vb += gridDim.x) {
        const BlockWork bw = map.work[vb];
        const SceneDesc &S = scenes[bw.scene];
        if (scene_idle(S)) continue;
        const unsigned end = min(bw.first + SPH_SCAN_TILE, S.num_cells);
        for (unsigned c = bw.first + threadIdx.x; c < end; c += blockDim.x) S.gridcount[c] = 0u;
        if (threadIdx.x == 0) {
            S.scan_sums[bw.first / SPH_SCAN_TILE] = 0u;
            if (bw.first == 0) S.big_cells[0] = 0u;
        }
    }
}

// count_particles_in_bins alone, for a driver that calls the reference's
// kernels one by one (gridcell already computed).
__global__ void k_count_only(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    const unsigned n = active_count(S);
    const bool valid = item < n;
    const unsigned lanes = __ballot_sync(SPH_FULL_MASK, valid);
    if (valid) {
        unsigned cell = S.gridcell[item];
        if (cell >= S.num_cells) cell = S.num_cells - 1;  // host-written garbage
        const unsigned peers = __match_any_sync(lanes, cell);
        const unsigned lane = threadIdx.x & 31u;
        const unsigned leader = __ffs(peers) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(S.gridcount + cell, (unsigned)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        S.slot[item] = base + __popc(peers & ((1u << lane) - 1u));
    }
    SPH_END_WORK
}

// ---- segmented exclusive scan of gridcount -> celloffset (prefix_sum,
// common.cl:409-515, restated as a correct two-phase scan) -------------------

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned *total) {
    __shared__ unsigned warp_sums[32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(SPH_FULL_MASK, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    const unsigned nw = blockDim.x >> 5;
    if (warp == 0) {
        unsigned w = lane < nw ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(SPH_FULL_MASK, w, o);
            if (lane >= (unsigned)o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    unsigned before = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[nw - 1];
    __syncthreads();
    return before + x - v;
}

// Phase 1: each tile's total, from coalesced loads.
__global__ void __launch_bounds__(SPH_SCAN_THREADS) k_scan_reduce(const SceneDesc *__restrict__ scenes,
                                                                  BlockMap map) {
    for (unsigned vb = blockIdx.x; vb < map.num; vb += gridDim.x) {
        const BlockWork bw = map.work[vb];
        const SceneDesc &S = scenes[bw.scene];
        if (scene_idle(S)) continue;
        const unsigned end = min(bw.first + SPH_SCAN_TILE, S.num_cells);
        unsigned sum = 0;
        for (unsigned c = bw.first + threadIdx.x; c < end; c += blockDim.x) sum += S.gridcount[c];
        unsigned total;
        block_exclusive_scan(sum, &total);
        if (threadIdx.x == 0) S.scan_sums[bw.first / SPH_SCAN_TILE] = total;
    }
}

// Phase 2: each tile adds up the totals of its scene's earlier tiles, then
// scans its cells through shared memory (coalesced loads and stores).
__global__ void __launch_bounds__(SPH_SCAN_THREADS) k_scan_down(const SceneDesc *__restrict__ scenes, BlockMap map) {
    __shared__ unsigned tile[SPH_SCAN_TILE];
    constexpr unsigned per = SPH_SCAN_TILE / SPH_SCAN_THREADS;
    for (unsigned vb = blockIdx.x; vb < map.num; vb += gridDim.x) {
        const BlockWork bw = map.work[vb];
        const SceneDesc &S = scenes[bw.scene];
        if (scene_idle(S)) continue;
        const unsigned t = bw.first / SPH_SCAN_TILE;
        unsigned part = 0;
        for (unsigned j = threadIdx.x; j < t; j += blockDim.x) part += S.scan_sums[j];
        unsigned base;
        block_exclusive_scan(part, &base);
        const unsigned end = min(bw.first + SPH_SCAN_TILE, S.num_cells);
        for (unsigned k = threadIdx.x; k < SPH_SCAN_TILE; k += blockDim.x) {
            const unsigned c = bw.first + k;
            tile[k] = c < end ? S.gridcount[c] : 0u;
        }
        __syncthreads();
        unsigned v[per], sum = 0;
#pragma unroll
        for (unsigned j = 0; j < per; ++j) {
            v[j] = tile[threadIdx.x * per + j];
            sum += v[j];
        }
        unsigned total;
        unsigned run = base + block_exclusive_scan(sum, &total);
#pragma unroll
        for (unsigned j = 0; j < per; ++j) {
            tile[threadIdx.x * per + j] = run;
            run += v[j];
        }
        __syncthreads();
        for (unsigned k = threadIdx.x; bw.first + k < end; k += blockDim.x) S.celloffset[bw.first + k] = tile[k];
        __syncthreads();  // the next tile reuses `tile`
    }
}

// insert_particles_in_bin_array (common.cl:523-529) without atomics: each
// particle goes to celloffset[cell] + its arrival slot, in arrival order,
// of an unsorted copy of cellparticles: the first pnum words of the sorted
// position buffer, which is free until the gather.
__device__ __forceinline__ unsigned *unsorted_cells(const SceneDesc &S) { return reinterpret_cast<unsigned *>(S.spos); }

__global__ void k_scatter(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WIDE(map)
    unsigned cell[SPH_WIDE], slot[SPH_WIDE];
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j)
        if (W[j].valid) {
            cell[j] = W[j].S->gridcell[W[j].item];
            slot[j] = W[j].S->slot[W[j].item];
        }
    unsigned off[SPH_WIDE];
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j) {
        off[j] = 0xffffffffu;
        if (W[j].valid && cell[j] < W[j].S->num_cells) off[j] = W[j].S->celloffset[cell[j]];
    }
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j)
        if (off[j] != 0xffffffffu) {
            const SceneDesc &S = *W[j].S;
            const unsigned dst = off[j] + slot[j];
            if (dst < S.pnum) unsorted_cells(S)[dst] = W[j].item;
        }
    SPH_END_WIDE
}

// Canonical order inside each cell: ascending particle index.  One thread
// per slot of the unsorted copy: its particle's place in the cell is the
// number of the cell's particles with a smaller index.  Cells of more than
// SPH_SMALL_CELL particles are copied as they are and queued (by the thread
// of their first slot) for k_sort_big_cells.
__global__ void k_rank_cells(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WIDE(map)
    unsigned x[SPH_WIDE], cell[SPH_WIDE];
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j) x[j] = W[j].valid ? unsorted_cells(*W[j].S)[W[j].item] : 0xffffffffu;
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j)
        cell[j] = W[j].valid && x[j] < W[j].S->pnum ? W[j].S->gridcell[x[j]] : 0xffffffffu;
    unsigned off[SPH_WIDE], cnt[SPH_WIDE];
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j) {
        off[j] = 0u;
        cnt[j] = 0u;
        if (W[j].valid && cell[j] < W[j].S->num_cells) {
            off[j] = W[j].S->celloffset[cell[j]];
            cnt[j] = W[j].S->gridcount[cell[j]];
        }
    }
#pragma unroll
    for (int j = 0; j < SPH_WIDE; ++j) {
        const unsigned item = W[j].item;
        // inconsistent tables come only from host-written garbage: skip
        if (cnt[j] && off[j] <= item && item - off[j] < cnt[j] && cnt[j] <= W[j].S->pnum - off[j]) {
            const SceneDesc &S = *W[j].S;
            if (cnt[j] > SPH_SMALL_CELL) {
                S.cellparticles[item] = x[j];
                if (item == off[j]) {
                    const unsigned k = atomicAdd(S.big_cells, 1u);
                    S.big_cells[1 + k] = cell[j];
                }
            } else {
                const unsigned *U = unsorted_cells(S) + off[j];
                unsigned r = 0;
                for (unsigned a2 = 0; a2 < cnt[j]; ++a2) r += U[a2] < x[j];
                S.cellparticles[off[j] + r] = x[j];
            }
        }
    }
    SPH_END_WIDE
}

// Fallback for crowded cells (e.g. particles clamped into an edge cell):
// one block bitonic-sorts each queued cell, padded to a power of two, in a
// scratch region of the sorted-position buffer ([2*off, 2*off + L) of its
// words, which cannot overlap another cell's region since L < 2*count).
// grid (blocks per scene, scenes): blockIdx.y is the scene, so a batch of
// many scenes without crowded cells costs one load per block.
__global__ void __launch_bounds__(1024) k_sort_big_cells(const SceneDesc *__restrict__ scenes, unsigned num_scenes) {
    for (unsigned s = blockIdx.y; s < num_scenes; s += gridDim.y) {
        const SceneDesc &S = scenes[s];
        if (scene_idle(S)) continue;
        const unsigned nbig = S.big_cells[0];
        for (unsigned b = blockIdx.x; b < nbig; b += gridDim.x) {
            const unsigned cell = S.big_cells[1 + b];
            const unsigned off = S.celloffset[cell], cnt = S.gridcount[cell];
            if (off > S.pnum || cnt > S.pnum - off) continue;
            unsigned L = 1;
            while (L < cnt) L <<= 1;
            unsigned *buf = reinterpret_cast<unsigned *>(S.spos) + 2u * off;
            unsigned *seg = S.cellparticles + off;
            for (unsigned t = threadIdx.x; t < L; t += blockDim.x) buf[t] = t < cnt ? seg[t] : 0xffffffffu;
            __syncthreads();
            for (unsigned k = 2; k <= L; k <<= 1) {
                for (unsigned j = k >> 1; j > 0; j >>= 1) {
                    for (unsigned t = threadIdx.x; t < L; t += blockDim.x) {
                        unsigned u = t ^ j;
                        if (u > t) {
                            unsigned a = buf[t], c = buf[u];
                            bool up = (t & k) == 0;
                            if ((a > c) == up) {
                                buf[t] = c;
                                buf[u] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            for (unsigned t = threadIdx.x; t < cnt; t += blockDim.x) seg[t] = buf[t];
            __syncthreads();
        }
    }
}

// Cell-sorted copies: spos[k] = position[cellparticles[k]] (and velocity,
// density when asked; for solids also the rest position with the body
// number -- and in a mixed scene SPH_SOLID_PHASE_BIT for a solid-phase
// particle -- and 1/density0 in the velocity copy's w).  Gathers once so
// the pair loops stream float4s.
__global__ void k_gather(const SceneDesc *__restrict__ scenes, BlockMap map, int with_vel, int with_dens,
                         int with_solid) {
    SPH_FOR_WORK(map)
    if (item < active_count(S)) {
        unsigned i = S.cellparticles[item];
        if (i >= S.pnum) i = 0;  // host-written garbage
        float3 p = ld3(S.position, i);
        S.spos[item] = make_float4(p.x, p.y, p.z, 0.f);
        const bool solid = with_solid && S.spos0;
        if (with_vel || solid) {
            float3 v = ld3(S.velocity, i);
            S.svel[item] = make_float4(v.x, v.y, v.z, solid ? __frcp_rn(S.density0[i]) : 0.f);
        }
        if (with_dens) S.sdens[item] = S.density[i];
        if (solid) {
            // rest position, and the body number's bits in w
            const float3 p0 = ld3(S.originalpos, i);
            unsigned w = S.body_number[i];
            if (S.phase && S.phase[i]) w |= SPH_SOLID_PHASE_BIT;
            S.spos0[item] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(w));
        }
    }
    SPH_END_WORK
}
