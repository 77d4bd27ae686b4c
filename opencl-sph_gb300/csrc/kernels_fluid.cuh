// kernels_fluid.cuh -- per-particle pair passes for density and WCSPH
// forces, the symplectic-Euler integrator and plane constraints (sm_103a).
//
// Pair passes run one thread per cell-sorted particle k (i =
// cellparticles[k]) so a warp covers a few neighbouring cells and shares
// their neighbour rows in L1; neighbours are streamed from the float4
// copies built by k_gather.  Sums are FP32, blocked per stencil row: a
// row's terms added in order, the nine row sums with Kahan compensation.
#pragma once

#include "kernels_common.cuh"
#include "kernels_rigid.cuh"


// compute_density (common.cl:610-690) and compute_original_density
// (solids.cl:99-170): rho_i = m * sum_j W_poly6(|x_j - x_i|), j = i
// included, plus mirror images across the symmetry planes.  With
// `original` the result goes to density0 and no neighbour count is kept.
//
// The stencil is walked as 9 rows (dz outer, dy inner, as the reference's
// z, y, x loops): cells x-1..x+1 of one (z, y) row are one contiguous range
// of the cell-sorted order.  Each warp stages its rows in shared memory:
// for every row the union of its lanes' ranges is copied once with
// coalesced float4 loads and each lane walks its own range there (lanes of
// one cell read the same address: a broadcast).  Values, order and
// arithmetic are those of a direct walk; a union wider than the buffer (a
// warp that spans two grid rows) is read from global memory instead.
// The sum is blocked: each stencil row's terms are added in candidate
// order, and the nine row sums with Kahan compensation (one compensated
// add per row instead of per neighbour).
//
// With `want_mask` (fused fluid substeps, where positions cannot change
// before the force pass) each fluid particle also records, per row, which
// candidates lie within h: bit t of row r's 64-bit mask is candidate
// b_r + t.  The low word goes to nbmask[(2r) * pnum + k], the high word to
// nbmask[(2r+1) * pnum + k] only when the row holds more than 32
// candidates; a row of more than 64 marks the particle for a scan
// (ncand[k] = SPH_NCAND_SCAN).  The stores of one row are one coalesced
// store per warp.
// 128 float4s per warp hold a warp's row union (about 48 candidates in a
// lattice); 256 measured the same and took twice the shared memory.
#define SPH_STAGE 128

__host__ __device__ constexpr size_t density_smem_bytes(unsigned block) {
    return sizeof(float4) * SPH_STAGE * (block / 32);
}

// p = (rho - rho0) stiffness (fluids.cl:33-36), rounded as written.
__device__ __forceinline__ float fluid_pressure(float rho, float rho0, float stiff) {
    return __fmul_rn(__fsub_rn(rho, rho0), stiff);
}

// COUNT: a masked pass that also counts num_neighbours (a named
// compute_density, whose caller may read the count before the force pass).
template <bool PLANES, bool MASK, bool COUNT = false>
__device__ __forceinline__ void density_one(const SceneDesc &S, unsigned n, unsigned item, unsigned lane,
                                            float4 *__restrict__ wstage, int original) {
    const bool active = item < n;
    const unsigned k = item;
    const unsigned i = active ? min(S.cellparticles[k], S.pnum - 1) : 0u;
    const float h = *S.h;
    const DistBounds B = dist_bounds(h);
    const float h2 = __fmul_rn(h, h);
    const float3 ipos = active ? xyz(S.spos[k]) : make_float3(0.f, 0.f, 0.f);
    const NegPoint nip = neg_point(ipos);
    Planes P;
    if (PLANES) {
        load_planes(S, ipos, h, P);
        if (!active) P.imask = 0;
    }
    Kahan rho;
    unsigned count = 0, total = 0;
    bool overflow = false;
    const StencilRows rows(S, active ? S.gridcell[i] : 0u);
    const float4 *__restrict__ spos = S.spos;
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        unsigned b = 0, e = 0;
        if (active) rows.row(S, r, &b, &e);
        const unsigned ub = __reduce_min_sync(SPH_FULL_MASK, b < e ? b : 0xffffffffu);
        const unsigned ue = __reduce_max_sync(SPH_FULL_MASK, b < e ? e : 0u);
        const bool staged = ub < ue && ue - ub <= SPH_STAGE;
        if (staged) {
            __syncwarp();
            for (unsigned t = lane; t < ue - ub; t += 32) wstage[t] = spos[ub + t];
            __syncwarp();
        }
        const unsigned len = e - b;
        // the row's mask in two words, each filled by its own loop below
        // (a 32-bit shift per neighbour, no test of the candidate's place)
        unsigned lo = 0, hi = 0;
        // the row's density terms in candidate order; the row sums are
        // added with Kahan compensation (blocked summation)
        float rowsum = 0.f;
        auto visit = [&](float4 j4, unsigned *word, unsigned bit) {
            const float r2 = dist2(j4, nip);
            if (r2 <= B.le) {
                const float d = fmaxf(h2 - r2, 0.f);
                rowsum = __fadd_rn(rowsum, d * d * d);
                // a fused plane-free substep counts in the force pass
                if (!MASK || PLANES || COUNT) count += r2 <= B.lt;
                if (MASK && word) *word |= 1u << bit;
            }
            if (PLANES && P.imask) {
                const float3 jpos = xyz(j4);
                const unsigned jm = plane_jmask(P, jpos, h);
                // subsets of jm in increasing order: the reference's
                // plane_bits order restricted to the subsets it keeps
                for (unsigned sb = (0u - jm) & jm; sb; sb = (sb - jm) & jm) {
                    float3 ref = jpos;
                    for (unsigned s2 = 0; s2 < P.count; ++s2)
                        if (sb & (1u << s2)) ref = reflect3(ref, P.p[s2], P.n[s2]);
                    const float m2 = norm2(sub3(ref, ipos));
                    if (m2 <= B.lt) {
                        const float d = fmaxf(h2 - m2, 0.f);
                        rowsum = __fadd_rn(rowsum, d * d * d);
                        ++count;
                    }
                }
            }
        };
        // candidates [0, 32) set bits of `lo`, [32, 64) of `hi`; a row
        // longer than 64 (the later passes scan it) records none past 64
        const unsigned n1 = len < 32u ? len : 32u, n2 = len < 64u ? len : 64u;
        if (staged) {
            const float4 *src = wstage + (b - ub);
#pragma unroll 4
            for (unsigned t = 0; t < n1; ++t) visit(src[t], &lo, t);
#pragma unroll 4
            for (unsigned t = n1; t < n2; ++t) visit(src[t], &hi, t - 32u);
            for (unsigned t = n2; t < len; ++t) visit(src[t], nullptr, 0u);
        } else {
            for (unsigned t = 0; t < n1; ++t) visit(spos[b + t], &lo, t);
            for (unsigned t = n1; t < n2; ++t) visit(spos[b + t], &hi, t - 32u);
            for (unsigned t = n2; t < len; ++t) visit(spos[b + t], nullptr, 0u);
        }
        rho.add(rowsum);
        if (MASK && active) {
            const unsigned long long bits = ((unsigned long long)hi << 32) | lo;
            store_row_mask(S, k, r, len, bits);
            overflow |= len > 64;
            total += len;
        }
    }
    if (active) {
        const float value = poly6_density(rho.s, h2, h, *S.mass);
        if (original) {
            S.density0[i] = value;
        } else {
            S.density[i] = value;
            if (!MASK || PLANES || COUNT) S.num_neighbours[i] = count;
            S.sdens[k] = value;
        }
        if (MASK) {
            S.ncand[k] = overflow ? SPH_NCAND_SCAN : total;
            // the force pass reads a neighbour's pressure with its position
            // and its reciprocal density with its velocity (spare w lanes);
            // a mixed scene's solid particle stores its pressure clamped at
            // 0 and its reciprocal density negated, which marks it solid
            float pv = fluid_pressure(value, *S.restdens, *S.stiffness);
            float rv = rcp_approx(value);
            if (S.phase && S.phase[i]) {
                pv = fmaxf(pv, 0.f);
                rv = -rv;
            }
            S.spos[k].w = pv;
            S.svel[k].w = rv;
        }
    }
}

// Two instantiations, each skipping the other's scenes: the plane variant
// (launched only when some scene has symmetry planes) keeps the common
// plane-free loop free of its registers.  COUNT: the masked pass counts
// num_neighbours too (a named compute_density recording masks); a kernel
// of its own, so the fused substep's keeps its register allocation.
template <bool PLANES, bool COUNT = false>
__global__ void __launch_bounds__(512, 2)
    k_density(const SceneDesc *__restrict__ scenes, BlockMap map, int original, int want_mask, int skip_solids) {
    extern __shared__ float4 sm_stage[];
    float4 *wstage = sm_stage + (threadIdx.x >> 5) * SPH_STAGE;
    const unsigned lane = threadIdx.x & 31u;
    SPH_FOR_WORK(map)
    if ((S.num_symmetry_planes != 0) != PLANES) continue;
    // in a fused substep a plane-free solid's first solid pass sums its density
    if (skip_solids && !PLANES && (S.programs & (PROG_COROT | PROG_SVK))) continue;
    const unsigned n = active_count(S);
    if (want_mask && S.nbmask && (S.programs & PROG_FLUIDS) && !original)
        density_one<PLANES, true, COUNT>(S, n, item, lane, wstage, original);
    else
        density_one<PLANES, false>(S, n, item, lane, wstage, original);
    SPH_END_WORK
}

// APPLY_CUBE_BOUNDS(ipos, f, -2.0, 2.0) (common.cl:37-43): a repulsive
// band 0.2 wide inside [-2, 2]^3; the bounds are double literals, so the
// tests and the update are evaluated in double as in the source.  The tests
// (double)p < -2 + (double)0.2f and (double)p > 2 - (double)0.2f run in FP32
// without changing a result: p converts to double exactly, and the bounds
// (-+1.7999999970197678) lie strictly between two floats, so they hold iff
// p <= -0x1.cccccep+0 or p >= 0x1.cccccep+0, the floats just outside them.
// Only a particle inside the band takes the double update; FP64 warp
// instructions are slow on this part, and the test runs for every particle.
#define SPH_CUBE_BAND_LO (-0x1.cccccep+0f)
#define SPH_CUBE_BAND_HI (0x1.cccccep+0f)
__device__ __forceinline__ float cube_bound(float p, float f) {
    const double mn = -2.0, mx = 2.0;
    if (p <= SPH_CUBE_BAND_LO) return (float)((double)f + (1.0 / (-(mn) + (double)p) - 5.0));
    if (p >= SPH_CUBE_BAND_HI) return (float)((double)f - (1.0 / (mx - (double)p) - 5.0));
    return f;
}

// compute_forces_fluids (kernels/fluids.cl:1-63): pressure
// p = (rho - rho0) * stiffness, spiky-gradient pressure and Laplacian
// viscosity pair terms divided by rho_i rho_j, times the mass, plus the
// cube band.  A pair at exactly zero distance contributes nothing (the
// reference produces NaN there).  `fuse_step` also integrates particle i (step_forward) from
// the sorted copies, which no other thread reads afterwards.
__device__ __forceinline__ void integrate(const SceneDesc &S, unsigned i, float3 f, float3 v, float3 p);

// Particle i's side of the fluid pair term.
struct FluidI {
    float3 ipos, ivel;
    float2 nxy, nvxy;  // -ipos and -ivel's x, y lanes (the packed differences)
    float inv_rhoi, pi, h, rho0, stiff, visc, kv;
    float vk, pk;  // visc kv and -kv / 2, the pair term's constant factors
    DistBounds B;
};

__device__ __forceinline__ FluidI fluid_i(const SceneDesc &S, float3 ipos, float3 ivel, float rhoi) {
    FluidI I;
    I.ipos = ipos;
    I.ivel = ivel;
    I.nxy = make_float2(-ipos.x, -ipos.y);
    I.nvxy = make_float2(-ivel.x, -ivel.y);
    I.inv_rhoi = rcp_approx(rhoi);
    I.h = *S.h;
    I.B = dist_bounds(I.h);
    I.rho0 = *S.restdens;
    I.stiff = *S.stiffness;
    I.visc = *S.viscosity;
    const float h3 = I.h * I.h * I.h;
    I.kv = 45.0f / (SPH_PI_F * h3 * h3);  // 45 / (pi h^6)
    I.pi = fluid_pressure(rhoi, I.rho0, I.stiff);
    I.vk = __fmul_rn(I.visc, I.kv);
    I.pk = __fmul_rn(-0.5f, I.kv);
    return I;
}

// One neighbour's pressure + viscosity term (fluids.cl:37-56), added to f,
// from the neighbour's pressure pj and reciprocal density inv_rhoj.  Every
// rounding is pinned, so the scan and the mask walk produce the same sum.
// Distinct particles at exactly zero distance (and i itself) contribute
// nothing.  Returns r^2 (the neighbour count's test).  IN_RANGE: the caller
// walks the density pass's masks, whose candidates passed r^2 <= le with
// the same positions and arithmetic, so that test is not repeated.
template <bool IN_RANGE = false>
__device__ __forceinline__ float fluid_pair_p(const FluidI &I, float pi, float3 jpos, float3 jvel, float pj,
                                              float inv_rhoj, BlockSum3 &f) {
    // d = x_j - x_i and r^2 as sub3 and norm2 compute them, the x and y
    // lanes in packed FP32x2 instructions (each lane rounded alike)
    const float2 dxy = __fadd2_rn(make_float2(jpos.x, jpos.y), I.nxy);
    const float dz = __fsub_rn(jpos.z, I.ipos.z);
    const float2 sq = __fmul2_rn(dxy, dxy);
    const float r2 = __fadd_rn(__fadd_rn(sq.x, sq.y), __fmul_rn(dz, dz));
    if ((!IN_RANGE && !(r2 <= I.B.le)) || r2 == 0.f) return r2;
    const float rinv = rsqrtf(r2);
    const float dist = __fmul_rn(r2, rinv);
    const float din = __fsub_rn(I.h, dist);
    const float inv_didj = __fmul_rn(I.inv_rhoi, inv_rhoj);
    const float vterm = __fmul_rn(din, I.vk);
    const float pterm = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fadd_rn(pi, pj), I.pk), rinv), din), din);
    // (d pterm + (v_j - v_i) vterm) / (rho_i rho_j), per lane as
    // __fmul_rn(__fmaf_rn(d, pterm, __fmul_rn(rv, vterm)), inv_didj)
    const float2 rvxy = __fadd2_rn(make_float2(jvel.x, jvel.y), I.nvxy);
    const float rvz = __fsub_rn(jvel.z, I.ivel.z);
    const float2 fxy = __fmul2_rn(__ffma2_rn(dxy, make_float2(pterm, pterm), __fmul2_rn(rvxy, make_float2(vterm, vterm))),
                                  make_float2(inv_didj, inv_didj));
    f.add2(fxy, __fmul_rn(__fmaf_rn(dz, pterm, __fmul_rn(rvz, vterm)), inv_didj));
    return r2;
}

template <bool IN_RANGE = false>
__device__ __forceinline__ float fluid_pair(const FluidI &I, float3 jpos, float3 jvel, float pj, float inv_rhoj,
                                            BlockSum3 &f) {
    return fluid_pair_p<IN_RANGE>(I, I.pi, jpos, jvel, pj, inv_rhoj, f);
}

// The end of a fluid particle's force pass: mass, cube band, store, step.
// `extra`: force already on the particle (a mixed scene's solid particle
// carries its elastic force, which the fluid pair terms add to).
__device__ __forceinline__ void fluid_finish(const SceneDesc &S, unsigned i, const FluidI &I, const BlockSum3 &f,
                                             int fuse_step, float3 extra = make_float3(0.f, 0.f, 0.f)) {
    const float m = *S.mass;
    float3 fi = f.get() * m;
    fi = make_float3(fi.x + extra.x, fi.y + extra.y, fi.z + extra.z);
    fi.x = cube_bound(I.ipos.x, fi.x);
    fi.y = cube_bound(I.ipos.y, fi.y);
    fi.z = cube_bound(I.ipos.z, fi.z);
    st3(S.force, i, fi);
    if (fuse_step) integrate(S, i, fi, I.ivel, I.ipos);
}

// Mixed fluid-solid scenes (extension; `phase` field): a solid particle's
// fluid pair terms cover its fluid neighbours only (its solid neighbours
// act through the elastic force), a fluid particle's cover every neighbour;
// a pair with a solid particle takes both pressures clamped at 0 (it
// pushes, never pulls).
template <bool MIXED>
__device__ __forceinline__ bool mixed_solid(const SceneDesc &S, unsigned i) {
    return MIXED && S.phase && S.phase[i] != 0u;
}
template <bool MIXED>
__device__ __forceinline__ float3 mixed_extra(const SceneDesc &S, unsigned i, bool solid_i) {
    return (MIXED && solid_i) ? ld3(S.force, i) : make_float3(0.f, 0.f, 0.f);
}
// One neighbour of the masked force walk, from its position (pressure in
// w) and velocity (reciprocal density in w, negated for a mixed scene's
// solid particle); adds to the neighbour count.
template <bool MIXED>
__device__ __forceinline__ void walk_pair(const FluidI &I, bool solid_i, float4 p, float4 v, BlockSum3 &f,
                                          unsigned &count) {
    if (MIXED) {
        const bool solid_j = v.w < 0.f;
        if (solid_i && solid_j) {
            count += norm2(sub3(xyz(p), I.ipos)) <= I.B.lt;
            return;
        }
        if (solid_i || solid_j) {
            count += fluid_pair_p<true>(I, fmaxf(I.pi, 0.f), xyz(p), xyz(v), fmaxf(p.w, 0.f), fabsf(v.w), f) <=
                     I.B.lt;
            return;
        }
    }
    count += fluid_pair<true>(I, xyz(p), xyz(v), p.w, v.w, f) <= I.B.lt;
}

// The stencil scan: every candidate of the 27 cells, in the reference's
// order; returns the count of candidates closer than h (j = i included).
template <bool MIXED>
__device__ __forceinline__ unsigned fluid_scan(const SceneDesc &S, unsigned cell, const FluidI &I, BlockSum3 &f,
                                               bool solid_i) {
    const float4 *__restrict__ spos = S.spos;
    const float4 *__restrict__ svel = S.svel;
    const float *__restrict__ sdens = S.sdens;
    unsigned count = 0;
    for_each_neighbour(S, cell, [&](unsigned kk) {
        const bool solid_j = MIXED && S.phase[min(S.cellparticles[kk], S.pnum - 1)] != 0u;
        if (solid_i && solid_j) {
            count += norm2(sub3(xyz(spos[kk]), I.ipos)) <= I.B.lt;
            return;
        }
        const float rho = sdens[kk];
        float pi = I.pi, pj = fluid_pressure(rho, I.rho0, I.stiff);
        if (MIXED && (solid_i || solid_j)) {
            pi = fmaxf(pi, 0.f);
            pj = fmaxf(pj, 0.f);
        }
        count += fluid_pair_p(I, pi, xyz(spos[kk]), xyz(svel[kk]), pj, rcp_approx(rho), f) <= I.B.lt;
    }, [&] { f.end_row(); });
    return count;
}

template <bool MIXED>
__global__ void k_forces_fluids(const SceneDesc *__restrict__ scenes, BlockMap map, int fuse_step) {
    SPH_FOR_WORK(map)
    if (MIXED && !S.phase) continue;  // the plain instantiation covers those
    if (!MIXED && S.phase) continue;
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const FluidI I = fluid_i(S, xyz(S.spos[k]), xyz(S.svel[k]), S.sdens[k]);
        const bool solid_i = mixed_solid<MIXED>(S, i);
        BlockSum3 f;
        fluid_scan<MIXED>(S, S.gridcell[i], I, f, solid_i);
        fluid_finish(S, i, I, f, fuse_step, mixed_extra<MIXED>(S, i, solid_i));
    }
    SPH_END_WORK
}

// The fused-substep force pass: walks the candidate masks the density pass
// recorded, row by row and two neighbours at a time, reading each
// neighbour's position with its pressure in w and its velocity with its
// reciprocal density in w (two float4 loads).  Lanes whose masks overflowed
// scan the stencil.  It also counts num_neighbours (the candidates closer
// than h, j = i included), which the fused density pass of a plane-free
// scene leaves to it.
// At most 64 registers: with the current walk 64 beats 56 (0.1886 ->
// 0.1859 ms at 1M particles), where the earlier walk ran best at 56.
template <bool MIXED>
__global__ void __maxnreg__(64) k_forces_fluids_masked(const SceneDesc *__restrict__ scenes, BlockMap map, int fuse_step) {
    SPH_FOR_WORK(map)
    if (MIXED && !S.phase) continue;  // the plain instantiation covers those
    if (!MIXED && S.phase) continue;
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const FluidI I = fluid_i(S, xyz(S.spos[k]), xyz(S.svel[k]), S.sdens[k]);
        const unsigned cell = S.gridcell[i];
        const bool solid_i = mixed_solid<MIXED>(S, i);
        BlockSum3 f;
        unsigned count = 0;  // num_neighbours, which the density pass left to this one
        if (S.ncand[k] != SPH_NCAND_SCAN) {
            count = 1;  // k itself (r^2 = 0), whose mask bit the walk clears
            const float4 *__restrict__ spos = S.spos;
            const float4 *__restrict__ svel = S.svel;
            // two neighbours per iteration: both loads are in flight
            // before the first pair's arithmetic (same order)
            const StencilRows rows(S, cell);
            // the next row's bounds and low mask word are loaded while this
            // row is walked
            unsigned nb, ne;
            rows.row(S, 0, &nb, &ne);
            unsigned nlo = S.nbmask[k];
#pragma unroll 1
            for (int r = 0; r < 9; ++r) {
                unsigned b = nb;
                const unsigned len = ne - nb;
                unsigned lo = nlo & (len >= 32u ? 0xffffffffu : (1u << len) - 1u);
                if (r < 8) {
                    rows.row(S, r + 1, &nb, &ne);
                    nlo = S.nbmask[(size_t)(2 * (r + 1)) * S.pnum + k];
                }
                unsigned hi = 0;
                if (len > 32u) {
                    hi = S.nbmask[(size_t)(2 * r + 1) * S.pnum + k];
                    hi &= len >= 64u ? 0xffffffffu : (1u << (len - 32u)) - 1u;
                }
                unsigned long long mask = ((unsigned long long)hi << 32) | lo;
                // k itself (row 4, its own cell's) adds no force and is
                // counted above
                if (r == 4 && k - b < 64u) mask &= ~(1ull << (k - b));
                // the row's two mask words in turn, with 32-bit bit scans
#pragma unroll 1
                for (unsigned w = 0, m = (unsigned)mask; w < 2; ++w, m = (unsigned)(mask >> 32), b += 32) {
                    while (m) {
                        const unsigned t1 = (unsigned)(__ffs(m) - 1);
                        m &= m - 1u;
                        const float4 p1 = spos[b + t1], v1 = svel[b + t1];
                        if (m) {
                            const unsigned t2 = (unsigned)(__ffs(m) - 1);
                            m &= m - 1u;
                            const float4 p2 = spos[b + t2], v2 = svel[b + t2];
                            walk_pair<MIXED>(I, solid_i, p1, v1, f, count);
                            walk_pair<MIXED>(I, solid_i, p2, v2, f, count);
                        } else {
                            walk_pair<MIXED>(I, solid_i, p1, v1, f, count);
                        }
                    }
                }
                f.end_row();
            }
        } else {
            count = fluid_scan<MIXED>(S, cell, I, f, solid_i);
        }
        if (!S.num_symmetry_planes) S.num_neighbours[i] = count;
        fluid_finish(S, i, I, f, fuse_step, mixed_extra<MIXED>(S, i, solid_i));
    }
    SPH_END_WORK
}

// step_forward (common.cl:691-722): a = f/m + g, v += dt a, x += dt v;
// particles of a fixed (non-dynamic) body are skipped, and so are those of
// a rigid body (extension), which its own step moves.  An optional
// `wallbounds` field (extension) mirrors particles that leave the box back
// inside and reverses their normal velocity.
__device__ __forceinline__ void integrate(const SceneDesc &S, unsigned i, float3 f, float3 v, float3 p) {
    // fixed bodies stay put; rigid bodies are moved by k_rigid_scatter
    if (body_skips_step(S, i)) return;
    const float m = *S.mass, dt = *S.timestep;
    const float3 g = make_float3(S.gravity[0], S.gravity[1], S.gravity[2]);
    const float3 a = make_float3(f.x / m + g.x, f.y / m + g.y, f.z / m + g.z);
    st3(S.acceleration, i, a);
    float3 vn = make_float3(v.x + dt * a.x, v.y + dt * a.y, v.z + dt * a.z);
    float3 pn = make_float3(p.x + dt * vn.x, p.y + dt * vn.y, p.z + dt * vn.z);
    if (S.wallbounds) {
        float *pc = &pn.x, *vc = &vn.x;
        for (int a2 = 0; a2 < 3; ++a2) {
            float lo = S.wallbounds[2 * a2], hi = S.wallbounds[2 * a2 + 1];
            if (pc[a2] < lo) {
                pc[a2] = lo + (lo - pc[a2]);
                vc[a2] = -vc[a2];
            } else if (pc[a2] > hi) {
                pc[a2] = hi - (pc[a2] - hi);
                vc[a2] = -vc[a2];
            }
        }
    }
    if (!(isfinite(pn.x) && isfinite(pn.y) && isfinite(pn.z))) atomicOr(S.status, (unsigned)STATUS_NONFINITE);
    st3(S.position, i, pn);
    st3(S.velocity, i, vn);
}

__global__ void k_step_forward(const SceneDesc *__restrict__ scenes, BlockMap map, int planes_only) {
    SPH_FOR_WORK(map)
    // a fused substep's plane-free solids were stepped by their force pass
    if (planes_only && !S.num_symmetry_planes) continue;
    if (item < active_count(S)) {
        const unsigned i = item;
        integrate(S, i, ld3(S.force, i), ld3(S.velocity, i), ld3(S.position, i));
    }
    SPH_END_WORK
}

// apply_plane_constraints (kernels/constraints.cl:1-30): project masked
// particles onto each of their planes and remove the normal velocity.
__global__ void k_plane_constraints(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (item < active_count(S)) {
        const unsigned i = item;
        const unsigned mask = S.plane_constraints_particles[i];
        if (mask) {
            float3 p = ld3(S.position, i), v = ld3(S.velocity, i);
            for (unsigned c = 0; c < S.num_plane_constraints && c < 32; ++c) {
                if (!(mask & (1u << c))) continue;
                const float *pl = S.plane_constraints + 6 * c;
                float3 pt = make_float3(pl[0], pl[1], pl[2]), nm = make_float3(pl[3], pl[4], pl[5]);
                float dp = dot3(nm, sub3(p, pt));
                p = make_float3(p.x - dp * nm.x, p.y - dp * nm.y, p.z - dp * nm.z);
                float dv = dot3(nm, v);
                v = make_float3(v.x - dv * nm.x, v.y - dv * nm.y, v.z - dv * nm.z);
            }
            st3(S.position, i, p);
            st3(S.velocity, i, v);
        }
    }
    SPH_END_WORK
}

// init_original_position (solids.cl:84-95)
__global__ void k_init_original_position(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (item < active_count(S)) st3(S.originalpos, item, ld3(S.position, item));
    SPH_END_WORK
}
