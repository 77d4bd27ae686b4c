// kernels_fluid.cuh -- per-particle pair passes for density and WCSPH
// forces, the symplectic-Euler integrator and plane constraints (sm_103a).
//
// Pair passes run one thread per cell-sorted particle k (i =
// cellparticles[k]) so a warp covers a few neighbouring cells and shares
// their neighbour rows in L1; neighbours are streamed from the float4
// copies built by k_gather.  Sums are Kahan-compensated FP32.
#pragma once

#include "kernels_common.cuh"

#define SPH_PI_F 3.1415926535f

// compute_density (common.cl:610-690) and compute_original_density
// (solids.cl:99-170): rho_i = m * sum_j W_poly6(|x_j - x_i|), j = i
// included, plus mirror images across the symmetry planes.  With
// `original` the result goes to density0 and no neighbour count is kept.
//
// With `want_mask` (fused fluid substeps, where positions cannot change
// before the force pass) each fluid particle also records which of its
// stencil candidates lie within h, in stencil order, as a bitmask
// (SceneDesc::nbmask).
//
// Each warp stages its neighbour rows in shared memory: for every (z, y)
// row of the stencil the union of its lanes' ranges is copied once with
// coalesced float4 loads, and each lane then walks its own range from
// shared memory (lanes of one cell read the same address: a broadcast).
// Values, order and arithmetic are those of a direct walk; a union wider
// than the buffer (a warp that spans two grid rows) is read from global
// memory instead.  Dynamic shared memory: SPH_MASK_WORDS words per thread
// when masking, then SPH_STAGE float4 per warp.
#define SPH_STAGE 256

__host__ __device__ constexpr size_t density_smem_bytes(unsigned block, bool mask) {
    return (mask ? sizeof(unsigned) * SPH_MASK_WORDS * block : 0) + sizeof(float4) * SPH_STAGE * (block / 32);
}

__global__ void k_density(const SceneDesc *__restrict__ scenes, BlockMap map, int original, int want_mask) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    unsigned *sm_mask = reinterpret_cast<unsigned *>(sm_raw);
    float4 *wstage = reinterpret_cast<float4 *>(sm_raw + (want_mask ? sizeof(unsigned) * SPH_MASK_WORDS * blockDim.x
                                                                      : 0)) +
                     (threadIdx.x >> 5) * SPH_STAGE;
    const unsigned lane = threadIdx.x & 31u;
    SPH_FOR_WORK(map)
    const unsigned n = active_count(S);
    const bool mask = want_mask && S.nbmask && (S.programs & PROG_FLUIDS) && !original;
    if (mask)
        for (unsigned w = 0; w < SPH_MASK_WORDS; ++w) sm_mask[w * blockDim.x + threadIdx.x] = 0u;
    const bool active = item < n;
    const unsigned k = item;
    const unsigned i = active ? min(S.cellparticles[k], S.pnum - 1) : 0u;
    const float h = *S.h;
    const DistBounds B = dist_bounds(h);
    const float h2 = h * h;
    const float3 ipos = active ? xyz(S.spos[k]) : make_float3(0.f, 0.f, 0.f);
    Planes P;
    load_planes(S, ipos, h, P);
    if (!active) P.imask = 0;
    Kahan rho;
    unsigned count = 0, cand = 0;
    auto visit = [&](float3 jpos) {
        const float r2 = norm2(sub3(jpos, ipos));
        if (r2 <= B.le) {
            float d = fmaxf(h2 - r2, 0.f);
            rho.add(d * d * d);
            count += r2 <= B.lt;
            if (mask && cand < SPH_MASK_BITS) sm_mask[(cand >> 5) * blockDim.x + threadIdx.x] |= 1u << (cand & 31u);
        }
        ++cand;
        if (P.imask) {
            unsigned jm = plane_jmask(P, jpos, h);
            // subsets of jm in increasing order: the reference's
            // plane_bits order restricted to the subsets it keeps
            for (unsigned bits = (0u - jm) & jm; bits; bits = (bits - jm) & jm) {
                float3 ref = jpos;
                for (unsigned s = 0; s < P.count; ++s)
                    if (bits & (1u << s)) ref = reflect3(ref, P.p[s], P.n[s]);
                float m2 = norm2(sub3(ref, ipos));
                if (m2 <= B.lt) {
                    float d = fmaxf(h2 - m2, 0.f);
                    rho.add(d * d * d);
                    ++count;
                }
            }
        }
    };
    // the stencil of for_each_neighbour, row by row
    const unsigned R0 = S.gridres[0], R1 = S.gridres[1], R2 = S.gridres[2];
    const unsigned layer = R0 * R1;
    const unsigned cell = active ? S.gridcell[i] : 0u;
    const unsigned cz = cell / layer, rem = cell - cz * layer, cy = rem / R0, cx = rem - cy * R0;
    const unsigned x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < R0 ? cx + 1 : R0 - 1;
    const float4 *__restrict__ spos = S.spos;
    for (int dz = -1; dz <= 1; ++dz) {
        for (int dy = -1; dy <= 1; ++dy) {
            const int z = (int)cz + dz, y = (int)cy + dy;
            unsigned b = 0, e = 0;
            if (active && z >= 0 && z < (int)R2 && y >= 0 && y < (int)R1) {
                const unsigned row = (unsigned)z * layer + (unsigned)y * R0;
                b = __ldg(S.celloffset + row + x0);
                e = __ldg(S.celloffset + row + x1) + __ldg(S.gridcount + row + x1);
                if (e > S.pnum) e = S.pnum;
                if (b > e) b = e;
            }
            const unsigned ub = __reduce_min_sync(SPH_FULL_MASK, b < e ? b : 0xffffffffu);
            const unsigned ue = __reduce_max_sync(SPH_FULL_MASK, b < e ? e : 0u);
            if (ub < ue && ue - ub <= SPH_STAGE) {
                __syncwarp();
                for (unsigned t = lane; t < ue - ub; t += 32) wstage[t] = spos[ub + t];
                __syncwarp();
                for (unsigned kk = b; kk < e; ++kk) visit(xyz(wstage[kk - ub]));
            } else {
                for (unsigned kk = b; kk < e; ++kk) visit(xyz(spos[kk]));
            }
        }
    }
    if (active) {
        // poly6 normalisation 315 / (64 pi h^9), applied once
        const float h3 = h2 * h;
        const float coef = 315.0f / (64.0f * SPH_PI_F * h3 * h3 * h3);
        const float value = rho.s * coef * (*S.mass);
        if (original) {
            S.density0[i] = value;
        } else {
            S.density[i] = value;
            S.num_neighbours[i] = count;
            S.sdens[k] = value;
        }
        if (mask) {
            S.ncand[k] = cand;
            const unsigned words = (min(cand, (unsigned)SPH_MASK_BITS) + 31u) >> 5;
            for (unsigned w = 0; w < words; ++w)
                S.nbmask[(size_t)w * S.pnum + k] = sm_mask[w * blockDim.x + threadIdx.x];
        }
    }
    SPH_END_WORK
}

// APPLY_CUBE_BOUNDS(ipos, f, -2.0, 2.0) (common.cl:37-43): a repulsive
// band 0.2 wide inside [-2, 2]^3; the bounds are double literals, so the
// tests and the update are evaluated in double as in the source.
__device__ __forceinline__ float cube_bound(float p, float f) {
    const double mn = -2.0, mx = 2.0, band = (double)0.2f;
    double dp = (double)p;
    if (dp < mn + band) return (float)((double)f + (1.0 / (-(mn) + dp) - 5.0));
    if (dp > mx - band) return (float)((double)f - (1.0 / (mx - dp) - 5.0));
    return f;
}

// compute_forces_fluids (kernels/fluids.cl:1-63): pressure
// p = (rho - rho0) * stiffness, spiky-gradient pressure and Laplacian
// viscosity pair terms divided by rho_i rho_j, times the mass, plus the
// cube band.  A pair at exactly zero distance contributes nothing (the
// reference produces NaN there).  `fuse_step` also integrates particle i (step_forward) from
// the sorted copies, which no other thread reads afterwards.
__device__ __forceinline__ void integrate(const SceneDesc &S, unsigned i, float3 f, float3 v, float3 p);

// One particle's fluid force, visiting its within-h neighbours either by
// scanning the stencil (`masked` false) or through the candidate mask the
// density pass recorded (`masked` true, SPH_MASK_BITS candidates at most;
// a particle with more is scanned).  Both visit the same neighbours in the
// same order with the same arithmetic, so the results are identical.
template <bool MASKED>
__device__ __forceinline__ void fluid_force(const SceneDesc &S, unsigned k, int fuse_step) {
    const unsigned i = min(S.cellparticles[k], S.pnum - 1);
    const float h = *S.h;
    const DistBounds B = dist_bounds(h);
    const float rho0 = *S.restdens, stiff = *S.stiffness, visc = *S.viscosity;
    const float h3 = h * h * h;
    const float kv = 45.0f / (SPH_PI_F * h3 * h3);  // 45 / (pi h^6)
    const float3 ipos = xyz(S.spos[k]);
    const float3 ivel = xyz(S.svel[k]);
    const float rhoi = S.sdens[k];
    const float pi = (rhoi - rho0) * stiff;
    Kahan3 f;
    const float4 *__restrict__ spos = S.spos;
    const float4 *__restrict__ svel = S.svel;
    const float *__restrict__ sdens = S.sdens;
    auto pair = [&](unsigned kk) {
        if (kk == k) return;
        const float3 d = sub3(xyz(spos[kk]), ipos);
        const float r2 = norm2(d);
        // distinct particles at exactly zero distance: no defined
        // direction (the reference divides by the distance, fluids.cl:48)
        if (!(r2 <= B.le) || r2 == 0.f) return;
        const float rinv = rsqrtf(r2);
        const float dist = r2 * rinv;
        const float din = h - dist;
        const float rhoj = sdens[kk];
        const float pj = (rhoj - rho0) * stiff;
        const float inv_didj = 1.0f / (rhoi * rhoj);
        const float vterm = visc * din * kv;
        const float pterm = -(pi + pj) * 0.5f * rinv * din * din * kv;
        const float3 rv = xyz(svel[kk]) - ivel;
        f.add(make_float3((d.x * pterm + rv.x * vterm) * inv_didj, (d.y * pterm + rv.y * vterm) * inv_didj,
                          (d.z * pterm + rv.z * vterm) * inv_didj));
    };
    const unsigned cell = S.gridcell[i];
    bool scanned = true;
    if (MASKED) {
        const unsigned cand = S.ncand[k];
        if (cand <= SPH_MASK_BITS) {
            scanned = false;
            RowWalk rows(S, cell);
            unsigned rb = 0, rl = 0, base = 0, total = 0;
            bool have = rows.next(&rb, &rl);
            const unsigned words = (cand + 31u) >> 5;
            for (unsigned w = 0; w < words && have; ++w) {
                unsigned m = S.nbmask[(size_t)w * S.pnum + k];
                while (m) {
                    const unsigned b = (w << 5) + (unsigned)(__ffs(m) - 1);
                    m &= m - 1u;
                    while (have && b >= base + rl) {
                        base += rl;
                        have = rows.next(&rb, &rl);
                    }
                    if (!have) break;
                    pair(rb + (b - base));
                }
            }
            (void)total;
        }
    }
    if (scanned) for_each_neighbour(S, cell, pair);
    const float m = *S.mass;
    float3 fi = f.get() * m;
    fi.x = cube_bound(ipos.x, fi.x);
    fi.y = cube_bound(ipos.y, fi.y);
    fi.z = cube_bound(ipos.z, fi.z);
    st3(S.force, i, fi);
    if (fuse_step) integrate(S, i, fi, ivel, ipos);
}

__global__ void k_forces_fluids(const SceneDesc *__restrict__ scenes, BlockMap map, int fuse_step) {
    SPH_FOR_WORK(map)
    if (item < active_count(S)) fluid_force<false>(S, item, fuse_step);
    SPH_END_WORK
}

// The fused-substep force pass: walks the density pass's candidate masks.
__global__ void k_forces_fluids_masked(const SceneDesc *__restrict__ scenes, BlockMap map, int fuse_step) {
    SPH_FOR_WORK(map)
    if (item < active_count(S)) fluid_force<true>(S, item, fuse_step);
    SPH_END_WORK
}

// step_forward (common.cl:691-722): a = f/m + g, v += dt a, x += dt v;
// particles of a fixed (non-dynamic) body are skipped.  An optional
// `wallbounds` field (extension) mirrors particles that leave the box back
// inside and reverses their normal velocity.
__device__ __forceinline__ void integrate(const SceneDesc &S, unsigned i, float3 f, float3 v, float3 p) {
    if (S.body_number) {
        // a body number beyond body_dynamic's size is treated as dynamic
        unsigned b = S.body_number[i];
        if (b > 0 && b <= S.body_capacity && !S.body_dynamic[b - 1]) return;
    }
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

__global__ void k_step_forward(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
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
