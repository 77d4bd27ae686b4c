// kernels_common.cuh -- device helpers shared by every sm_103a kernel of the
// pipeline: scene/block-map iteration, IEEE-exact distance tests, Kahan
// sums, the 27-cell neighbour walk and the symmetry-plane images.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_internal.h"

#define SPH_FULL_MASK 0xffffffffu
#define SPH_PI_F 3.1415926535f

// rho = m * sum * 315 / (64 pi h^9): the poly6 normalisation applied once
// to a particle's sum of (h^2 - r^2)^3 (common.cl:78-80, 610-690).
__device__ __forceinline__ float poly6_density(float sum, float h2, float h, float mass) {
    const float h3 = h2 * h;
    const float coef = 315.0f / (64.0f * SPH_PI_F * h3 * h3 * h3);
    return sum * coef * mass;
}

// A batched scene whose substep quota is used up: every kernel leaves it
// (fields, grid tables and scratch) untouched.
__device__ __forceinline__ bool scene_idle(const SceneDesc &S) { return S.steps_left && *S.steps_left == 0u; }

// Iterate the virtual blocks of a segment-aware launch.  Inside the body,
// `S` is the block's scene and `item` this thread's item index in it.
// Blocks of idle scenes are skipped (uniformly for the whole block).
#define SPH_FOR_WORK(map)                                                      \
    for (unsigned vb_ = blockIdx.x; vb_ < (map).num; vb_ += gridDim.x) {       \
        const BlockWork bw_ = (map).work[vb_];                                 \
        const SceneDesc &S = scenes[bw_.scene];                                \
        if (scene_idle(S)) continue;                                           \
        const unsigned item = bw_.first + threadIdx.x;
#define SPH_END_WORK }

// Active particle count, clamped to the store's capacity so that a bad `n`
// written from the host can never index past the fields.
__device__ __forceinline__ unsigned active_count(const SceneDesc &S) {
    unsigned n = *S.n;
    return n < S.pnum ? n : S.pnum;
}

// ---- IEEE-exact helpers (no FMA contraction) --------------------------------
// These reproduce the oracle's individually rounded float operations so that
// cell indices and neighbour decisions are bit-identical.

__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
// (x*x + y*y) + z*z, the order OpenCL's length()/dot() are restated in
__device__ __forceinline__ float norm2(float3 d) {
    return __fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y)), __fmul_rn(d.z, d.z));
}
// norm2(sub3(a, b)) with the x and y lanes in packed FP32x2 instructions
// (sm_100 and later; each lane rounds as the scalar instruction does, and
// a + (-b) is a - b exactly): the same value in 6 instructions instead of
// 8.  `b` is passed as its negated x, y pair and its z.
struct NegPoint {
    float2 nxy;
    float z;
};
__device__ __forceinline__ NegPoint neg_point(float3 b) {
    NegPoint o;
    o.nxy = make_float2(-b.x, -b.y);
    o.z = b.z;
    return o;
}
__device__ __forceinline__ float dist2(float4 a, const NegPoint &b) {
    const float2 dxy = __fadd2_rn(make_float2(a.x, a.y), b.nxy);
    const float dz = __fsub_rn(a.z, b.z);
    const float2 sq = __fmul2_rn(dxy, dxy);
    return __fadd_rn(__fadd_rn(sq.x, sq.y), __fmul_rn(dz, dz));
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// v - (2n) * dot(n, v - p): a mirror image across a symmetry plane
__device__ __forceinline__ float3 reflect3(float3 v, float3 p, float3 n) {
    float d = dot3(n, sub3(v, p));
    float3 tn = make_float3(2.f * n.x, 2.f * n.y, 2.f * n.z);
    return make_float3(__fsub_rn(v.x, __fmul_rn(tn.x, d)), __fsub_rn(v.y, __fmul_rn(tn.y, d)),
                       __fsub_rn(v.z, __fmul_rn(tn.z, d)));
}

// Squared-distance bounds equivalent to the reference's tests on
// dist = sqrt(r2) (correctly rounded):
//   r2 <= lt  <=>  dist <  h        r2 <= le  <=>  dist <= h
struct DistBounds {
    float lt, le;
};
__device__ __forceinline__ float next_up(float x) { return __uint_as_float(__float_as_uint(x) + 1u); }
__device__ __forceinline__ float next_down(float x) { return __uint_as_float(__float_as_uint(x) - 1u); }
__device__ __forceinline__ DistBounds dist_bounds(float h) {
    DistBounds b;
    float x = __fmul_rn(h, h);
    // largest x with sqrt_rn(x) < h
    float lt = x;
    for (int k = 0; k < 6 && lt > 0.f && __fsqrt_rn(lt) >= h; ++k) lt = next_down(lt);
    for (int k = 0; k < 6 && __fsqrt_rn(next_up(lt)) < h; ++k) lt = next_up(lt);
    // largest x with sqrt_rn(x) <= h
    float le = x;
    for (int k = 0; k < 6 && le > 0.f && __fsqrt_rn(le) > h; ++k) le = next_down(le);
    for (int k = 0; k < 6 && __fsqrt_rn(next_up(le)) <= h; ++k) le = next_up(le);
    b.lt = lt;
    b.le = le;
    return b;
}

// Kahan-compensated float accumulator.
// 1/x from the special-function unit (rcp.approx.ftz.f32: at most 1 ulp
// from the rounded reciprocal, denormals flushed).  One instruction in place
// of the IEEE-rounded reciprocal's sequence; deterministic, so every walk of
// a pair sum that uses it rounds alike.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

struct Kahan {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        float y = __fsub_rn(x, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};
struct Kahan3 {
    Kahan x, y, z;
    __device__ __forceinline__ void add(float3 v) { x.add(v.x); y.add(v.y); z.add(v.z); }
    __device__ __forceinline__ float3 get() const { return make_float3(x.s, y.s, z.s); }
};
// Blocked compensated sum of float3 terms: the terms of one stencil row are
// added in order into a row sum (rounded adds, no compensation), and each
// row's sum into the total with Kahan compensation.  end_row() closes a row;
// every walk over a particle's stencil calls it once for each of the nine
// rows, empty or outside the grid, so that two walks over the same
// neighbours in the same order give the same bits.
// The row sum's x and y lanes are one packed FP32x2 add.
struct BlockSum3 {
    float2 rxy = make_float2(0.f, 0.f);
    float rz = 0.f;
    Kahan3 total;
    __device__ __forceinline__ void add2(float2 vxy, float vz) {
        rxy = __fadd2_rn(rxy, vxy);
        rz = __fadd_rn(rz, vz);
    }
    __device__ __forceinline__ void add(float3 v) { add2(make_float2(v.x, v.y), v.z); }
    __device__ __forceinline__ void end_row() {
        total.add(make_float3(rxy.x, rxy.y, rz));
        rxy = make_float2(0.f, 0.f);
        rz = 0.f;
    }
    __device__ __forceinline__ float3 get() const { return total.get(); }
};

__device__ __forceinline__ float3 ld3(const float *p, size_t i) {
    return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
__device__ __forceinline__ void st3(float *p, size_t i, float3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
__device__ __forceinline__ float3 xyz(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }

// ---- cell walk ----------------------------------------------------------------

// FOR_PARTICLES_IN_RANGE (common.cl:49-68) on the cell-sorted order: the 27
// cells are visited z, y, x as in the reference, and because cells x-1..x+1
// of one (z, y) row are consecutive in the sort, each row is one contiguous
// range [celloffset[first], celloffset[last] + gridcount[last]).  `f(kk)` is
// called for every sorted neighbour index kk in the reference's order.
// `row_end()` is called after each of the nine rows (dz outer, dy inner),
// including rows outside the grid.
template <class F, class G>
__device__ __forceinline__ void for_each_neighbour(const SceneDesc &S, unsigned cell, F &&f, G &&row_end) {
    const unsigned R0 = S.gridres[0], R1 = S.gridres[1], R2 = S.gridres[2];
    const unsigned layer = R0 * R1;
    const unsigned cz = cell / layer;
    const unsigned rem = cell - cz * layer;
    const unsigned cy = rem / R0;
    const unsigned cx = rem - cy * R0;
    const unsigned x0 = cx > 0 ? cx - 1 : 0;
    const unsigned x1 = cx + 1 < R0 ? cx + 1 : R0 - 1;
    const unsigned *__restrict__ off = S.celloffset;
    const unsigned *__restrict__ cnt = S.gridcount;
    for (int dz = -1; dz <= 1; ++dz) {
        int z = (int)cz + dz;
        for (int dy = -1; dy <= 1; ++dy) {
            int y = (int)cy + dy;
            if (z >= 0 && z < (int)R2 && y >= 0 && y < (int)R1) {
                unsigned row = (unsigned)z * layer + (unsigned)y * R0;
                unsigned b = __ldg(off + row + x0);
                unsigned e = __ldg(off + row + x1) + __ldg(cnt + row + x1);
                if (e > S.pnum) e = S.pnum;  // only reachable with inconsistent host-written tables
                for (unsigned kk = b; kk < e; ++kk) f(kk);
            }
            row_end();
        }
    }
}
template <class F>
__device__ __forceinline__ void for_each_neighbour(const SceneDesc &S, unsigned cell, F &&f) {
    for_each_neighbour(S, cell, f, [] {});
}

// Row r of particle k's stencil (dz outer, dy inner, as the reference's
// z, y, x loops): cells x-1..x+1 of one (z, y) row are consecutive in the
// cell-sorted order, so a row is one range [b, e); empty when the row lies
// outside the grid.  The rows' presence and x extent are packed into one
// word when the stencil is set up.
struct StencilRows {
    unsigned cell, layer, R0;
    // bit r: row r lies in the grid; bit 9 + r: its cell x-1 exists;
    // bit 18 + r: its cell x+1 exists
    unsigned bits;
    __device__ __forceinline__ StencilRows(const SceneDesc &S, unsigned cell_) {
        cell = cell_;
        R0 = S.gridres[0];
        const unsigned R1 = S.gridres[1], R2 = S.gridres[2];
        layer = R0 * R1;
        const unsigned cz = cell / layer;
        const unsigned rem = cell - cz * layer;
        const unsigned cy = rem / R0;
        const unsigned cx = rem - cy * R0;
        const unsigned xm = cx > 0, xp = cx + 1 < R0;
        bits = 0;
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            const int z = (int)cz + r / 3 - 1, y = (int)cy + r % 3 - 1;
            if (z < 0 || z >= (int)R2 || y < 0 || y >= (int)R1) continue;
            bits |= (1u << r) | (xm << (9 + r)) | (xp << (18 + r));
        }
    }
    __device__ __forceinline__ void row(const SceneDesc &S, int r, unsigned *b, unsigned *e) const {
        *b = *e = 0;
        if (!((bits >> r) & 1u)) return;
        const int dz = r / 3 - 1, dy = r % 3 - 1;
        const unsigned c = (unsigned)((int)cell + dz * (int)layer + dy * (int)R0);
        const unsigned x0 = c - ((bits >> (9 + r)) & 1u), x1 = c + ((bits >> (18 + r)) & 1u);
        unsigned bb = __ldg(S.celloffset + x0);
        unsigned ee = __ldg(S.celloffset + x1) + __ldg(S.gridcount + x1);
        if (ee > S.pnum) ee = S.pnum;  // only with inconsistent host-written tables
        if (bb > ee) bb = ee;
        *b = bb;
        *e = ee;
    }
};

// ---- candidate masks -----------------------------------------------------------
// The first pair pass of a fused substep records, per stencil row r of
// sorted particle k, which candidates the later passes need: bit t of the
// row's 64-bit mask is candidate b_r + t; the low word is at
// nbmask[(2r) * pnum + k], the high word at nbmask[(2r+1) * pnum + k] (only
// for rows of more than 32 candidates); ncand[k] = SPH_NCAND_SCAN when a
// row exceeds 64 and the later passes must scan.

// Records row r's mask: low word always, high word for rows over 32.
__device__ __forceinline__ void store_row_mask(const SceneDesc &S, unsigned k, int r, unsigned len,
                                               unsigned long long bits) {
    S.nbmask[(size_t)(2 * r) * S.pnum + k] = (unsigned)bits;
    if (len > 32) S.nbmask[(size_t)(2 * r + 1) * S.pnum + k] = (unsigned)(bits >> 32);
}

// Row r's mask as recorded, with bits past the row's end cleared (every
// visited index stays inside [b, e)).
__device__ __forceinline__ unsigned long long load_row_mask(const SceneDesc &S, unsigned k, int r, unsigned len) {
    unsigned lo = S.nbmask[(size_t)(2 * r) * S.pnum + k];
    lo &= len >= 32 ? 0xffffffffu : (1u << len) - 1u;
    unsigned hi = 0;
    if (len > 32) {
        hi = S.nbmask[(size_t)(2 * r + 1) * S.pnum + k];
        hi &= len >= 64 ? 0xffffffffu : (1u << (len - 32)) - 1u;
    }
    return ((unsigned long long)hi << 32) | lo;
}

// Calls f(kk) for the candidates of particle k's recorded masks, in order.
// PREFETCH: the next row's bounds and low mask word are loaded while a row
// is walked (it pays in the corotational pass 2; the solid force passes,
// at their register cap, run slower with it).
template <bool PREFETCH = false, class F, class G>
__device__ __forceinline__ void for_each_masked(const SceneDesc &S, unsigned k, const StencilRows &rows, F &&f,
                                                G &&row_end) {
    unsigned nb = 0, ne = 0, nlo = 0;
    if (PREFETCH) {
        rows.row(S, 0, &nb, &ne);
        nlo = S.nbmask[k];
    }
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        unsigned b, e;
        unsigned long long mask;
        if (PREFETCH) {
            b = nb;
            e = ne;
            const unsigned len = e - b;
            const unsigned lo = nlo & (len >= 32u ? 0xffffffffu : (1u << len) - 1u);
            if (r < 8) {
                rows.row(S, r + 1, &nb, &ne);
                nlo = S.nbmask[(size_t)(2 * (r + 1)) * S.pnum + k];
            }
            unsigned hi = 0;
            if (len > 32u) {
                hi = S.nbmask[(size_t)(2 * r + 1) * S.pnum + k];
                hi &= len >= 64u ? 0xffffffffu : (1u << (len - 32u)) - 1u;
            }
            mask = ((unsigned long long)hi << 32) | lo;
        } else {
            rows.row(S, r, &b, &e);
            mask = load_row_mask(S, k, r, e - b);
        }
        // the row's two mask words in turn, with 32-bit bit scans
#pragma unroll 1
        for (unsigned w = 0, m = (unsigned)mask; w < 2; ++w, m = (unsigned)(mask >> 32), b += 32) {
            while (m) {
                const unsigned t = (unsigned)(__ffs(m) - 1);
                m &= m - 1u;
                f(b + t);
            }
        }
        row_end();
    }
}
template <bool PREFETCH = false, class F>
__device__ __forceinline__ void for_each_masked(const SceneDesc &S, unsigned k, const StencilRows &rows, F &&f) {
    for_each_masked<PREFETCH>(S, k, rows, f, [] {});
}

// ---- symmetry planes (the SYMMETRY blocks, e.g. common.cl:647-686) ----------

#define SPH_MAX_PLANES 8

struct Planes {
    float3 p[SPH_MAX_PLANES], n[SPH_MAX_PLANES];
    unsigned count;
    unsigned imask;  // planes that i itself passes (|n.(x_i - p)| <= h)
};

__device__ __forceinline__ void load_planes(const SceneDesc &S, float3 ipos, float h, Planes &P) {
    P.count = S.num_symmetry_planes < SPH_MAX_PLANES ? S.num_symmetry_planes : SPH_MAX_PLANES;
    P.imask = 0;
    for (unsigned k = 0; k < P.count; ++k) {
        const float *pl = S.symmetry_planes + 6 * k;
        P.p[k] = make_float3(pl[0], pl[1], pl[2]);
        P.n[k] = make_float3(pl[3], pl[4], pl[5]);
        // a zero normal makes jplane_dist 0 < 1e-5 for every j: never live
        bool live = !(P.n[k].x == 0.f && P.n[k].y == 0.f && P.n[k].z == 0.f);
        if (live && !(fabsf(dot3(P.n[k], sub3(ipos, P.p[k]))) > h)) P.imask |= 1u << k;
    }
}

// Planes of the i-live set that j also passes (|n.(x_j - p)| in [1e-5, h]).
// The reference tests (double)jd < 1.0e-5; jd converts to double exactly
// and 1e-5 lies strictly between two floats, so the test holds iff jd <=
// 0x1.4f8b58p-17f, the float just below it (FP32, no FP64 instruction per
// candidate).
#define SPH_PLANE_EPS_BELOW 0x1.4f8b58p-17f
__device__ __forceinline__ unsigned plane_jmask(const Planes &P, float3 jpos, float h) {
    unsigned m = 0;
    for (unsigned k = 0; k < P.count; ++k) {
        if (!(P.imask & (1u << k))) continue;
        float jd = fabsf(dot3(P.n[k], sub3(jpos, P.p[k])));
        if (!(jd > h) && !(jd <= SPH_PLANE_EPS_BELOW)) m |= 1u << k;
    }
    return m;
}
