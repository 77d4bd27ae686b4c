// kernels_solid.cuh -- elastic solids on sm_103a: the corotational linear
// model (kernels/solid_corotation.cl) with its polar decomposition,
// the St. Venant-Kirchhoff model (kernels/solid_svk.cl), the shared solid
// force pass, kinematic bodies (kernels/rigidbody.cl) and the scene-init
// kernels of common.cl.
//
// The 3x3 symmetric eigen-solver (SVK's Aqq inverse, jacobiInvert) keeps
// the reference's scheme (common.cl:101-305): eight Givens rotations, each
// zeroing the largest remaining off-diagonal.  The rotation for a pivot
// (a = off-diagonal, b, c = its diagonal pair) is the one with
// tan(2 theta) = 2a / (b - c) and |theta| <= pi/4, computed with
// Rutishauser's algebraic form t = tan(theta) = sign(tau) / (|tau| +
// sqrt(1 + tau^2)), tau = (b - c)/(2a), written as 2a sign(b - c) /
// (|b - c| + sqrt((b - c)^2 + 4a^2)), cos = rsqrt(1 + t^2), sin = t cos,
// instead of atan/cos/sin.  A zero pivot gives the identity (the reference
// evaluates atan(0/0) = NaN when b == c there).  The corotational rotation
// itself is the polar factor from Newton's iteration (polar_rotation_fp64).
#pragma once

#include "kernels_common.cuh"


// One Givens rotation of the symmetric 6-vector s ([xx,yy,zz,xy,xz,yz])
// zeroing the off-diagonal `off` (3, 4 or 5), applied in place to s and to
// the columns of the accumulated rotation p (row-major 3x3).  The index
// sets are those of common.cl:95-99.  The pivot's entries are picked and
// written back with selects, so all lanes run one arithmetic path and s and
// p stay in registers.
template <typename T>
__device__ __forceinline__ void givens_rotate(T s[6], T p[9], int off) {
    const bool o3 = off == 3, o4 = off == 4, o5 = off == 5;
    // xx = o5 ? 1 : 0, yy = o3 ? 1 : 2, (ex, ey) = o3 ? (4, 5) : o4 ? (3, 5) : (3, 4)
    const T a = o3 ? s[3] : o4 ? s[4] : s[5];
    const T b = o5 ? s[1] : s[0];
    const T c = o3 ? s[1] : s[2];
    const T ex = o3 ? s[4] : s[3];
    const T ey = o5 ? s[4] : s[5];
    T cs = 1, sn = 0;
    if (a != T(0)) {
        // tau = (b - c) / (2a), t = sign(tau) / (|tau| + sqrt(1 + tau^2)),
        // multiplied through by 2|a|: one sqrt and one division.  Equal
        // diagonals (tau = +-0) give t = sign(a) directly: there 4a^2 may
        // underflow to 0 in FP32 while a does not.
        const T d = b - c;
        T t;
        if (d == T(0)) {
            t = copysign(T(1), a);
        } else {
            const T r = sqrt(d * d + T(4) * a * a);
            t = (d < T(0) ? -T(2) : T(2)) * a / (fabs(d) + r);
        }
        cs = rsqrt(T(1) + t * t);
        sn = t * cs;
    }
    const T c2 = cs * cs, s2 = sn * sn, csn = cs * sn;
    const T nb = b * c2 + c * s2 + T(2) * a * csn;
    const T na = -b * csn + c * csn + a * (c2 - s2);
    const T nc = b * s2 + c * c2 - T(2) * a * csn;
    const T nex = ex * cs + ey * sn;
    const T ney = -ex * sn + ey * cs;
    s[0] = o5 ? s[0] : nb;
    s[1] = o5 ? nb : o3 ? nc : s[1];
    s[2] = o3 ? s[2] : nc;
    s[3] = o3 ? na : nex;
    s[4] = o4 ? na : o3 ? nex : ney;
    s[5] = o5 ? na : ney;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        T *row = p + 3 * r;
        const T px = o5 ? row[1] : row[0], py = o3 ? row[1] : row[2];
        const T nx = px * cs + py * sn, ny = -px * sn + py * cs;
        row[0] = o5 ? row[0] : nx;
        row[1] = o5 ? nx : o3 ? ny : row[1];
        row[2] = o3 ? row[2] : ny;
    }
}

template <typename T>
__device__ __forceinline__ int max_offdiag(const T t[6]) {
    T m = 0;
    int im = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T v = fabs(t[3 + k]);
        if (v > m) { m = v; im = k; }
    }
    return im + 3;
}

// jacobi(i, 0, 8, ...) of common.cl:257-295: eight rotations, each on the
// largest remaining off-diagonal.
template <typename T>
__device__ void jacobi8(const T in[6], T eig[3], T p[9]) {
    T t[6];
#pragma unroll
    for (int k = 0; k < 9; ++k) p[k] = (k % 4 == 0) ? T(1) : T(0);
#pragma unroll
    for (int k = 0; k < 6; ++k) t[k] = in[k];
#pragma unroll 1
    for (int it = 0; it < 8; ++it) givens_rotate(t, p, max_offdiag(t));
#pragma unroll
    for (int k = 0; k < 3; ++k) eig[k] = t[k];
}

// P diag(d) P^T as a symmetric 6-vector (multiplyBothSides, common.cl:169-186)
template <typename T>
__device__ __forceinline__ void p_d_pt(const T d[3], const T p[9], T out[6]) {
    auto e = [&](int r, int c) { return p[3 * r] * d[0] * p[3 * c] + p[3 * r + 1] * d[1] * p[3 * c + 1] + p[3 * r + 2] * d[2] * p[3 * c + 2]; };
    out[0] = e(0, 0); out[1] = e(1, 1); out[2] = e(2, 2);
    out[3] = e(0, 1); out[4] = e(0, 2); out[5] = e(1, 2);
}
// A S with S symmetric (multiplyAS, common.cl:187-199)
template <typename T>
__device__ __forceinline__ void mul_as(const T a[9], const T s[6], T out[9]) {
    const T S9[9] = {s[0], s[3], s[4], s[3], s[1], s[5], s[4], s[5], s[2]};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[3 * r + c] = a[3 * r] * S9[c] + a[3 * r + 1] * S9[3 + c] + a[3 * r + 2] * S9[6 + c];
}

// One step of Newton's polar iteration, X <- (X + X^-T) / 2, with X^-T the
// cofactor matrix over the determinant; returns max |change|.
template <typename T>
__device__ __forceinline__ T newton_polar_step(T X[9]) {
    const T C[9] = {X[4] * X[8] - X[5] * X[7], X[5] * X[6] - X[3] * X[8], X[3] * X[7] - X[4] * X[6],
                    X[2] * X[7] - X[1] * X[8], X[0] * X[8] - X[2] * X[6], X[1] * X[6] - X[0] * X[7],
                    X[1] * X[5] - X[2] * X[4], X[2] * X[3] - X[0] * X[5], X[0] * X[4] - X[1] * X[3]};
    const T rd = T(1) / (X[0] * C[0] + X[1] * C[1] + X[2] * C[2]);
    T delta = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const T nx = T(0.5) * (X[k] + C[k] * rd);
        delta = fmax(delta, fabs(nx - X[k]));
        X[k] = nx;
    }
    return delta;
}

// getR (common.cl:306-331): the rotation R of the polar decomposition
// A = R U.  The reference forms R = A (A^T A)^(-1/2) through its 8-rotation
// Jacobi eigensolver in FP64.  Here Newton's polar iteration
// X <- (X + X^-T) / 2 (Higham, 1986) converges quadratically to the same
// factor.  It starts from A scaled to the Frobenius norm of a rotation and
// runs in FP32 until the steps stall (about 1e-6), then takes one FP64
// step.  Write X = R (I + H + K), H symmetric, K skew: a Newton step
// squares H away but keeps K to first order, so the FP64 step leaves X
// orthogonal to ~1e-14 while the FP32 steps' rounding along the rotation
// (K, ~5e-8) stays.  R is thus an exact rotation within about one float
// ulp of the exact polar factor of A (max 9e-8 over 2,000 seeded
// near-rotations times stretches).  The FP64 pipe, narrow on GB300, does
// one step's work (about 1% of the pass).  A singular A (NaN in the
// reference) gives NaN here as well.
__device__ void polar_rotation_fp64(const float apq[9], float r[9]) {
    float X[9];
    float n2 = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        X[k] = apq[k];
        n2 += X[k] * X[k];
    }
    const float g = 1.7320508f * rsqrtf(n2);  // sqrt(3) / |A|_F
#pragma unroll
    for (int k = 0; k < 9; ++k) X[k] *= g;
#pragma unroll 1
    for (int it = 0; it < 24; ++it)
        if (!(newton_polar_step(X) > 1e-6f)) break;  // converged to FP32 (or NaN: stop)
    double D[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) D[k] = (double)X[k];
    newton_polar_step(D);
#pragma unroll
    for (int k = 0; k < 9; ++k) r[k] = (float)D[k];
}

// jacobiInvert (common.cl:296-305) in FP32
__device__ void sym_inverse(const float m[6], float out[6]) {
    float eig[3], P[9];
    jacobi8(m, eig, P);
    for (int k = 0; k < 3; ++k) eig[k] = 1.0f / eig[k];
    p_d_pt(eig, P, out);
}

// a0 b0 + a1 b1 + a2 b2 with every rounding written out: the products and
// sums below run in several kernels (the named and the fused passes), and
// each copy must round alike whatever the compiler would contract.
__device__ __forceinline__ float dot3_rn(float a0, float b0, float a1, float b1, float a2, float b2) {
    return __fmaf_rn(a2, b2, __fmaf_rn(a1, b1, __fmul_rn(a0, b0)));
}
__device__ __forceinline__ float3 mat_vec(const float m[9], float3 v) {
    return make_float3(dot3_rn(m[0], v.x, m[1], v.y, m[2], v.z), dot3_rn(m[3], v.x, m[4], v.y, m[5], v.z),
                       dot3_rn(m[6], v.x, m[7], v.y, m[8], v.z));
}
__device__ __forceinline__ float3 mat_t_vec(const float m[9], float3 v) {
    return make_float3(dot3_rn(m[0], v.x, m[3], v.y, m[6], v.z), dot3_rn(m[1], v.x, m[4], v.y, m[7], v.z),
                       dot3_rn(m[2], v.x, m[5], v.y, m[8], v.z));
}
__device__ __forceinline__ float3 sym_vec(const float s[6], float3 v) {
    return make_float3(dot3_rn(s[0], v.x, s[3], v.y, s[4], v.z), dot3_rn(s[3], v.x, s[1], v.y, s[5], v.z),
                       dot3_rn(s[4], v.x, s[5], v.y, s[2], v.z));
}
// m += a b^T, one fused multiply-add per entry, written out so that every
// copy of a sum rounds alike whatever the compiler would contract.
__device__ __forceinline__ void add_outer(float3 a, float3 b, float m[9]) {
    m[0] = __fmaf_rn(a.x, b.x, m[0]); m[1] = __fmaf_rn(a.x, b.y, m[1]); m[2] = __fmaf_rn(a.x, b.z, m[2]);
    m[3] = __fmaf_rn(a.y, b.x, m[3]); m[4] = __fmaf_rn(a.y, b.y, m[4]); m[5] = __fmaf_rn(a.y, b.z, m[5]);
    m[6] = __fmaf_rn(a.z, b.x, m[6]); m[7] = __fmaf_rn(a.z, b.y, m[7]); m[8] = __fmaf_rn(a.z, b.z, m[8]);
}

// Spiky gradient dir(d) * -45/(pi h^6) * (h - |d|)^2, zero beyond h
// (applyKernelGradient, common.cl:81-87); kv = 45/(pi h^6).
__device__ __forceinline__ float3 spiky_grad(float3 d, float h, float kv, float le) {
    float r2 = norm2(d);
    if (!(r2 <= le) || r2 == 0.f) return make_float3(0.f, 0.f, 0.f);
    float rinv = rsqrtf(r2);
    const float din = __fsub_rn(h, __fmul_rn(r2, rinv));
    const float s = -kv * din * din * rinv;
    return d * s;
}

struct SolidConsts {
    float h, h2, le, lt, kv, coef, mass;
};
__device__ __forceinline__ SolidConsts solid_consts(const SceneDesc &S) {
    SolidConsts c;
    c.h = *S.h;
    // rounded on its own, as the density pass rounds it: inlined, h * h
    // could otherwise fuse with a later h2 - r2 into one FMA in some kernels
    c.h2 = __fmul_rn(c.h, c.h);
    DistBounds b = dist_bounds(c.h);
    c.le = b.le;
    c.lt = b.lt;
    float h3 = c.h2 * c.h;
    c.kv = 45.0f / (SPH_PI_F * h3 * h3);
    c.coef = 315.0f / (64.0f * SPH_PI_F * h3 * h3 * h3);
    c.mass = *S.mass;
    return c;
}

// Images of j (and optionally of x0_j and x0_i) across the planes of `bits`.
__device__ __forceinline__ float3 reflect_bits(const Planes &P, unsigned bits, float3 v) {
    for (unsigned s = 0; s < P.count; ++s)
        if (bits & (1u << s)) v = reflect3(v, P.p[s], P.n[s]);
    return v;
}

// compute_rotations_and_strains (solid_corotation.cl:28-195): pass 1 sums
// Apq = sum W(|p|) p q^T (+ images), R = polar(Apq) in FP64, pass 2 sums
// D = sum (R^T p - q) m / rho0_i (x) gradW(-q) (+ images), strain =
// sym(D).  Body particles keep their rotation and strain.  This variant
// serves scenes with symmetry planes (every candidate's images are
// tested); k_rotations_and_strains serves the others.
__global__ void k_rotations_and_strains_planes(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (S.num_symmetry_planes == 0) continue;  // k_rotations_and_strains covers those
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        if (!(S.body_number && S.body_number[i] > 0)) {
            const SolidConsts C = solid_consts(S);
            const float3 ipos = xyz(S.spos[k]);
            const float3 ipos0 = ld3(S.originalpos, i);
            Planes P;
            load_planes(S, ipos, C.h, P);
            const unsigned cell = S.gridcell[i];
            float apq[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for_each_neighbour(S, cell, [&](unsigned kk) {
                const unsigned j = min(S.cellparticles[kk], S.pnum - 1);
                const float3 jpos = xyz(S.spos[kk]);
                const float3 jpos0 = ld3(S.originalpos, j);
                if (j != i) {
                    float3 p = sub3(jpos, ipos);
                    float r2 = norm2(p);
                    if (r2 <= C.le) {
                        float d = fmaxf(C.h2 - r2, 0.f);
                        add_outer(p * (d * d * d), sub3(jpos0, ipos0), apq);
                    }
                }
                if (P.imask) {
                    unsigned jm = plane_jmask(P, jpos, C.h);
                    for (unsigned bits = (0u - jm) & jm; bits; bits = (bits - jm) & jm) {
                        float3 p = sub3(reflect_bits(P, bits, jpos), ipos);
                        float r2 = norm2(p);
                        if (r2 <= C.lt) {
                            float d = fmaxf(C.h2 - r2, 0.f);
                            add_outer(p * (d * d * d), sub3(reflect_bits(P, bits, jpos0), ipos0), apq);
                        }
                    }
                }
            });
            for (int c = 0; c < 9; ++c) apq[c] *= C.coef;
            float R[9];
            polar_rotation_fp64(apq, R);
            for (int c = 0; c < 9; ++c) {
                S.apq_temp[9 * (size_t)i + c] = apq[c];
                S.intermediate[9 * (size_t)i + c] = apq[c];
                S.rotation[9 * (size_t)i + c] = R[c];
            }
            const float scale = C.mass / S.density0[i];
            float D[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for_each_neighbour(S, cell, [&](unsigned kk) {
                const unsigned j = min(S.cellparticles[kk], S.pnum - 1);
                const float3 jpos = xyz(S.spos[kk]);
                const float3 jpos0 = ld3(S.originalpos, j);
                if (j != i) {
                    float3 q = sub3(jpos0, ipos0);
                    float3 g = spiky_grad(-q, C.h, C.kv, C.le);
                    if (g.x != 0.f || g.y != 0.f || g.z != 0.f) {
                        float3 u = mat_t_vec(R, sub3(jpos, ipos)) - q;
                        add_outer(u * scale, g, D);
                    }
                }
                if (P.imask) {
                    unsigned jm = plane_jmask(P, jpos, C.h);
                    for (unsigned bits = (0u - jm) & jm; bits; bits = (bits - jm) & jm) {
                        float3 p = mat_t_vec(R, sub3(reflect_bits(P, bits, jpos), ipos));
                        if (norm2(p) <= C.lt) {
                            float3 q = sub3(reflect_bits(P, bits, jpos0), ipos0);
                            add_outer((p - q) * scale, spiky_grad(-q, C.h, C.kv, C.le), D);
                        }
                    }
                }
            });
            float *st = S.strain + 6 * (size_t)i;
            st[0] = D[0];
            st[1] = D[4];
            st[2] = D[8];
            st[3] = 0.5f * (D[1] + D[3]);
            st[4] = 0.5f * (D[2] + D[6]);
            st[5] = 0.5f * (D[5] + D[7]);
        }
    }
    SPH_END_WORK
}

// Stress laws (solid_corotation.cl:197-208; solid_svk.cl:45-80).  Every
// rounding is written out: the laws run in the named stress pass and inside
// the fused first solid pass, and both must give the same bits.

struct Lame {
    float lam, mu2;  // lambda and 2 mu
};
__device__ __forceinline__ Lame lame(const SceneDesc &S) {
    const float E = *S.youngs_modulus, nu = *S.poisson;
    Lame L;
    L.lam = __fdiv_rn(__fdiv_rn(__fmul_rn(E, nu), __fadd_rn(1.0f, nu)), __fsub_rn(1.0f, __fmul_rn(2.0f, nu)));
    L.mu2 = __fmul_rn(2.0f, __fdiv_rn(__fdiv_rn(E, 2.0f), __fadd_rn(1.0f, nu)));
    return L;
}

__device__ __forceinline__ void corot_stress(const SceneDesc &S, const float e[6], float o[6]) {
    const Lame L = lame(S);
    const float lt = __fmul_rn(L.lam, __fadd_rn(__fadd_rn(e[0], e[1]), e[2]));
    for (int c = 0; c < 3; ++c) o[c] = __fmaf_rn(L.mu2, e[c], lt);
    for (int c = 3; c < 6; ++c) o[c] = __fmul_rn(L.mu2, e[c]);
}

__device__ __forceinline__ void svk_stress(const SceneDesc &S, const float f[9], float o[6]) {
    const Lame L = lame(S);
    // Green strain G = (F^T F - I) / 2
    auto ftf = [&](int r, int c) { return dot3_rn(f[r], f[c], f[3 + r], f[3 + c], f[6 + r], f[6 + c]); };
    const float g[6] = {__fmaf_rn(0.5f, ftf(0, 0), -0.5f), __fmaf_rn(0.5f, ftf(1, 1), -0.5f),
                        __fmaf_rn(0.5f, ftf(2, 2), -0.5f), __fmul_rn(0.5f, ftf(0, 1)),
                        __fmul_rn(0.5f, ftf(0, 2)), __fmul_rn(0.5f, ftf(1, 2))};
    const float first = __fmul_rn(L.lam, __fadd_rn(__fadd_rn(g[0], g[1]), g[2]));
    const float sv[6] = {__fmaf_rn(L.mu2, g[0], first), __fmaf_rn(L.mu2, g[1], first), __fmaf_rn(L.mu2, g[2], first),
                         __fmul_rn(L.mu2, g[3]), __fmul_rn(L.mu2, g[4]), __fmul_rn(L.mu2, g[5])};
    // F S (S symmetric), then the Cauchy stress (F S F^T) / det F
    const float S9[9] = {sv[0], sv[3], sv[4], sv[3], sv[1], sv[5], sv[4], sv[5], sv[2]};
    float fs[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            fs[3 * r + c] = dot3_rn(f[3 * r], S9[c], f[3 * r + 1], S9[3 + c], f[3 * r + 2], S9[6 + c]);
    const float c0 = __fsub_rn(__fmul_rn(f[4], f[8]), __fmul_rn(f[5], f[7]));
    const float c1 = __fsub_rn(__fmul_rn(f[3], f[8]), __fmul_rn(f[5], f[6]));
    const float c2 = __fsub_rn(__fmul_rn(f[3], f[7]), __fmul_rn(f[4], f[6]));
    const float det = __fadd_rn(__fsub_rn(__fmul_rn(f[0], c0), __fmul_rn(f[1], c1)), __fmul_rn(f[2], c2));
    const float rdet = __fdiv_rn(1.0f, det);
    auto cau = [&](int r, int c) {
        return __fmul_rn(dot3_rn(fs[3 * r], f[3 * c], fs[3 * r + 1], f[3 * c + 1], fs[3 * r + 2], f[3 * c + 2]), rdet);
    };
    o[0] = cau(0, 0);
    o[1] = cau(1, 1);
    o[2] = cau(2, 2);
    o[3] = cau(0, 1);
    o[4] = cau(0, 2);
    o[5] = cau(1, 2);
}

// The corotational force pass uses a particle's rotation and stress only
// as the product R sigma -- or, for a body particle, R alone (its pairs use
// the partner's stress).  N = R sigma (row-major), or R for a body.
__device__ __forceinline__ void corot_nmat(const float R[9], const float s[6], bool body, float N[9]) {
    if (body) {
        for (int c = 0; c < 9; ++c) N[c] = R[c];
        return;
    }
    const float S9[9] = {s[0], s[3], s[4], s[3], s[1], s[5], s[4], s[5], s[2]};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) N[3 * r + c] = dot3_rn(R[3 * r], S9[c], R[3 * r + 1], S9[3 + c], R[3 * r + 2], S9[6 + c]);
}

// A particle's stress into the field and the sorted copies: sstress[k]
// (sigma with mass/density) and, for the corotational model, srot[k] = N
// (with mass/density in w).
__device__ __forceinline__ void store_stress(const SceneDesc &S, unsigned i, unsigned k, const float o[6], float mrho,
                                             const float *R, bool body) {
    for (int c = 0; c < 6; ++c) S.stress[6 * (size_t)i + c] = o[c];
    S.sstress[2 * (size_t)k] = make_float4(o[0], o[1], o[2], o[3]);
    S.sstress[2 * (size_t)k + 1] = make_float4(o[4], o[5], mrho, 0.f);
    if (R && S.srot) {
        float N[9];
        corot_nmat(R, o, body, N);
        for (int c = 0; c < 3; ++c)
            S.srot[3 * (size_t)k + c] = make_float4(N[3 * c], N[3 * c + 1], N[3 * c + 2], c == 0 ? mrho : 0.f);
    }
}

// compute_stresses, corotational (solid_corotation.cl:9-26,197-208):
// isotropic Hooke's law with the Lame constants.
__global__ void k_stresses_corot(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (item < active_count(S)) {
        float e[6], o[6];
        for (int c = 0; c < 6; ++c) e[c] = S.strain[6 * (size_t)item + c];
        corot_stress(S, e, o);
        for (int c = 0; c < 6; ++c) S.stress[6 * (size_t)item + c] = o[c];
    }
    SPH_END_WORK
}

// compute_deformations (solid_svk.cl:82-175): F = Apq Aqq^-1.  The poly6
// normalisation cancels in the product and is left out.  Scenes with
// symmetry planes; k_deformations serves the others.
__global__ void k_deformations_planes(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (S.num_symmetry_planes == 0) continue;  // k_deformations covers those
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const SolidConsts C = solid_consts(S);
        const float3 ipos = xyz(S.spos[k]);
        const float3 ipos0 = ld3(S.originalpos, i);
        Planes P;
        load_planes(S, ipos, C.h, P);
        float apq[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        float aqq[6] = {0, 0, 0, 0, 0, 0};
        auto contrib = [&](float3 p, float3 q, float w) {
            add_outer(p * w, q, apq);
            float3 wq = q * w;
            aqq[0] += wq.x * q.x; aqq[3] += wq.x * q.y; aqq[4] += wq.x * q.z;
            aqq[1] += wq.y * q.y; aqq[5] += wq.y * q.z;
            aqq[2] += wq.z * q.z;
        };
        for_each_neighbour(S, S.gridcell[i], [&](unsigned kk) {
            const unsigned j = min(S.cellparticles[kk], S.pnum - 1);
            const float3 jpos = xyz(S.spos[kk]);
            const float3 jpos0 = ld3(S.originalpos, j);
            if (j != i) {
                float3 p = sub3(jpos, ipos);
                float r2 = norm2(p);
                if (r2 <= C.le) {
                    float d = fmaxf(C.h2 - r2, 0.f);
                    contrib(p, sub3(jpos0, ipos0), d * d * d);
                }
            }
            if (P.imask) {
                unsigned jm = plane_jmask(P, jpos, C.h);
                for (unsigned bits = (0u - jm) & jm; bits; bits = (bits - jm) & jm) {
                    float3 p = sub3(reflect_bits(P, bits, jpos), ipos);
                    float r2 = norm2(p);
                    if (r2 <= C.lt) {
                        float d = fmaxf(C.h2 - r2, 0.f);
                        contrib(p, sub3(reflect_bits(P, bits, jpos0), ipos0), d * d * d);
                    }
                }
            }
        });
        float inv[6];
        sym_inverse(aqq, inv);
        float F[9];
        mul_as(apq, inv, F);
        for (int c = 0; c < 9; ++c) S.deformation[9 * (size_t)i + c] = F[c];
    }
    SPH_END_WORK
}

// compute_stresses, SVK (solid_svk.cl:1-80): E = (F^T F - I)/2,
// S = lambda tr(E) I + 2 mu E, sigma = F S F^T / det F.
__global__ void k_stresses_svk(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    // a mixed scene's fluid particles have no deformation gradient
    if (item < active_count(S) && !(S.phase && S.phase[item] == 0u)) {
        float f[9], o[6];
        for (int c = 0; c < 9; ++c) f[c] = S.deformation[9 * (size_t)item + c];
        svk_stress(S, f, o);
        for (int c = 0; c < 6; ++c) S.stress[6 * (size_t)item + c] = o[c];
    }
    SPH_END_WORK
}

// compute_forces_solids (solid_corotation.cl:215-403 when COROT,
// solid_svk.cl:182-367 otherwise): elastic pair forces from the stresses
// in the rest configuration, rotated by R_i / R_j for the corotational
// model, plus Laplacian viscosity; symmetry images; the force, its elastic
// and viscous parts and the test-axis cut-off force are all written.
// Scenes with symmetry planes; k_forces_solids serves the others.
template <bool COROT>
__global__ void k_forces_solids_planes(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (S.num_symmetry_planes == 0) continue;  // k_forces_solids covers those
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const SolidConsts C = solid_consts(S);
        const float3 ipos = xyz(S.spos[k]);
        const float3 ivel = ld3(S.velocity, i);
        const float3 ipos0 = ld3(S.originalpos, i);
        float si[6], Ri[9];
        for (int c = 0; c < 6; ++c) si[c] = S.stress[6 * (size_t)i + c];
        if (COROT)
            for (int c = 0; c < 9; ++c) Ri[c] = S.rotation[9 * (size_t)i + c];
        const float rho0i = S.density0[i];
        Planes P;
        load_planes(S, ipos, C.h, P);
        Kahan3 fe_s, fv_s, fec_s, fvc_s;
        for_each_neighbour(S, S.gridcell[i], [&](unsigned kk) {
            const unsigned j = min(S.cellparticles[kk], S.pnum - 1);
            const float3 jpos = xyz(S.spos[kk]);
            const float3 jpos0 = ld3(S.originalpos, j);
            const float3 x = sub3(ipos0, jpos0);
            const bool direct = j != i && (norm2(x) <= C.le || norm2(sub3(jpos, ipos)) <= C.le);
            unsigned jm = 0;
            if (P.imask) jm = plane_jmask(P, jpos, C.h);
            if (!direct && !jm) return;
            const float3 jvel = ld3(S.velocity, j);
            const float vivj = C.mass * C.mass / rho0i / S.density0[j];
            const float mrj = C.mass / S.density[j];
            float sj[6], Rj[9];
            for (int c = 0; c < 6; ++c) sj[c] = S.stress[6 * (size_t)j + c];
            if (COROT)
                for (int c = 0; c < 9; ++c) Rj[c] = S.rotation[9 * (size_t)j + c];
            if (direct) {
                const float3 gx = spiky_grad(x, C.h, C.kv, C.le);
                const float3 f_ji = sym_vec(si, gx) * (-vivj);
                const float3 f_ij = S.body_number[j] > 0 ? -f_ji : sym_vec(sj, -gx) * (-vivj);
                const float3 fe = COROT ? mat_vec(Rj, f_ij) - mat_vec(Ri, f_ji) : f_ij - f_ji;
                const float r2 = norm2(sub3(jpos, ipos));
                const float lap = r2 <= C.le ? C.kv * (C.h - sqrtf(r2)) : 0.f;
                const float3 fv = (jvel - ivel) * (mrj * lap);
                fe_s.add(fe);
                fv_s.add(fv);
                fec_s.add(fe);
                fvc_s.add(fv);
            }
            for (unsigned bits = (0u - jm) & jm; bits; bits = (bits - jm) & jm) {
                const float3 rp = reflect_bits(P, bits, jpos);
                const float3 rp0 = reflect_bits(P, bits, jpos0);
                const float3 rip0 = reflect_bits(P, bits, ipos0);
                const float3 xm = sub3(ipos0, rp0);
                const float3 refx = sub3(rip0, jpos0);
                const float3 f_ji = sym_vec(si, spiky_grad(xm, C.h, C.kv, C.le)) * (-vivj);
                float3 f_ij = sym_vec(sj, spiky_grad(-refx, C.h, C.kv, C.le)) * (-vivj);
                if (COROT) f_ij = mat_vec(Rj, f_ij);
                // reflect back across the subset's planes, highest first; the
                // last normal used (the lowest plane's) also mirrors j's
                // velocity, as in the source
                float3 nlast = make_float3(0.f, 0.f, 0.f);
                for (int s = (int)P.count - 1; s >= 0; --s) {
                    if (!(bits & (1u << s))) continue;
                    nlast = P.n[s];
                    f_ij = f_ij - nlast * (2.f * dot3(nlast, f_ij));
                }
                const float3 fe = COROT ? f_ij - mat_vec(Ri, f_ji) : f_ij - f_ji;
                const float3 refvel = jvel - nlast * (2.f * dot3(nlast, jvel));
                const float r2 = norm2(sub3(rp, ipos));
                const float lap = r2 <= C.le ? C.kv * (C.h - sqrtf(r2)) : 0.f;
                const float3 fv = (refvel - ivel) * (mrj * lap);
                fe_s.add(fe);
                fv_s.add(fv);
                if (!(bits & 1u)) {
                    fec_s.add(fe);
                    fvc_s.add(fv);
                }
            }
        });
        const float visc = *S.viscosity;
        const float3 fe = fe_s.get() * 0.5f, fv = fv_s.get() * visc;
        st3(S.force, i, fe + fv);
        st3(S.force_elastic, i, fe);
        st3(S.force_viscous, i, fv);
        st3(S.cutoff_force, i, fec_s.get() * 0.5f + fvc_s.get() * visc);
    }
    SPH_END_WORK
}

// ---- plane-free solids: sorted copies and candidate masks -------------------
//
// Scenes without symmetry planes.  The first pair pass of the substep
// (k_rotations_and_strains, k_deformations) walks every stencil candidate
// from the cell-sorted copies (spos, spos0) and records, per row as the
// fluid density pass does, the candidates that are direct neighbours of
// the force pass: j != i with the rest distance |x0_j - x0_i| <= h or the
// current distance |x_j - x_i| <= h.  The corotational second pass and, in
// a fused substep, the force pass walk only those.  They visit the same
// neighbours in the same order with the same arithmetic as a walk over all
// candidates, so the results are identical; the named force pass (whose
// masks may be stale) scans.

// Pass 1 of the plane-free solid passes over particle k's stencil rows,
// from the cell-sorted copies.  Each row is taken in chunks of 32
// candidates, one mask word each: a tight loop over the chunk records the
// mask bits (|p| <= h or |q| <= h, k itself excluded) and the bits of the
// chunk's current neighbours (|p| <= h, k itself included).  Then a walk
// over those neighbours, in candidate order, adds each one's density term
// (the density pass's blocked sum, in its order: row sums in candidate
// order, Kahan-added row by row) and for j != i runs sum(p, q, w),
// w = (h^2 - |p|^2)^3.  The scan loop thus stays free of the sums' work,
// which otherwise every lane would issue whenever any lane of its warp met
// a neighbour, and every sum sees the neighbours in the order a plain scan
// would.  Only a row's first 64 candidates have mask bits; `overflow`
// records a longer row.
//
// The density terms are summed whether or not the caller stores them: a
// flag tested inside the loops lets the compiler emit one copy of them per
// value, and copies may contract the sums' products differently, which
// would break the equality of the named and fused passes.
template <class Sum>
__device__ __forceinline__ void scan_solid_rows(const SceneDesc &S, unsigned k, const StencilRows &rows,
                                                float3 ipos, float3 ipos0, const SolidConsts &C, Kahan &rho,
                                                unsigned &count, unsigned &total, bool &overflow, Sum &&sum) {
    const float4 *__restrict__ spos = S.spos;
    const float4 *__restrict__ spos0 = S.spos0;
    const NegPoint nip = neg_point(ipos), nip0 = neg_point(ipos0);
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        unsigned b, e;
        rows.row(S, r, &b, &e);
        const unsigned len = e - b;
        float rowsum = 0.f;  // the row's density terms, as the density pass sums them
#pragma unroll 1
        for (unsigned c0 = 0; c0 < len; c0 += 32) {
            const unsigned cb = b + c0, cn = min(len - c0, 32u);
            unsigned bits = 0, near = 0;
#pragma unroll 4
            for (unsigned t = 0; t < cn; ++t) {
                const unsigned kk = cb + t;
                const float r2 = dist2(spos[kk], nip);
                const float q2 = dist2(spos0[kk], nip0);
                const unsigned bit = 1u << t;
                if (r2 <= C.le) near |= bit;
                if (r2 <= C.le || q2 <= C.le) bits |= bit;
            }
            if (k - cb < cn) bits &= ~(1u << (k - cb));  // k itself has no mask bit
            // mask words 2r and 2r + 1 (store_row_mask's layout)
            if (c0 < 64) S.nbmask[(size_t)(2 * r + (c0 >> 5)) * S.pnum + k] = bits;
            while (near) {
                const unsigned kk = cb + (unsigned)(__ffs(near) - 1);
                near &= near - 1u;
                const float3 p = sub3(xyz(spos[kk]), ipos);
                const float r2 = norm2(p);
                const float d = fmaxf(C.h2 - r2, 0.f);
                const float w = d * d * d;
                rowsum = __fadd_rn(rowsum, w);
                count += r2 <= C.lt;
                if (kk != k) sum(p, sub3(xyz(spos0[kk]), ipos0), w);
            }
        }
        rho.add(rowsum);
        overflow |= len > 64;
        total += len;
    }
}

// compute_rotations_and_strains (solid_corotation.cl:28-195) for
// plane-free scenes: pass 1 (scan_solid_rows) sums Apq over candidates
// with |p| <= h and records the masks, R = polar(Apq), pass 2 sums D over
// the masked candidates with |q| <= h.  Body particles keep their rotation and strain
// (their masks are still recorded).  Also writes the sorted rotation copy.
// At most 64 registers (about 100 bytes spill to L1): eight 128-thread
// blocks per SM.  On batched-256, with the packed distance tests: 64 ->
// 0.581 ms, 72 -> 0.590 ms, 80 -> 0.626 ms.
__global__ void __maxnreg__(64) k_rotations_and_strains(const SceneDesc *__restrict__ scenes, BlockMap map,
                                                        int with_density, int with_stress) {
    SPH_FOR_WORK(map)
    if (S.num_symmetry_planes || !S.spos0) continue;  // sorted copies exist with solids.cl
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const SolidConsts C = solid_consts(S);
        const float4 p4 = S.spos[k], q4 = S.spos0[k];
        const float3 ipos = xyz(p4), ipos0 = xyz(q4);
        const StencilRows rows(S, S.gridcell[i]);
        const float4 *__restrict__ spos = S.spos;
        const float4 *__restrict__ spos0 = S.spos0;
        float apq[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        unsigned total = 0, count = 0;
        bool overflow = false;
        Kahan rho;
        scan_solid_rows(S, k, rows, ipos, ipos0, C, rho, count, total, overflow,
                        [&](float3 p, float3 q, float w) { add_outer(p * w, q, apq); });
        S.ncand[k] = overflow ? SPH_NCAND_SCAN : total;
        // the sorted density copy (scratch) is written either way: a value
        // the named pass would discard lets the compiler emit a second copy
        // of this kernel without the density sums, whose other sums may
        // then round differently
        const float value = poly6_density(rho.s, C.h2, C.h, C.mass);
        S.sdens[k] = value;
        if (with_density) {
            S.density[i] = value;
            S.num_neighbours[i] = count;
        }
        float R[9];
        if (__float_as_uint(q4.w) > 0) {
            // a body particle: rotation and strain stay as they are
            for (int c = 0; c < 9; ++c) R[c] = S.rotation[9 * (size_t)i + c];
        } else {
            for (int c = 0; c < 9; ++c) apq[c] *= C.coef;
            polar_rotation_fp64(apq, R);
            for (int c = 0; c < 9; ++c) {
                S.apq_temp[9 * (size_t)i + c] = apq[c];
                S.intermediate[9 * (size_t)i + c] = apq[c];
                S.rotation[9 * (size_t)i + c] = R[c];
            }
            const float scale = C.mass / S.density0[i];
            float D[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            // the masks hold no bit for k itself
            auto pass2_masked = [&](unsigned kk) {
                const float3 q = sub3(xyz(spos0[kk]), ipos0);
                const float3 g = spiky_grad(-q, C.h, C.kv, C.le);
                if (g.x != 0.f || g.y != 0.f || g.z != 0.f) {
                    const float3 u = mat_t_vec(R, sub3(xyz(spos[kk]), ipos)) - q;
                    add_outer(u * scale, g, D);
                }
            };
            auto pass2 = [&](unsigned kk) {
                if (kk != k) pass2_masked(kk);
            };
            if (overflow) for_each_neighbour(S, S.gridcell[i], pass2);
            else for_each_masked<true>(S, k, rows, pass2_masked);
            float *st = S.strain + 6 * (size_t)i;
            st[0] = D[0];
            st[1] = D[4];
            st[2] = D[8];
            st[3] = 0.5f * (D[1] + D[3]);
            st[4] = 0.5f * (D[2] + D[6]);
            st[5] = 0.5f * (D[5] + D[7]);
        }
        if (with_stress && S.sstress) {
            // compute_stresses for this particle, as k_stresses_sorted<true>
            // would (a body particle keeps its strain)
            float e[6], o[6];
            for (int c = 0; c < 6; ++c) e[c] = S.strain[6 * (size_t)i + c];
            corot_stress(S, e, o);
            store_stress(S, i, k, o, __fdiv_rn(C.mass, S.sdens[k]), R, __float_as_uint(q4.w) > 0);
        }
    }
    SPH_END_WORK
}

// compute_deformations (solid_svk.cl:82-175) for plane-free scenes, from
// the sorted copies, recording the candidate masks.  No register cap (80):
// on batched-256 uncapped 0.441 ms, 72 -> 0.446 ms, 64 -> 0.451 ms.
__global__ void k_deformations(const SceneDesc *__restrict__ scenes, BlockMap map, int with_density,
                               int with_stress) {
    SPH_FOR_WORK(map)
    if (S.num_symmetry_planes || !S.spos0) continue;  // sorted copies exist with solids.cl
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const SolidConsts C = solid_consts(S);
        const float3 ipos = xyz(S.spos[k]), ipos0 = xyz(S.spos0[k]);
        const StencilRows rows(S, S.gridcell[i]);
        float apq[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        float aqq[6] = {0, 0, 0, 0, 0, 0};
        unsigned total = 0, count = 0;
        bool overflow = false;
        Kahan rho;
        scan_solid_rows(S, k, rows, ipos, ipos0, C, rho, count, total, overflow,
                        [&](float3 p, float3 q, float w) {
                            add_outer(p * w, q, apq);
                            const float3 wq = q * w;
                            aqq[0] = __fmaf_rn(wq.x, q.x, aqq[0]);
                            aqq[1] = __fmaf_rn(wq.y, q.y, aqq[1]);
                            aqq[2] = __fmaf_rn(wq.z, q.z, aqq[2]);
                            aqq[3] = __fmaf_rn(wq.x, q.y, aqq[3]);
                            aqq[4] = __fmaf_rn(wq.x, q.z, aqq[4]);
                            aqq[5] = __fmaf_rn(wq.y, q.z, aqq[5]);
                        });
        S.ncand[k] = overflow ? SPH_NCAND_SCAN : total;
        // the sorted density copy (scratch) is written either way: a value
        // the named pass would discard lets the compiler emit a second copy
        // of this kernel without the density sums, whose other sums may
        // then round differently
        const float value = poly6_density(rho.s, C.h2, C.h, C.mass);
        S.sdens[k] = value;
        if (with_density) {
            S.density[i] = value;
            S.num_neighbours[i] = count;
        }
        float inv[6];
        sym_inverse(aqq, inv);
        float F[9];
        mul_as(apq, inv, F);
        for (int c = 0; c < 9; ++c) S.deformation[9 * (size_t)i + c] = F[c];
        if (with_stress && S.sstress) {
            // compute_stresses for this particle, as k_stresses_sorted<false> would
            float o[6];
            svk_stress(S, F, o);
            store_stress(S, i, k, o, __fdiv_rn(C.mass, S.sdens[k]), nullptr, false);
        }
    }
    SPH_END_WORK
}

// compute_stresses in a fused substep: per sorted particle k, the field
// stress[i] and the sorted copies sstress[k] (with mass/density) and, for
// the corotational model, srot[k] = N (with mass/density in w).
template <bool COROT>
__global__ void k_stresses_sorted(const SceneDesc *__restrict__ scenes, BlockMap map, int planes_only) {
    SPH_FOR_WORK(map)
    // a plane-free scene's first pass stored its stresses already
    if (planes_only && !S.num_symmetry_planes) continue;
    if (item < active_count(S) && S.sstress) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        float o[6];
        if (COROT) {
            float e[6];
            for (int c = 0; c < 6; ++c) e[c] = S.strain[6 * (size_t)i + c];
            corot_stress(S, e, o);
        } else {
            float f[9];
            for (int c = 0; c < 9; ++c) f[c] = S.deformation[9 * (size_t)i + c];
            svk_stress(S, f, o);
        }
        const float mrho = __fdiv_rn(*S.mass, S.sdens[k]);
        if (COROT) {
            float R[9];
            for (int c = 0; c < 9; ++c) R[c] = S.rotation[9 * (size_t)i + c];
            store_stress(S, i, k, o, mrho, R, S.body_number[i] > 0);
        } else {
            store_stress(S, i, k, o, mrho, nullptr, false);
        }
    }
    SPH_END_WORK
}

// One side of a solid pair: position, rest position, velocity, densities,
// stress, and for the corotational model N (corot_nmat) -- the partner's
// side of a pair needs N, this particle's side needs sigma and R sigma.
struct SolidSide {
    float3 pos, pos0, vel;
    float inv_rho0;  // 1 / density0, correctly rounded
    float mrho;      // mass / density, correctly rounded
    float s[6];      // stress
    float N[9];      // corotational: R sigma, or R for a body particle
    bool body;
};

template <bool COROT>
__device__ __forceinline__ void side_from_fields(const SceneDesc &S, unsigned j, float3 pos, float mass,
                                                 SolidSide &J) {
    J.pos = pos;
    J.pos0 = ld3(S.originalpos, j);
    J.vel = ld3(S.velocity, j);
    J.inv_rho0 = __frcp_rn(S.density0[j]);
    J.mrho = __fdiv_rn(mass, S.density[j]);
    for (int c = 0; c < 6; ++c) J.s[c] = S.stress[6 * (size_t)j + c];
    J.body = S.body_number[j] > 0;
    if (COROT) {
        float R[9];
        for (int c = 0; c < 9; ++c) R[c] = S.rotation[9 * (size_t)j + c];
        corot_nmat(R, J.s, J.body, J.N);
    }
}

// The same values from the sorted copies: k_gather put 1/density0 in the
// velocity copy's w, k_stresses_sorted put mass/density in the second
// stress float4's z and N with mass/density in srot.  `need_s`: load the
// stress too (the corotational partner side does without it).
template <bool COROT>
__device__ __forceinline__ void side_from_sorted(const SceneDesc &S, unsigned kk, bool need_s, SolidSide &J) {
    const float4 p = S.spos[kk], p0 = S.spos0[kk], v = S.svel[kk];
    J.pos = xyz(p);
    J.pos0 = xyz(p0);
    J.vel = xyz(v);
    J.inv_rho0 = v.w;
    J.body = __float_as_uint(p0.w) > 0;
    if (!COROT || need_s) {
        const float4 s0 = S.sstress[2 * (size_t)kk], s1 = S.sstress[2 * (size_t)kk + 1];
        J.s[0] = s0.x; J.s[1] = s0.y; J.s[2] = s0.z; J.s[3] = s0.w; J.s[4] = s1.x; J.s[5] = s1.y;
        J.mrho = s1.z;
    }
    if (COROT)
        for (int c = 0; c < 3; ++c) {
            const float4 r = S.srot[3 * (size_t)kk + c];
            J.N[3 * c] = r.x;
            J.N[3 * c + 1] = r.y;
            J.N[3 * c + 2] = r.z;
            if (c == 0) J.mrho = r.w;
        }
}

__device__ __forceinline__ float3 mat3_vec(const float m[9], float3 v) { return mat_vec(m, v); }

// Particle i's side of the pair term: its stress, R sigma and (corotational
// body particles pair with) its stress again.
struct SolidI {
    SolidSide side;
    float M[9];  // R_i sigma_i (corotational)
};

// The direct pair term of compute_forces_solids (solid_corotation.cl:
// 215-403, solid_svk.cl:182-367) without symmetry images, gathered per
// partner type:
//   f_ji = -v sigma_i gW,  f_ij = -f_ji for a body partner, else v sigma_j gW
//   (v = m^2 / (rho0_i rho0_j), gW = spiky gradient at x0_i - x0_j);
//   corotational fe = R_j f_ij - R_i f_ji = v (M_i + M_j) gW, or
//   v (R_j sigma_i gW + M_i gW) for a body partner (M = R sigma);
//   SVK fe = f_ij - f_ji = v (sigma_i + sigma_j) gW, or 2 v sigma_i gW.
// The volume factor comes from per-particle reciprocals and the Laplacian's
// distance from rsqrt, so a pair costs no division or square root.
// IN_RANGE: the caller walks the first pass's masks, whose candidates
// passed this range test with the same positions and arithmetic.
template <bool COROT, bool IN_RANGE = false>
__device__ __forceinline__ void solid_pair(const SolidConsts &C, const SolidI &II, const SolidSide &J,
                                           Kahan3 &fe_s, Kahan3 &fv_s) {
    const SolidSide &I = II.side;
    const float3 x = sub3(I.pos0, J.pos0);
    const float r2 = norm2(sub3(J.pos, I.pos));
    if (!IN_RANGE && !(norm2(x) <= C.le || r2 <= C.le)) return;
    const float vivj = __fmul_rn(__fmul_rn(__fmul_rn(C.mass, C.mass), I.inv_rho0), J.inv_rho0);
    const float3 gx = spiky_grad(x, C.h, C.kv, C.le);
    float3 fe;
    if (COROT) {
        const float3 mi = mat3_vec(II.M, gx);
        fe = J.body ? (mat3_vec(J.N, sym_vec(I.s, gx)) + mi) * vivj : (mat3_vec(J.N, gx) + mi) * vivj;
    } else {
        const float3 si = sym_vec(I.s, gx);
        fe = J.body ? si * (2.f * vivj) : (sym_vec(J.s, gx) + si) * vivj;
    }
    const float dist = r2 > 0.f ? __fmul_rn(r2, rsqrtf(r2)) : 0.f;
    const float lap = r2 <= C.le ? C.kv * (C.h - dist) : 0.f;
    const float3 fv = (J.vel - I.vel) * (J.mrho * lap);
    fe_s.add(fe);
    fv_s.add(fv);
}

// compute_forces_solids for plane-free scenes.  MASKED (a fused substep):
// walks the masks of the substep's first pair pass, reading the sorted
// copies; otherwise (a named call) scans every candidate, reading the
// fields.  Without images the cut-off force equals the force.
// At most 80 registers (a few bytes spill to L1): six 128-thread blocks per
// SM instead of five keep more gathers in flight in this latency-bound pass
// (corotational 0.415 -> 0.383 ms, SVK 0.379 -> 0.344 ms on batched-256).
template <bool COROT, bool MASKED>
__global__ void __maxnreg__(80) k_forces_solids(const SceneDesc *__restrict__ scenes, BlockMap map, int fuse_step) {
    SPH_FOR_WORK(map)
    if (S.num_symmetry_planes || (MASKED && !S.sstress)) continue;
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const SolidConsts C = solid_consts(S);
        SolidI I;
        if (MASKED) side_from_sorted<COROT>(S, k, true, I.side);
        else side_from_fields<COROT>(S, i, xyz(S.spos[k]), C.mass, I.side);
        if (COROT) {
            float R[9];
            for (int c = 0; c < 9; ++c) R[c] = S.rotation[9 * (size_t)i + c];
            corot_nmat(R, I.side.s, false, I.M);
        }
        Kahan3 fe_s, fv_s;
        auto visit = [&](unsigned kk) {
            if (kk == k) return;
            SolidSide J;
            if (MASKED) side_from_sorted<COROT>(S, kk, false, J);
            else side_from_fields<COROT>(S, min(S.cellparticles[kk], S.pnum - 1), xyz(S.spos[kk]), C.mass, J);
            solid_pair<COROT>(C, I, J, fe_s, fv_s);
        };
        // the masks hold neither k itself nor a candidate out of range
        auto visit_masked = [&](unsigned kk) {
            SolidSide J;
            side_from_sorted<COROT>(S, kk, false, J);
            solid_pair<COROT, true>(C, I, J, fe_s, fv_s);
        };
        if (MASKED && S.ncand[k] != SPH_NCAND_SCAN)
            for_each_masked(S, k, StencilRows(S, S.gridcell[i]), visit_masked);
        else
            for_each_neighbour(S, S.gridcell[i], visit);
        const float visc = *S.viscosity;
        const float3 fe = fe_s.get() * 0.5f, fv = fv_s.get() * visc;
        st3(S.force, i, fe + fv);
        st3(S.force_elastic, i, fe);
        st3(S.force_viscous, i, fv);
        st3(S.cutoff_force, i, fe_s.get() * 0.5f + fv_s.get() * visc);
        // step_forward for this particle, from the sorted copies of its
        // position and velocity, which nothing has changed since the gather
        if (MASKED && fuse_step) integrate(S, i, fe + fv, I.side.vel, I.side.pos);
    }
    SPH_END_WORK
}

// ---- kinematic bodies (kernels/rigidbody.cl) --------------------------------

// set_body_position (rigidbody.cl:1-33): translate the body's particles to
// the new pose and give them velocity (new - old) / dt.  Every particle
// reads the old pose; k_store_body_vec records the new one afterwards.
__global__ void k_set_body_position(const SceneDesc *__restrict__ scenes, BlockMap map, unsigned body, float3 np) {
    SPH_FOR_WORK(map)
    if (item < active_count(S) && body < *S.body_count && body < S.body_capacity && S.body_number[item] == body + 1) {
        const float3 old = ld3(S.body_position, body);
        const float dt = *S.timestep;
        st3(S.position, item, ld3(S.position, item) - old + np);
        const float3 dv = np - old;
        st3(S.velocity, item, make_float3(dv.x / dt, dv.y / dt, dv.z / dt));
    }
    SPH_END_WORK
}

// get_matrix_from_euler, XYX (rigidbody.cl:35-68)
__device__ void euler_xyx(float3 e, float out[9]) {
    float cx = cosf(e.x), sx = sinf(e.x), cy = cosf(e.y), sy = sinf(e.y), cx2 = cosf(e.z), sx2 = sinf(e.z);
    const float rx[9] = {1, 0, 0, 0, cx, -sx, 0, sx, cx};
    const float ry[9] = {cy, 0, -sy, 0, 1, 0, sy, 0, cy};
    const float rx2[9] = {1, 0, 0, 0, cx2, -sx2, 0, sx2, cx2};
    float ryx[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) ryx[3 * r + c] = ry[3 * r] * rx[c] + ry[3 * r + 1] * rx[3 + c] + ry[3 * r + 2] * rx[6 + c];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[3 * r + c] = rx2[3 * r] * ryx[c] + rx2[3 * r + 1] * ryx[3 + c] + rx2[3 * r + 2] * ryx[6 + c];
}

// set_body_rotation (rigidbody.cl:70-120).  As in the source, the matrix
// applied is built from the body's stored Euler angles and the particle's
// rotation field; the new angles are only recorded (by k_store_body_vec).
__global__ void k_set_body_rotation(const SceneDesc *__restrict__ scenes, BlockMap map, unsigned body) {
    SPH_FOR_WORK(map)
    if (item < active_count(S) && body < *S.body_count && body < S.body_capacity && S.body_number[item] == body + 1) {
        float b[9];
        euler_xyx(ld3(S.body_euler_rotation, body), b);
        float *pr = S.rotation + 9 * (size_t)item;
        float prot[9], t2[9], t3[9];
        for (int c = 0; c < 9; ++c) prot[c] = pr[c];
        // t2 = b^T prot
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) t2[3 * r + c] = b[r] * prot[c] + b[3 + r] * prot[3 + c] + b[6 + r] * prot[6 + c];
        const float3 rpos = mat_vec(t2, ld3(S.position, item));
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) t3[3 * r + c] = t2[3 * r] * prot[c] + t2[3 * r + 1] * prot[3 + c] + t2[3 * r + 2] * prot[6 + c];
        for (int c = 0; c < 9; ++c) pr[c] = t3[c];
        st3(S.position, item, rpos);
    }
    SPH_END_WORK
}

// Records the body's new pose (which == 0) or Euler angles (which == 1)
// after the particle update, as particle 0 does in the source.
__global__ void k_store_body_vec(const SceneDesc *__restrict__ scenes, int which, unsigned body, float3 v) {
    const SceneDesc &S = scenes[0];
    if (threadIdx.x == 0 && blockIdx.x == 0 && body < *S.body_count && body < S.body_capacity)
        st3(which == 0 ? S.body_position : S.body_euler_rotation, body, v);
}

// ---- scene init (common.cl:533-604) ------------------------------------------

// populate_position_cuboid: a size.x x size.y x size.z lattice spanning
// corner1..corner2; sets n as the reference does.  Each coordinate is
// (i / (size - 1)) (c2 - c1) + c1 with every operation rounded on its own
// (no contraction), so positions equal the reference's bit for bit.
__device__ __forceinline__ float cuboid_coord(unsigned i, unsigned size, float c1, float c2) {
    return __fadd_rn(__fmul_rn(__fdiv_rn((float)i, (float)(size - 1)), __fsub_rn(c2, c1)), c1);
}
__global__ void k_populate_cuboid(const SceneDesc *__restrict__ scenes, float3 c1, float3 c2, uint3 size) {
    const SceneDesc &S = scenes[0];
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned j = blockIdx.y * blockDim.y + threadIdx.y;
    const unsigned k = blockIdx.z * blockDim.z + threadIdx.z;
    if (i >= size.x || j >= size.y || k >= size.z) return;
    const unsigned p = i + size.x * j + size.x * size.y * k;
    if (p >= S.pnum) return;
    unsigned *n = const_cast<unsigned *>(S.n);
    if (p == S.pnum - 1) *n = S.pnum;
    else if (i == size.x - 1 && j == size.y - 1 && k == size.z - 1) *n = size.x * size.y * size.z;
    st3(S.position, p, make_float3(cuboid_coord(i, size.x, c1.x, c2.x), cuboid_coord(j, size.y, c1.y, c2.y),
                                   cuboid_coord(k, size.z, c1.z, c2.z)));
}

// rotate_particles: positions rotated by Rx(ax) (Ry(ay) Rz(az)) with the
// source's sign conventions.  The matrix products and the matrix-vector
// product are rounded term by term in the source's order (no contraction);
// only cosf/sinf may differ from the host libm's in the last bit.
__device__ __forceinline__ void mat_mul_rn(const float a[9], const float b[9], float out[9]) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            out[3 * r + c] = __fadd_rn(__fadd_rn(__fmul_rn(a[3 * r], b[c]), __fmul_rn(a[3 * r + 1], b[3 + c])),
                                       __fmul_rn(a[3 * r + 2], b[6 + c]));
}
__global__ void k_rotate_particles(const SceneDesc *__restrict__ scenes, BlockMap map, float ax, float ay, float az) {
    SPH_FOR_WORK(map)
    if (item < active_count(S)) {
        float cx = cosf(ax), sx = sinf(ax), cy = cosf(ay), sy = sinf(ay), cz = cosf(az), sz = sinf(az);
        const float rx[9] = {1, 0, 0, 0, cx, -sx, 0, sx, cx};
        const float ry[9] = {cy, 0, -sy, 0, 1, 0, sy, 0, cy};
        const float rz[9] = {cz, -sz, 0, sz, cz, 0, 0, 0, 1};
        float ryz[9], r[9];
        mat_mul_rn(ry, rz, ryz);
        mat_mul_rn(rx, ryz, r);
        const float3 p = ld3(S.position, item);
        float3 q;
        q.x = __fadd_rn(__fadd_rn(__fmul_rn(r[0], p.x), __fmul_rn(r[1], p.y)), __fmul_rn(r[2], p.z));
        q.y = __fadd_rn(__fadd_rn(__fmul_rn(r[3], p.x), __fmul_rn(r[4], p.y)), __fmul_rn(r[5], p.z));
        q.z = __fadd_rn(__fadd_rn(__fmul_rn(r[6], p.x), __fmul_rn(r[7], p.y)), __fmul_rn(r[8], p.z));
        st3(S.position, item, q);
    }
    SPH_END_WORK
}
