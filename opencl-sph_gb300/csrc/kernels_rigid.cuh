// kernels_rigid.cuh -- rigid bodies (an extension; the reference's bodies
// are only fixed or kinematic, kernels/rigidbody.cl).
//
// A body b whose body_dynamic[b-1] is SPH_BODY_RIGID moves rigidly: every
// substep, after the material's force pass, its particles' forces are
// summed into the body's total force and torque (FP64), the body's centre,
// linear velocity, orientation and angular momentum are advanced with the
// same semi-implicit Euler step the particles use (v += dt a, x += dt v;
// L += dt tau, q += dt/2 (0, w) q), and the particles are placed back on
// the body: x_i = c + R r_i, v_i = v + w x (R r_i), with r_i the particle's
// offset from the centre when the body was set up.
//
// The body is set up (centre, mean velocity, inertia tensor, angular
// momentum, particle offsets) from its particles' current state on its
// first substep, and again after the host rewrites positions, velocities
// or body tables.
//
// Sums are deterministic: each of SPH_RIGID_BLOCKS blocks sums a fixed
// stride of the body's particle range (per thread in index order, then the
// lanes' sums in lane order and the warps' in warp order), and the
// per-block partials are added in block order.  A body's result is therefore the same alone and in any
// batch.
//
// FP64 arithmetic runs at a small fraction of the FP32 rate on this part
// (each warp instruction occupies the unit for many cycles whatever the
// number of active lanes), so the kernels spend as few FP64 warp
// instructions as they can: no shuffle trees (a column sum per value, one
// lane per value, through shared memory), one warp per body for the body's
// step.
#pragma once

#include "kernels_common.cuh"

// rigid_state layout (doubles, per body)
enum RigidSlot {
    RS_FLAG = 0,  // 0: to set up, 1: set up this substep (offsets written by the scatter), 2: running
    RS_N = 1,     // particle count
    RS_LO = 2,    // lowest and highest particle index of the body
    RS_HI = 3,
    RS_C = 4,     // centre (3)
    RS_V = 7,     // linear velocity (3)
    RS_Q = 10,    // orientation quaternion (w, x, y, z)
    RS_L = 14,    // angular momentum (3)
    RS_IINV0 = 17,  // inverse inertia tensor in the body frame (3x3, row-major)
    RS_W = 26,    // angular velocity (3)
    RS_A = 29,    // linear acceleration of the last substep (3)
    RS_R = 32,    // rotation matrix of q (3x3, row-major)
    RS_C0 = 41,   // centre at set-up (3): the offsets are taken from it
};

// Reduced quantities (per block, then per body).
enum RigidQ {
    RQ_N = 0,
    RQ_X = 1,    // sum x (3)
    RQ_V = 4,    // sum v (3)
    RQ_XX = 7,   // sum x x^T: xx, yy, zz, xy, xz, yz
    RQ_XV = 13,  // sum x cross v (3)
    RQ_F = 16,   // sum f (3)
    RQ_XF = 19,  // sum x cross f (3)
    RQ_SUMS = 22,
    RQ_MIN = 22,  // lowest particle index
    RQ_MAX = 23,  // highest particle index
};
static_assert(SPH_RIGID_Q == 24, "rigid reduction layout");

__device__ __forceinline__ bool rigid_particle_of(const SceneDesc &S, unsigned i, unsigned body) {
    return S.body_number[i] == body;
}

// Particles of rigid bodies are moved by k_rigid_scatter, not by step_forward.
__device__ __forceinline__ bool body_skips_step(const SceneDesc &S, unsigned i) {
    if (!S.body_number) return false;
    const unsigned b = S.body_number[i];
    if (b == 0 || b > S.body_capacity) return false;  // beyond body_dynamic: treated as dynamic
    const unsigned dyn = S.body_dynamic[b - 1];
    return dyn == 0u || dyn == SPH_BODY_RIGID;
}

// grid (SPH_RIGID_BLOCKS, rigid bodies), SPH_RIGID_THREADS threads: thread
// t of block b sums particles lo + T b + t, lo + T (b + B) + t, ... in index
// order (T threads, B blocks); lane q of each warp then adds value q of its
// warp's 32 lanes in lane order, and lane q of warp 0 the warps' sums in
// warp order.
__global__ void __launch_bounds__(SPH_RIGID_THREADS)
    k_rigid_reduce(const SceneDesc *__restrict__ scenes, const RigidWork *__restrict__ work) {
    constexpr int W = SPH_RIGID_THREADS / 32;
    __shared__ double cols[W][RQ_SUMS][33];  // value q of lane l, per warp (padded rows)
    __shared__ double wsum[W][RQ_SUMS];
    __shared__ unsigned wmin[W], wmax1[W];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const RigidWork w = work[blockIdx.y];
    const SceneDesc &S = scenes[w.scene];
    if (scene_idle(S) || !S.rigid_state || w.body == 0 || w.body > S.body_capacity) return;
    const double *st = S.rigid_state + (size_t)(w.body - 1) * SPH_RIGID_STRIDE;
    const unsigned n = active_count(S);
    unsigned lo = 0, hi = n;
    if (st[RS_FLAG] != 0.0) {
        lo = (unsigned)st[RS_LO];
        const unsigned h1 = (unsigned)st[RS_HI] + 1u;
        hi = h1 < n ? h1 : n;
    }
    double acc[RQ_SUMS];
#pragma unroll
    for (int q = 0; q < RQ_SUMS; ++q) acc[q] = 0.0;
    unsigned mn = 0xffffffffu, mx1 = 0;  // lowest index, highest index + 1 (0: none)
    for (unsigned i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
        if (!rigid_particle_of(S, i, w.body)) continue;
        const float3 xf = ld3(S.position, i), vf = ld3(S.velocity, i), ff = ld3(S.force, i);
        const double x = xf.x, y = xf.y, z = xf.z;
        const double vx = vf.x, vy = vf.y, vz = vf.z;
        const double fx = ff.x, fy = ff.y, fz = ff.z;
        acc[RQ_N] += 1.0;
        acc[RQ_X] += x;
        acc[RQ_X + 1] += y;
        acc[RQ_X + 2] += z;
        acc[RQ_V] += vx;
        acc[RQ_V + 1] += vy;
        acc[RQ_V + 2] += vz;
        acc[RQ_XX] += x * x;
        acc[RQ_XX + 1] += y * y;
        acc[RQ_XX + 2] += z * z;
        acc[RQ_XX + 3] += x * y;
        acc[RQ_XX + 4] += x * z;
        acc[RQ_XX + 5] += y * z;
        acc[RQ_XV] += y * vz - z * vy;
        acc[RQ_XV + 1] += z * vx - x * vz;
        acc[RQ_XV + 2] += x * vy - y * vx;
        acc[RQ_F] += fx;
        acc[RQ_F + 1] += fy;
        acc[RQ_F + 2] += fz;
        acc[RQ_XF] += y * fz - z * fy;
        acc[RQ_XF + 1] += z * fx - x * fz;
        acc[RQ_XF + 2] += x * fy - y * fx;
        mn = min(mn, i);
        mx1 = max(mx1, i + 1u);
    }
#pragma unroll
    for (int q = 0; q < RQ_SUMS; ++q) cols[warp][q][lane] = acc[q];
    __syncwarp();
    if (lane < RQ_SUMS) {
        double v = cols[warp][lane][0];
        for (int l = 1; l < 32; ++l) v += cols[warp][lane][l];
        wsum[warp][lane] = v;
    }
    const unsigned rmn = __reduce_min_sync(SPH_FULL_MASK, mn);
    const unsigned rmx1 = __reduce_max_sync(SPH_FULL_MASK, mx1);
    if (lane == 0) {
        wmin[warp] = rmn;
        wmax1[warp] = rmx1;
    }
    __syncthreads();
    if (warp != 0) return;
    double *part = S.rigid_partial + ((size_t)(w.body - 1) * SPH_RIGID_BLOCKS + blockIdx.x) * SPH_RIGID_Q;
    if (lane < RQ_SUMS) {
        double v = wsum[0][lane];
        for (int u = 1; u < W; ++u) v += wsum[u][lane];
        part[lane] = v;
    }
    if (lane == 0) {
        unsigned bmn = wmin[0], bmx1 = wmax1[0];
        for (int u = 1; u < W; ++u) {
            bmn = min(bmn, wmin[u]);
            bmx1 = max(bmx1, wmax1[u]);
        }
        part[RQ_MIN] = bmn == 0xffffffffu ? 4294967296.0 : (double)bmn;
        part[RQ_MAX] = bmx1 == 0u ? -1.0 : (double)(bmx1 - 1u);
    }
}

__device__ __forceinline__ void quat_to_matrix(const double q[4], double R[9]) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    R[0] = 1 - 2 * (y * y + z * z);
    R[1] = 2 * (x * y - w * z);
    R[2] = 2 * (x * z + w * y);
    R[3] = 2 * (x * y + w * z);
    R[4] = 1 - 2 * (x * x + z * z);
    R[5] = 2 * (y * z - w * x);
    R[6] = 2 * (x * z - w * y);
    R[7] = 2 * (y * z + w * x);
    R[8] = 1 - 2 * (x * x + y * y);
}

// w = R Iinv0 R^T L
__device__ __forceinline__ void angular_velocity(const double R[9], const double Iinv0[9], const double L[3],
                                                 double w[3]) {
    double a[3], b[3];
    for (int r = 0; r < 3; ++r) a[r] = R[r] * L[0] + R[3 + r] * L[1] + R[6 + r] * L[2];  // R^T L
    for (int r = 0; r < 3; ++r) b[r] = Iinv0[3 * r] * a[0] + Iinv0[3 * r + 1] * a[1] + Iinv0[3 * r + 2] * a[2];
    for (int r = 0; r < 3; ++r) w[r] = R[3 * r] * b[0] + R[3 * r + 1] * b[1] + R[3 * r + 2] * b[2];
}

// Inverse of a symmetric 3x3 matrix; a (near-)singular one (a body of one
// particle, or of collinear particles) gets the zero matrix: no rotation.
__device__ __forceinline__ void sym_inverse(const double I[9], double out[9]) {
    const double c00 = I[4] * I[8] - I[5] * I[7], c01 = I[5] * I[6] - I[3] * I[8], c02 = I[3] * I[7] - I[4] * I[6];
    const double det = I[0] * c00 + I[1] * c01 + I[2] * c02;
    const double tr = I[0] + I[4] + I[8];
    for (int k = 0; k < 9; ++k) out[k] = 0.0;
    if (!(tr > 0.0) || !(fabs(det) > 1e-12 * tr * tr * tr)) return;
    const double inv = 1.0 / det;
    out[0] = c00 * inv;
    out[1] = (I[2] * I[7] - I[1] * I[8]) * inv;
    out[2] = (I[1] * I[5] - I[2] * I[4]) * inv;
    out[3] = c01 * inv;
    out[4] = (I[0] * I[8] - I[2] * I[6]) * inv;
    out[5] = (I[2] * I[3] - I[0] * I[5]) * inv;
    out[6] = c02 * inv;
    out[7] = (I[1] * I[6] - I[0] * I[7]) * inv;
    out[8] = (I[0] * I[4] - I[1] * I[3]) * inv;
}

// One warp per rigid body (grid: rigid bodies): lane q adds the blocks'
// partials of value q in block order (the index range's min and max in
// lanes RQ_MIN and RQ_MAX); lane 0 then sets the body up when due and takes
// its substep.
__global__ void __launch_bounds__(32)
    k_rigid_integrate(const SceneDesc *__restrict__ scenes, const RigidWork *__restrict__ work, unsigned num) {
    __shared__ double sum[SPH_RIGID_Q];
    const unsigned p = blockIdx.x, lane = threadIdx.x;
    if (p >= num) return;
    const RigidWork wk = work[p];
    const SceneDesc &S = scenes[wk.scene];
    if (scene_idle(S) || !S.rigid_state || wk.body == 0 || wk.body > S.body_capacity) return;
    double *st = S.rigid_state + (size_t)(wk.body - 1) * SPH_RIGID_STRIDE;
    const double *part = S.rigid_partial + (size_t)(wk.body - 1) * SPH_RIGID_BLOCKS * SPH_RIGID_Q;
    if (lane < SPH_RIGID_Q) {
        // the min and max as integers on the bit patterns: the partials'
        // indices are whole and >= 0, their sentinels 2^32 and -1, so
        // signed 64-bit order is numeric order (no extra FP64 work)
        double v = 0.0;
        long long mnb = __double_as_longlong(4294967296.0), mxb = __double_as_longlong(-1.0);
        for (int blk = 0; blk < SPH_RIGID_BLOCKS; ++blk) {
            const double u = part[(size_t)blk * SPH_RIGID_Q + lane];
            v += u;
            const long long ub = __double_as_longlong(u);
            mnb = min(mnb, ub);
            mxb = max(mxb, ub);
        }
        sum[lane] = lane == RQ_MIN ? __longlong_as_double(mnb) : lane == RQ_MAX ? __longlong_as_double(mxb) : v;
    }
    __syncwarp();
    if (lane != 0) return;
    const double mn = sum[RQ_MIN], mx = sum[RQ_MAX];
    if (sum[RQ_N] == 0.0) {
        st[RS_FLAG] = 0.0;  // no particles (yet): set up when some appear
        return;
    }
    const double m = (double)*S.mass, dt = (double)*S.timestep;
    if (st[RS_FLAG] == 0.0) {
        const double N = sum[RQ_N];
        double c[3], v[3];
        for (int k = 0; k < 3; ++k) {
            c[k] = sum[RQ_X + k] / N;
            v[k] = sum[RQ_V + k] / N;
        }
        // second moments about the centre
        const double cxx = sum[RQ_XX] - N * c[0] * c[0], cyy = sum[RQ_XX + 1] - N * c[1] * c[1],
                     czz = sum[RQ_XX + 2] - N * c[2] * c[2], cxy = sum[RQ_XX + 3] - N * c[0] * c[1],
                     cxz = sum[RQ_XX + 4] - N * c[0] * c[2], cyz = sum[RQ_XX + 5] - N * c[1] * c[2];
        const double I0[9] = {m * (cyy + czz), -m * cxy, -m * cxz, -m * cxy, m * (cxx + czz),
                              -m * cyz, -m * cxz, -m * cyz, m * (cxx + cyy)};
        sym_inverse(I0, st + RS_IINV0);
        // L = m sum (x - c) x (v - vbar) = m (sum x x v - N c x vbar)
        st[RS_L] = m * (sum[RQ_XV] - N * (c[1] * v[2] - c[2] * v[1]));
        st[RS_L + 1] = m * (sum[RQ_XV + 1] - N * (c[2] * v[0] - c[0] * v[2]));
        st[RS_L + 2] = m * (sum[RQ_XV + 2] - N * (c[0] * v[1] - c[1] * v[0]));
        for (int k = 0; k < 3; ++k) {
            st[RS_C + k] = c[k];
            st[RS_C0 + k] = c[k];
            st[RS_V + k] = v[k];
        }
        st[RS_Q] = 1.0;
        st[RS_Q + 1] = st[RS_Q + 2] = st[RS_Q + 3] = 0.0;
        st[RS_N] = N;
        st[RS_LO] = mn;
        st[RS_HI] = mx;
        st[RS_FLAG] = 1.0;
    } else if (st[RS_FLAG] == 1.0) {
        st[RS_FLAG] = 2.0;
    }
    // forces of this substep
    const double M = st[RS_N] * m;
    double c[3] = {st[RS_C], st[RS_C + 1], st[RS_C + 2]};
    const double F[3] = {sum[RQ_F], sum[RQ_F + 1], sum[RQ_F + 2]};
    // torque about the centre: sum x cross f - c cross F
    const double tau[3] = {sum[RQ_XF] - (c[1] * F[2] - c[2] * F[1]), sum[RQ_XF + 1] - (c[2] * F[0] - c[0] * F[2]),
                           sum[RQ_XF + 2] - (c[0] * F[1] - c[1] * F[0])};
    double v[3], L[3], q[4], R[9], w[3];
    for (int k = 0; k < 3; ++k) {
        const double a = F[k] / M + (double)S.gravity[k];
        st[RS_A + k] = a;
        v[k] = st[RS_V + k] + dt * a;
        c[k] += dt * v[k];
        L[k] = st[RS_L + k] + dt * tau[k];
    }
    for (int k = 0; k < 4; ++k) q[k] = st[RS_Q + k];
    quat_to_matrix(q, R);
    angular_velocity(R, st + RS_IINV0, L, w);
    // q += dt/2 (0, w) q, normalised
    const double h = 0.5 * dt;
    const double dq[4] = {-(w[0] * q[1] + w[1] * q[2] + w[2] * q[3]), w[0] * q[0] + w[1] * q[3] - w[2] * q[2],
                          w[1] * q[0] + w[2] * q[1] - w[0] * q[3], w[2] * q[0] + w[0] * q[2] - w[1] * q[1]};
    double nq = 0.0;
    for (int k = 0; k < 4; ++k) {
        q[k] += h * dq[k];
        nq += q[k] * q[k];
    }
    nq = 1.0 / sqrt(nq);
    for (int k = 0; k < 4; ++k) q[k] *= nq;
    quat_to_matrix(q, R);
    angular_velocity(R, st + RS_IINV0, L, w);
    for (int k = 0; k < 3; ++k) {
        st[RS_C + k] = c[k];
        st[RS_V + k] = v[k];
        st[RS_L + k] = L[k];
        st[RS_W + k] = w[k];
    }
    for (int k = 0; k < 4; ++k) st[RS_Q + k] = q[k];
    for (int k = 0; k < 9; ++k) st[RS_R + k] = R[k];
    if (S.body_position)
        for (int k = 0; k < 3; ++k) S.body_position[3 * (wk.body - 1) + k] = (float)c[k];
}

// grid (SPH_RIGID_BLOCKS, rigid bodies), SPH_RIGID_THREADS threads: puts
// the body's particles on it.
__global__ void __launch_bounds__(SPH_RIGID_THREADS)
    k_rigid_scatter(const SceneDesc *__restrict__ scenes, const RigidWork *__restrict__ work) {
    const RigidWork wk = work[blockIdx.y];
    const SceneDesc &S = scenes[wk.scene];
    if (scene_idle(S) || !S.rigid_state || wk.body == 0 || wk.body > S.body_capacity) return;
    const double *st = S.rigid_state + (size_t)(wk.body - 1) * SPH_RIGID_STRIDE;
    const double flag = st[RS_FLAG];
    if (flag == 0.0) return;
    const unsigned n = active_count(S);
    const unsigned lo = (unsigned)st[RS_LO];
    const unsigned h1 = (unsigned)st[RS_HI] + 1u;
    const unsigned hi = h1 < n ? h1 : n;
    double R[9], c[3], v[3], w[3], c0[3];
    for (int k = 0; k < 9; ++k) R[k] = st[RS_R + k];
    for (int k = 0; k < 3; ++k) {
        c[k] = st[RS_C + k];
        v[k] = st[RS_V + k];
        w[k] = st[RS_W + k];
        c0[k] = st[RS_C0 + k];
    }
    const float3 a = make_float3((float)st[RS_A], (float)st[RS_A + 1], (float)st[RS_A + 2]);
    for (unsigned i = lo + blockIdx.x * blockDim.x + threadIdx.x; i < hi; i += gridDim.x * blockDim.x) {
        if (!rigid_particle_of(S, i, wk.body)) continue;
        double r0[3];
        if (flag == 1.0) {
            // set up this substep: the offset from the set-up centre, in
            // the body frame (the orientation starts as the identity)
            const float3 x = ld3(S.position, i);
            const float4 o = make_float4((float)((double)x.x - c0[0]), (float)((double)x.y - c0[1]),
                                         (float)((double)x.z - c0[2]), 0.f);
            S.rigid_offset[i] = o;
            r0[0] = o.x;
            r0[1] = o.y;
            r0[2] = o.z;
        } else {
            const float4 o = S.rigid_offset[i];
            r0[0] = o.x;
            r0[1] = o.y;
            r0[2] = o.z;
        }
        double rr[3];
        for (int k = 0; k < 3; ++k) rr[k] = R[3 * k] * r0[0] + R[3 * k + 1] * r0[1] + R[3 * k + 2] * r0[2];
        const float3 x = make_float3((float)(c[0] + rr[0]), (float)(c[1] + rr[1]), (float)(c[2] + rr[2]));
        const float3 u = make_float3((float)(v[0] + (w[1] * rr[2] - w[2] * rr[1])),
                                     (float)(v[1] + (w[2] * rr[0] - w[0] * rr[2])),
                                     (float)(v[2] + (w[0] * rr[1] - w[1] * rr[0])));
        if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) atomicOr(S.status, (unsigned)STATUS_NONFINITE);
        st3(S.position, i, x);
        st3(S.velocity, i, u);
        st3(S.acceleration, i, a);
    }
}

// The host rewrote state the bodies were set up from: set them up again.
__global__ void k_rigid_reset(const SceneDesc *__restrict__ scenes, unsigned num_scenes) {
    for (unsigned s = blockIdx.x; s < num_scenes; s += gridDim.x) {
        const SceneDesc &S = scenes[s];
        if (!S.rigid_state) continue;
        for (unsigned b = threadIdx.x; b < S.body_capacity; b += blockDim.x)
            S.rigid_state[(size_t)b * SPH_RIGID_STRIDE + RS_FLAG] = 0.0;
    }
}
