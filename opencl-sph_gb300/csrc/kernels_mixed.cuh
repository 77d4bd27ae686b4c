// kernels_mixed.cuh -- fluid and elastic solid particles in one scene
// (extension; sm_103a).
//
// The reference runs one program per store (src/opencl/particle_system_host.c:
// 184-313), so a scene is either a fluid (kernels/fluids.cl) or a solid
// (kernels/solid_svk.cl).  A mixed scene lists both programs and carries a
// per-particle `phase` field: 0 = fluid, 1 = St. Venant-Kirchhoff solid.
//   - Density (common.cl:610-690) covers every neighbour, whatever its
//     phase; a solid particle's rest density (solids.cl:99-170) covers its
//     solid neighbours only.
//   - A solid particle's deformation gradient and elastic pair forces
//     (solid_svk.cl:82-367) cover its solid neighbours only, with the
//     store's `solid_viscosity` in place of `viscosity` when present.
//   - Every pair with at least one fluid particle takes the fluid pair term
//     of fluids.cl:1-63 -- pressure from each particle's own density
//     through the fluid's equation of state, plus viscosity -- which is
//     antisymmetric, so the momentum one particle gains the other loses.
//     A fluid particle sums it over all its neighbours; a solid particle
//     over its fluid neighbours, added to its elastic force
//     (k_forces_fluids_masked<true>, kernels_fluid.cuh).
// Rigid bodies (body_dynamic 2) are fluid-phase particles and move as
// bodies, as in a fluid scene.
#pragma once

#include "kernels_solid.cuh"

// Rest density of a mixed scene's particles: the poly6 sum over neighbours
// of the particle's own phase (j = i included), from the cell-sorted
// positions, in the stencil's order.
__global__ void k_original_density_mixed(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (!S.phase) continue;
    if (item < active_count(S)) {
        const unsigned k = item;
        const unsigned i = min(S.cellparticles[k], S.pnum - 1);
        const SolidConsts C = solid_consts(S);
        const float3 ipos = xyz(S.spos[k]);
        const unsigned ph = S.phase[i];
        Kahan rho;
        for_each_neighbour(S, S.gridcell[i], [&](unsigned kk) {
            const unsigned j = min(S.cellparticles[kk], S.pnum - 1);
            if (S.phase[j] != ph) return;
            const float r2 = norm2(sub3(xyz(S.spos[kk]), ipos));
            if (r2 <= C.le) {
                const float d = fmaxf(C.h2 - r2, 0.f);
                rho.add(d * d * d);
            }
        });
        S.density0[i] = poly6_density(rho.s, C.h2, C.h, C.mass);
    }
    SPH_END_WORK
}

// A candidate kk of a mixed scene's solid particle k is a solid partner
// when it is another particle (kk != k) of the solid phase: both read from
// the sorted rest-position copy (spos0, gathered with the phase bit), so
// the test needs no dependent load through cellparticles.
__device__ __forceinline__ bool solid_partner(float4 q4, unsigned kk, unsigned k) {
    return kk != k && (__float_as_uint(q4.w) & SPH_SOLID_PHASE_BIT) != 0u;
}

// f(kk, p4, q4) for particle k's stencil candidates in the reference's
// order, with the candidate's sorted position and rest position loaded at
// the top of each step: the row loop is unrolled by 4, so four candidates'
// loads are in flight before the first one's tests (the solid particles of
// a mixed scene are too few warps to hide the latency otherwise).
template <class F>
__device__ __forceinline__ void for_each_candidate_sorted(const SceneDesc &S, unsigned cell, F &&f) {
    const StencilRows rows(S, cell);
    const float4 *__restrict__ spos = S.spos;
    const float4 *__restrict__ spos0 = S.spos0;
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        unsigned b, e;
        rows.row(S, r, &b, &e);
#pragma unroll 4
        for (unsigned kk = b; kk < e; ++kk) f(kk, spos[kk], spos0[kk]);
    }
}

// compute_deformations (solid_svk.cl:82-175) of a mixed scene's solid
// particles over their solid neighbours: F = Apq Aqq^-1 with
// Apq = sum W(|p|) p q^T and Aqq = sum W(|p|) q q^T over j != i, |p| <= h.
// Needs the sorted copies gathered with the rest positions.  `masked` (a
// fused substep, after the density pass of the same positions): walks the
// density pass's candidate masks, which hold exactly the candidates with
// |p| <= h, in candidate order, so the sums are those of the scan (which a
// named call runs).
__global__ void k_deformations_mixed(const SceneDesc *__restrict__ scenes, BlockMap map, int masked) {
    SPH_FOR_WORK(map)
    if (!S.phase || !S.spos0) continue;
    if (item < active_count(S)) {
        const unsigned k = item;
        const float4 k0 = S.spos0[k];
        if (__float_as_uint(k0.w) & SPH_SOLID_PHASE_BIT) {
            const unsigned i = min(S.cellparticles[k], S.pnum - 1);
            const SolidConsts C = solid_consts(S);
            const float3 ipos = xyz(S.spos[k]);
            const float3 ipos0 = xyz(k0);
            float apq[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            float aqq[6] = {0, 0, 0, 0, 0, 0};
            auto visit = [&](unsigned kk, float4 p4, float4 q4) {
                if (!solid_partner(q4, kk, k)) return;
                const float3 p = sub3(xyz(p4), ipos);
                const float r2 = norm2(p);
                if (!(r2 <= C.le)) return;
                const float d = fmaxf(C.h2 - r2, 0.f);
                const float w = d * d * d;
                const float3 q = sub3(xyz(q4), ipos0);
                add_outer(p * w, q, apq);
                const float3 wq = q * w;
                aqq[0] = __fmaf_rn(wq.x, q.x, aqq[0]);
                aqq[1] = __fmaf_rn(wq.y, q.y, aqq[1]);
                aqq[2] = __fmaf_rn(wq.z, q.z, aqq[2]);
                aqq[3] = __fmaf_rn(wq.x, q.y, aqq[3]);
                aqq[4] = __fmaf_rn(wq.x, q.z, aqq[4]);
                aqq[5] = __fmaf_rn(wq.y, q.z, aqq[5]);
            };
            if (masked && S.ncand[k] != SPH_NCAND_SCAN)
                for_each_masked(S, k, StencilRows(S, S.gridcell[i]),
                                [&](unsigned kk) { visit(kk, S.spos[kk], S.spos0[kk]); });
            else
                for_each_candidate_sorted(S, S.gridcell[i], visit);
            float inv[6];
            sym_inverse(aqq, inv);
            float F[9];
            mul_as(apq, inv, F);
            for (int c = 0; c < 9; ++c) S.deformation[9 * (size_t)i + c] = F[c];
        }
    }
    SPH_END_WORK
}

// compute_forces_solids (solid_svk.cl:182-367) of a mixed scene's solid
// particles over their solid neighbours j != i with rest or current
// distance <= h: the elastic pair term from both stresses and the
// Laplacian viscosity (solid_viscosity when the store has it).  Writes
// force, force_elastic, force_viscous and cutoff_force (no symmetry
// planes: the cut-off force is the whole force); the fluid force pass then
// adds the particle's fluid pair terms and steps it.  The candidate tests
// read the sorted copies (gathered with the rest positions); the fields of
// j are read for the neighbours only.
__global__ void k_forces_solids_mixed(const SceneDesc *__restrict__ scenes, BlockMap map) {
    SPH_FOR_WORK(map)
    if (!S.phase || !S.spos0) continue;
    if (item < active_count(S)) {
        const unsigned k = item;
        const float4 k0 = S.spos0[k];
        if (__float_as_uint(k0.w) & SPH_SOLID_PHASE_BIT) {
            const unsigned i = min(S.cellparticles[k], S.pnum - 1);
            const SolidConsts C = solid_consts(S);
            const float3 ipos = xyz(S.spos[k]);
            const float3 ivel = ld3(S.velocity, i);
            const float3 ipos0 = xyz(k0);
            float si[6];
            for (int c = 0; c < 6; ++c) si[c] = S.stress[6 * (size_t)i + c];
            const float rho0i = S.density0[i];
            Kahan3 fe_s, fv_s;
            for_each_candidate_sorted(S, S.gridcell[i], [&](unsigned kk, float4 p4, float4 q4) {
                if (!solid_partner(q4, kk, k)) return;
                const float3 jpos = xyz(p4);
                const float3 x = sub3(ipos0, xyz(q4));
                const float r2 = norm2(sub3(jpos, ipos));
                if (!(norm2(x) <= C.le || r2 <= C.le)) return;
                const unsigned j = min(S.cellparticles[kk], S.pnum - 1);
                const float3 jvel = ld3(S.velocity, j);
                const float vivj = C.mass * C.mass / rho0i / S.density0[j];
                const float mrj = C.mass / S.density[j];
                float sj[6];
                for (int c = 0; c < 6; ++c) sj[c] = S.stress[6 * (size_t)j + c];
                const float3 gx = spiky_grad(x, C.h, C.kv, C.le);
                const float3 f_ji = sym_vec(si, gx) * (-vivj);
                const bool jbody = (__float_as_uint(q4.w) & ~SPH_SOLID_PHASE_BIT) != 0u;
                const float3 f_ij = jbody ? -f_ji : sym_vec(sj, -gx) * (-vivj);
                const float3 fe = f_ij - f_ji;
                const float lap = r2 <= C.le ? C.kv * (C.h - sqrtf(r2)) : 0.f;
                const float3 fv = (jvel - ivel) * (mrj * lap);
                fe_s.add(fe);
                fv_s.add(fv);
            });
            const float visc = S.solid_viscosity ? *S.solid_viscosity : *S.viscosity;
            const float3 fe = fe_s.get() * 0.5f, fv = fv_s.get() * visc;
            st3(S.force, i, fe + fv);
            st3(S.force_elastic, i, fe);
            st3(S.force_viscous, i, fv);
            st3(S.cutoff_force, i, fe + fv);
        }
    }
    SPH_END_WORK
}
