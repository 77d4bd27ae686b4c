/*
 * sph_oracle_impl.h -- body of the CPU oracle, included once per precision
 * by sph_oracle.c with REAL, SFX and the R_* math macros defined.
 *
 * Test infrastructure only (see sph_oracle.h).  Each function below is a
 * restatement of one OpenCL kernel of tauroid/opencl-sph; the comment above
 * it names the file:line range it follows.  Arithmetic is kept in the same
 * order and the same types as the OpenCL source, including the places where
 * a double literal promotes a float expression to double (the C promotion
 * rules match OpenCL C's there), so that the FP32 instantiation reproduces
 * what the reference computes under IEEE rounding.
 */

#define O_CAT_(a, b) a##b
#define O_CAT(a, b) O_CAT_(a, b)
#define OF(name) O_CAT(name, SFX)
#define OST O_CAT(sph_oracle_state, SFX)
#define V3 O_CAT(ov3, SFX)

/* The reference's PI is a float literal in both precisions (common.cl:15). */
#define O_PI ((REAL)3.1415926535f)

typedef struct { REAL x, y, z; } V3;

static inline V3 OF(v3)(REAL x, REAL y, REAL z) { V3 v; v.x = x; v.y = y; v.z = z; return v; }
static inline V3 OF(v3_load)(const REAL *p, size_t i) { return OF(v3)(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
static inline void OF(v3_store)(V3 v, REAL *p, size_t i) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }
static inline V3 OF(v3_add)(V3 a, V3 b) { return OF(v3)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 OF(v3_sub)(V3 a, V3 b) { return OF(v3)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 OF(v3_mul)(V3 a, REAL s) { return OF(v3)(a.x * s, a.y * s, a.z * s); }
static inline V3 OF(v3_div)(V3 a, REAL s) { return OF(v3)(a.x / s, a.y / s, a.z / s); }
static inline V3 OF(v3_neg)(V3 a) { return OF(v3)(-a.x, -a.y, -a.z); }
/* OpenCL dot/length: ((x*x + y*y) + z*z) */
static inline REAL OF(v3_dot)(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline REAL OF(v3_len)(V3 a) { return R_SQRT(a.x * a.x + a.y * a.y + a.z * a.z); }
/* v - 2*n*dot(n, v - p): the reflection used throughout the SYMMETRY blocks */
static inline V3 OF(v3_reflect)(V3 v, V3 point, V3 normal) {
    V3 twon = OF(v3_mul)(normal, (REAL)2);
    return OF(v3_sub)(v, OF(v3_mul)(twon, OF(v3_dot)(normal, OF(v3_sub)(v, point))));
}

/* ---- kernel functions, common.cl:78-90 ---------------------------------- */

static inline REAL OF(k_poly6)(REAL dist, REAL h) {
    if (dist > h) return 0;
    return (REAL)315.0f / (REAL)64.0f / O_PI / R_POW(h, (REAL)9.0f) *
           R_POW(R_POW(h, (REAL)2.0f) - R_POW(dist, (REAL)2.0f), (REAL)3.0f);
}
static inline V3 OF(k_spiky_grad)(V3 d, REAL h, int guard) {
    REAL norm = OF(v3_len)(d);
    if (guard && norm == 0) return OF(v3)(0, 0, 0);
    V3 dir = OF(v3_div)(d, norm);
    if (norm > h) return OF(v3)(0, 0, 0);
    /* direction * -45.0f/PI/pow(h,6) * pow(h - norm, 2), left-associative */
    V3 t = OF(v3_mul)(dir, (REAL)-45.0f);
    t = OF(v3_div)(t, O_PI);
    t = OF(v3_div)(t, R_POW(h, (REAL)6.0f));
    return OF(v3_mul)(t, R_POW(h - norm, (REAL)2.0f));
}
static inline REAL OF(k_visc_lap)(REAL dist, REAL h) {
    if (dist > h) return 0;
    return (REAL)45.0f / O_PI / R_POW(h, (REAL)6.0f) * (h - dist);
}

/* ---- matrix helpers, common.cl:92-350 ----------------------------------- */
/* 3x3 row-major I_rc = 3r+c; symmetric S = [00,11,22,01,02,12] */
#ifndef SPH_ORACLE_INDEX_ENUMS_
#define SPH_ORACLE_INDEX_ENUMS_
enum { I00 = 0, I01, I02, I10, I11, I12, I20, I21, I22 };
enum { S00 = 0, S11 = 1, S22 = 2, S01 = 3, S02 = 4, S12 = 5 };
#endif
#define S10 S01
#define S20 S02
#define S21 S12

/* givens index tables, common.cl:95-99 */
static const unsigned OF(g_xx)[3] = {0, 0, 1};
static const unsigned OF(g_yy)[3] = {1, 2, 2};
static const unsigned OF(g_ee)[3] = {2, 1, 0};
static const unsigned OF(g_ex)[3] = {4, 3, 3};
static const unsigned OF(g_ey)[3] = {5, 5, 4};

/* givensRotateToZero, common.cl:101-155 */
static void OF(givens)(const REAL in[6], const REAL pin[9], unsigned offdiag, REAL o[6], REAL pout[9],
                       int guard) {
    unsigned ix = offdiag - 3;
    unsigned xx = OF(g_xx)[ix], yy = OF(g_yy)[ix], ee = OF(g_ee)[ix], xy = offdiag;
    unsigned ex = OF(g_ex)[ix], ey = OF(g_ey)[ix];
    REAL angle;
    if (guard && in[xy] == 0) angle = 0;
    else angle = (REAL)0.5f * R_ATAN((REAL)2.0f * in[xy] / (in[xx] - in[yy]));
    REAL c = R_COS(angle), s = R_SIN(angle);
    REAL c2 = c * c, s2 = s * s, cs = c * s;
    o[xx] = in[xx] * c2 + in[yy] * s2 + (REAL)2.0f * in[xy] * cs;
    o[xy] = -in[xx] * cs + in[yy] * cs + in[xy] * (c2 - s2);
    o[yy] = in[xx] * s2 + in[yy] * c2 - (REAL)2.0f * in[xy] * cs;
    o[ee] = in[ee];
    o[ex] = in[ex] * c + in[ey] * s;
    o[ey] = -in[ex] * s + in[ey] * c;
    for (unsigned r = 0; r < 3; ++r) {
        pout[3 * r + xx] = pin[3 * r + xx] * c + pin[3 * r + yy] * s;
        pout[3 * r + yy] = -pin[3 * r + xx] * s + pin[3 * r + yy] * c;
        pout[3 * r + ee] = pin[3 * r + ee];
    }
}
/* maxAbsInArray, common.cl:156-168 (first index of the strict maximum) */
static unsigned OF(maxabs3)(const REAL *a) {
    REAL m = 0; unsigned im = 0;
    for (unsigned i = 0; i < 3; ++i) { REAL v = R_FABS(a[i]); if (v > m) { m = v; im = i; } }
    return im;
}
/* multiplyBothSides P*D*P^T, common.cl:169-186 */
static void OF(both_sides)(const REAL d[3], const REAL p[9], REAL out[6]) {
    REAL d0p00 = d[0] * p[I00], d1p01 = d[1] * p[I01], d2p02 = d[2] * p[I02];
    REAL d0p10 = d[0] * p[I10], d1p11 = d[1] * p[I11], d2p12 = d[2] * p[I12];
    REAL d0p20 = d[0] * p[I20], d1p21 = d[1] * p[I21], d2p22 = d[2] * p[I22];
    out[S00] = p[I00] * d0p00 + p[I01] * d1p01 + p[I02] * d2p02;
    out[S01] = p[I00] * d0p10 + p[I01] * d1p11 + p[I02] * d2p12;
    out[S02] = p[I00] * d0p20 + p[I01] * d1p21 + p[I02] * d2p22;
    out[S11] = p[I10] * d0p10 + p[I11] * d1p11 + p[I12] * d2p12;
    out[S12] = p[I10] * d0p20 + p[I11] * d1p21 + p[I12] * d2p22;
    out[S22] = p[I20] * d0p20 + p[I21] * d1p21 + p[I22] * d2p22;
}
/* multiplyAS A*S (S symmetric), common.cl:187-199 */
static void OF(mul_as)(const REAL a[9], const REAL s[6], REAL out[9]) {
    for (unsigned r = 0; r < 3; ++r) {
        const REAL *ar = a + 3 * r;
        out[3 * r + 0] = ar[0] * s[S00] + ar[1] * s[S10] + ar[2] * s[S20];
        out[3 * r + 1] = ar[0] * s[S01] + ar[1] * s[S11] + ar[2] * s[S21];
        out[3 * r + 2] = ar[0] * s[S02] + ar[1] * s[S12] + ar[2] * s[S22];
    }
}
/* multiplyMatrices A*B, common.cl:208-220 */
static void OF(mul_mm)(const REAL a[9], const REAL b[9], REAL out[9]) {
    for (unsigned r = 0; r < 3; ++r)
        for (unsigned c = 0; c < 3; ++c)
            out[3 * r + c] = a[3 * r] * b[c] + a[3 * r + 1] * b[3 + c] + a[3 * r + 2] * b[6 + c];
}
/* multiplyMatrixVector, common.cl:221-229 */
static inline V3 OF(mul_mv)(const REAL m[9], V3 v) {
    return OF(v3)(m[I00] * v.x + m[I01] * v.y + m[I02] * v.z,
                  m[I10] * v.x + m[I11] * v.y + m[I12] * v.z,
                  m[I20] * v.x + m[I21] * v.y + m[I22] * v.z);
}
/* multiplySymMatrixVector, common.cl:230-238 */
static inline V3 OF(mul_sv)(const REAL s[6], V3 v) {
    return OF(v3)(s[S00] * v.x + s[S01] * v.y + s[S02] * v.z,
                  s[S10] * v.x + s[S11] * v.y + s[S12] * v.z,
                  s[S20] * v.x + s[S21] * v.y + s[S22] * v.z);
}
/* addOuterProduct out += a b^T, common.cl:252-256 */
static inline void OF(add_outer)(V3 a, V3 b, REAL out[9]) {
    out[I00] += a.x * b.x; out[I01] += a.x * b.y; out[I02] += a.x * b.z;
    out[I10] += a.y * b.x; out[I11] += a.y * b.y; out[I12] += a.y * b.z;
    out[I20] += a.z * b.x; out[I21] += a.z * b.y; out[I22] += a.z * b.z;
}
/* transpose, common.cl:337-350 */
static void OF(transpose)(const REAL m[9], REAL t[9]) {
    for (unsigned r = 0; r < 3; ++r)
        for (unsigned c = 0; c < 3; ++c) t[3 * c + r] = m[3 * r + c];
}
/* determinant, common.cl:332-336 */
static REAL OF(det)(const REAL m[9]) {
    return m[I00] * (m[I11] * m[I22] - m[I12] * m[I21]) - m[I01] * (m[I10] * m[I22] - m[I12] * m[I20]) +
           m[I02] * (m[I10] * m[I21] - m[I11] * m[I20]);
}
/* jacobi with threshold 0, common.cl:257-295: `iterations` Givens rotations,
 * each zeroing the largest remaining off-diagonal. */
static void OF(jacobi)(const REAL in[6], unsigned iterations, REAL eig[3], REAL p[9], int guard) {
    REAL p2[9], t[6], t2[6];
    for (unsigned k = 0; k < 9; ++k) p[k] = (k % 4 == 0) ? (REAL)1 : (REAL)0;
    for (unsigned k = 0; k < 9; ++k) p2[k] = p[k];
    for (unsigned k = 0; k < 6; ++k) t[k] = in[k];
    unsigned imax = OF(maxabs3)(t + 3) + 3;
    for (unsigned it = 0; it < iterations; it += 2) {
        OF(givens)(t, p, imax, t2, p2, guard);
        imax = OF(maxabs3)(t2 + 3) + 3;
        OF(givens)(t2, p2, imax, t, p, guard);
        imax = OF(maxabs3)(t + 3) + 3;
    }
    for (unsigned k = 0; k < 3; ++k) eig[k] = t[k];
}
/* jacobiInvert, common.cl:296-305 (1.0/x is a double division there) */
void OF(oracle_jacobi_invert)(const REAL *m, REAL *out, int guard) {
    REAL eig[3], vec[9];
    OF(jacobi)(m, 8, eig, vec, guard);
    for (unsigned k = 0; k < 3; ++k) eig[k] = (REAL)(1.0 / (double)eig[k]);
    OF(both_sides)(eig, vec, out);
}
/* getR = Apq (Apq^T Apq)^(-1/2), common.cl:306-331 */
void OF(oracle_get_r)(const REAL *apq, REAL *r, int guard) {
    REAL s[6];
    s[0] = apq[I00] * apq[I00] + apq[I10] * apq[I10] + apq[I20] * apq[I20];
    s[1] = apq[I01] * apq[I01] + apq[I11] * apq[I11] + apq[I21] * apq[I21];
    s[2] = apq[I02] * apq[I02] + apq[I12] * apq[I12] + apq[I22] * apq[I22];
    s[3] = apq[I00] * apq[I01] + apq[I10] * apq[I11] + apq[I20] * apq[I21];
    s[4] = apq[I00] * apq[I02] + apq[I10] * apq[I12] + apq[I20] * apq[I22];
    s[5] = apq[I01] * apq[I02] + apq[I11] * apq[I12] + apq[I21] * apq[I22];
    REAL eig[3], vec[9], tmp[6];
    OF(jacobi)(s, 8, eig, vec, guard);
    for (unsigned k = 0; k < 3; ++k) eig[k] = (REAL)1 / R_SQRT(eig[k]);
    OF(both_sides)(eig, vec, tmp);
    OF(mul_as)(apq, tmp, r);
}

/* ---- neighbour grid ----------------------------------------------------- */

/* Saturating float->uint (the GPU conversion rule; see sph_oracle.h). */
static inline unsigned OF(sat_uint)(REAL v) {
    if (!(v > 0)) return 0u;
    if (v >= (REAL)4294967296.0) return 0xFFFFFFFFu;
    return (unsigned)v;
}
/* find_particle_bins, common.cl:372-391 */
void OF(oracle_find_particle_bins)(OST *s) {
    const REAL *gb = s->gridbounds;
    const unsigned *R = s->gridres;
    long n = s->n;
#pragma omp parallel for schedule(static) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long i = 0; i < n; ++i) {
        const REAL *p = s->position + 3 * i;
        unsigned c[3];
        for (int a = 0; a < 3; ++a) {
            REAL q = (p[a] - gb[2 * a]) / (gb[2 * a + 1] - gb[2 * a]) * (REAL)R[a];
            unsigned u = OF(sat_uint)(q);
            c[a] = u > R[a] - 1 ? R[a] - 1 : u;
        }
        s->gridcell[i] = c[2] * R[0] * R[1] + c[1] * R[0] + c[0];
    }
}
/* zero_gridcount + count_particles_in_bins + prefix_sum +
 * copy_celloffset_to_backup + insert_particles_in_bin_array,
 * common.cl:392-529, restated as a serial stable counting sort. */
void OF(oracle_sort_particles)(OST *s) {
    size_t C = (size_t)s->gridres[0] * s->gridres[1] * s->gridres[2];
    memset(s->gridcount, 0, C * sizeof(unsigned));
    for (size_t i = 0; i < s->n; ++i) s->gridcount[s->gridcell[i]]++;
    unsigned run = 0;
    for (size_t c = 0; c < C; ++c) { s->celloffset[c] = run; run += s->gridcount[c]; }
    unsigned *cursor = (unsigned *)malloc((C ? C : 1) * sizeof(unsigned));
    memcpy(cursor, s->celloffset, C * sizeof(unsigned));
    for (size_t i = 0; i < s->n; ++i) s->cellparticles[cursor[s->gridcell[i]]++] = (unsigned)i;
    free(cursor);
}
/* compute_particle_bins_device_opencl, particle_system_host.c:448-454 */
void OF(oracle_compute_particle_bins)(OST *s) {
    OF(oracle_find_particle_bins)(s);
    OF(oracle_sort_particles)(s);
}

/* get_cell_at_offset, common.cl:354-371 */
static inline long OF(cell_at)(const unsigned *R, unsigned orig, int x, int y, int z) {
    unsigned row = R[0], layer = R[0] * R[1];
    unsigned zo = orig / layer;
    unsigned yo = (orig - layer * zo) / row;
    unsigned xo = orig - layer * zo - row * yo;
    long zn = (long)zo + z, yn = (long)yo + y, xn = (long)xo + x;
    if (xn >= (long)R[0] || xn < 0 || yn >= (long)R[1] || yn < 0 || zn >= (long)R[2] || zn < 0) return -1;
    return zn * layer + yn * row + xn;
}

/* FOR_PARTICLES_IN_RANGE, common.cl:49-68: 27 cells in z,y,x order, each
 * cell's particles in cellparticles order. */
#define O_FOR_NEIGHBOURS(s, i, j, ...)                                                  \
    for (int gz_ = -1; gz_ <= 1; ++gz_)                                                  \
        for (int gy_ = -1; gy_ <= 1; ++gy_)                                              \
            for (int gx_ = -1; gx_ <= 1; ++gx_) {                                        \
                long cell_ = OF(cell_at)((s)->gridres, (s)->gridcell[i], gx_, gy_, gz_); \
                if (cell_ < 0) continue;                                                 \
                unsigned off_ = (s)->celloffset[cell_];                                  \
                unsigned end_ = off_ + (s)->gridcount[cell_];                            \
                for (unsigned jp_ = off_; jp_ < end_; ++jp_) {                           \
                    unsigned j = (s)->cellparticles[jp_];                                \
                    __VA_ARGS__                                                          \
                }                                                                        \
            }

#define O_PLANE_POINT(pl, k) OF(v3)((pl)[6 * (k)], (pl)[6 * (k) + 1], (pl)[6 * (k) + 2])
#define O_PLANE_NORMAL(pl, k) OF(v3)((pl)[6 * (k) + 3], (pl)[6 * (k) + 4], (pl)[6 * (k) + 5])

/* The SYMMETRY region test shared by every mirrored pass (e.g.
 * common.cl:666-670): skip when i or j is farther than h from the plane,
 * or j lies on it.  1.0e-5 is a double literal. */
static inline int OF(plane_skip)(V3 ipos, V3 jpos, V3 point, V3 normal, REAL h) {
    REAL jd = R_FABS(OF(v3_dot)(normal, OF(v3_sub)(jpos, point)));
    return R_FABS(OF(v3_dot)(normal, OF(v3_sub)(ipos, point))) > h || jd > h || (double)jd < 1.0e-5;
}

/* ---- density ------------------------------------------------------------ */

/* compute_density, common.cl:610-690; with_count selects the
 * compute_original_density variant (solids.cl:99-170) when 0. */
static void OF(density_pass)(OST *s, REAL *out, int with_count) {
    const REAL h = s->smoothingradius;
    const unsigned nsp = s->num_symmetry_planes;
    const REAL *sp = s->symmetry_planes;
    long n = s->n;
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long ii = 0; ii < n; ++ii) {
        unsigned i = (unsigned)ii;
        V3 ipos = OF(v3_load)(s->position, i);
        out[i] = 0;
        if (with_count) s->num_neighbours[i] = 0;
        O_FOR_NEIGHBOURS(s, i, j, {
            /* a mixed scene's rest density: neighbours of i's own phase */
            if (!with_count && s->phase && s->phase[j] != s->phase[i]) continue;
            V3 jpos = OF(v3_load)(s->position, j);
            V3 diff = OF(v3_sub)(jpos, ipos);
            REAL dist = OF(v3_len)(diff);
            out[i] += OF(k_poly6)(dist, h);
            if (with_count && dist < h) ++s->num_neighbours[i];
            for (unsigned bits = 1; bits < (1u << nsp); ++bits) {
                V3 refpos = jpos;
                int skip = 0;
                for (unsigned k = 0; k < nsp; ++k) {
                    if ((bits & (1u << k)) == 0) continue;
                    V3 point = O_PLANE_POINT(sp, k), normal = O_PLANE_NORMAL(sp, k);
                    if (OF(plane_skip)(ipos, jpos, point, normal, h)) { skip = 1; break; }
                    refpos = OF(v3_reflect)(refpos, point, normal);
                }
                if (skip) continue;
                dist = OF(v3_len)(OF(v3_sub)(refpos, ipos));
                if (dist < h) {
                    out[i] += OF(k_poly6)(dist, h);
                    if (with_count) ++s->num_neighbours[i];
                }
            }
        })
        out[i] *= s->mass;
    }
}
void OF(oracle_compute_density)(OST *s) { OF(density_pass)(s, s->density, 1); }
/* compute_original_density, solids.cl:99-170 */
void OF(oracle_compute_original_density)(OST *s) { OF(density_pass)(s, s->density0, 0); }
/* init_original_position, solids.cl:84-95 */
void OF(oracle_init_original_position)(OST *s) {
    memcpy(s->originalpos, s->position, (size_t)s->n * 3 * sizeof(REAL));
}

/* ---- WCSPH forces, fluids.cl:1-63 --------------------------------------- */

/* APPLY_CUBE_BOUNDS(ipos, f, -2.0, 2.0), common.cl:37-43: the bounds are
 * double literals, so every test and update is evaluated in double. */
static inline REAL OF(cube_bound)(REAL p, REAL f) {
    const double mn = -2.0, mx = 2.0;
    if ((double)p < mn + (double)0.2f) return (REAL)((double)f + (1.0 / (-(mn) + (double)p) - 5.0));
    if ((double)p > mx - (double)0.2f) return (REAL)((double)f - (1.0 / (mx - (double)p) - 5.0));
    return f;
}
void OF(oracle_compute_forces_fluids)(OST *s) {
    const REAL h = s->smoothingradius;
    long n = s->n;
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long ii = 0; ii < n; ++ii) {
        unsigned i = (unsigned)ii;
        V3 ipos = OF(v3_load)(s->position, i), ivel = OF(v3_load)(s->velocity, i);
        V3 fi = OF(v3)(0, 0, 0);
        /* a mixed scene's solid particle: fluid neighbours only, added to
         * the elastic force compute_forces_solids left in force */
        const int solid_i = s->phase && s->phase[i];
        O_FOR_NEIGHBOURS(s, i, j, {
            if (j == i) continue;
            if (solid_i && s->phase[j]) continue;
            REAL p_i = (s->density[i] - s->restdens) * s->stiffness;
            REAL p_j = (s->density[j] - s->restdens) * s->stiffness;
            /* a fluid-solid pair of a mixed scene pushes, never pulls: both
             * pressures clamped at 0 (the solid's density deficit at its
             * surface would otherwise draw fluid into it) */
            if (s->phase && (s->phase[i] || s->phase[j])) {
                if (p_i < 0) p_i = 0;
                if (p_j < 0) p_j = 0;
            }
            V3 jpos = OF(v3_load)(s->position, j), jvel = OF(v3_load)(s->velocity, j);
            V3 diff = OF(v3_sub)(jpos, ipos), relvel = OF(v3_sub)(jvel, ivel);
            REAL dist = OF(v3_len)(diff);
            if (dist > h) continue;
            if ((s->guards & 2) && dist == 0) continue;
            REAL dist_in = h - dist;
            REAL didj = s->density[i] * s->density[j];
            REAL sr6 = R_POW(h, (REAL)6);
            REAL vterm = s->viscosity * dist_in * (REAL)45 / O_PI / sr6;
            /* fluids.cl:48: the 0.5 literal makes this product double */
            REAL pterm = (REAL)((double)(p_i + p_j) * 0.5 / (double)dist * (double)dist_in * (double)dist_in *
                                (double)((REAL)-45 / O_PI / sr6));
            fi = OF(v3_add)(fi, OF(v3_div)(OF(v3_add)(OF(v3_mul)(diff, pterm), OF(v3_mul)(relvel, vterm)), didj));
        })
        fi = OF(v3_mul)(fi, s->mass);
        if (solid_i) fi = OF(v3_add)(fi, OF(v3_load)(s->force, i));
        fi.x = OF(cube_bound)(ipos.x, fi.x);
        fi.y = OF(cube_bound)(ipos.y, fi.y);
        fi.z = OF(cube_bound)(ipos.z, fi.z);
        OF(v3_store)(fi, s->force, i);
    }
}

/* ---- corotational solid, solid_corotation.cl ----------------------------- */

/* contributeApq, solids.cl:66-72 */
static inline void OF(contrib_apq)(V3 p, V3 q, REAL w, REAL apq[9]) {
    V3 wp = OF(v3_mul)(p, w);
    apq[I00] += wp.x * q.x; apq[I01] += wp.x * q.y; apq[I02] += wp.x * q.z;
    apq[I10] += wp.y * q.x; apq[I11] += wp.y * q.y; apq[I12] += wp.y * q.z;
    apq[I20] += wp.z * q.x; apq[I21] += wp.z * q.y; apq[I22] += wp.z * q.z;
}
/* contributeAqq, solids.cl:74-80 */
static inline void OF(contrib_aqq)(V3 q, REAL w, REAL aqq[6]) {
    V3 wq = OF(v3_mul)(q, w);
    aqq[S00] += wq.x * q.x; aqq[S01] += wq.x * q.y; aqq[S02] += wq.x * q.z;
    aqq[S11] += wq.y * q.y; aqq[S12] += wq.y * q.z;
    aqq[S22] += wq.z * q.z;
}

/* compute_rotations_and_strains, solid_corotation.cl:28-195 */
void OF(oracle_compute_rotations_and_strains)(OST *s) {
    const REAL h = s->smoothingradius, mass = s->mass;
    const unsigned nsp = s->num_symmetry_planes;
    const REAL *sp = s->symmetry_planes;
    long n = s->n;
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long ii = 0; ii < n; ++ii) {
        unsigned i = (unsigned)ii;
        if (s->body_number[i] > 0) continue;
        V3 ipos = OF(v3_load)(s->position, i), ipos0 = OF(v3_load)(s->originalpos, i);
        REAL *apq = s->apq_temp + 9 * (size_t)i;
        for (int d = 0; d < 9; ++d) apq[d] = 0;
        /* pass 1: Apq = sum W(|p|) p q^T (+ mirrored images) */
        O_FOR_NEIGHBOURS(s, i, j, {
            V3 jpos = OF(v3_load)(s->position, j), jpos0 = OF(v3_load)(s->originalpos, j);
            V3 p = OF(v3_sub)(jpos, ipos), q = OF(v3_sub)(jpos0, ipos0);
            if (j != i) OF(contrib_apq)(p, q, OF(k_poly6)(OF(v3_len)(p), h), apq);
            for (unsigned bits = 1; bits < (1u << nsp); ++bits) {
                V3 rp = jpos, rp0 = jpos0;
                int skip = 0;
                for (unsigned k = 0; k < nsp; ++k) {
                    if ((bits & (1u << k)) == 0) continue;
                    V3 point = O_PLANE_POINT(sp, k), normal = O_PLANE_NORMAL(sp, k);
                    if (OF(plane_skip)(ipos, jpos, point, normal, h)) { skip = 1; break; }
                    rp = OF(v3_reflect)(rp, point, normal);
                    rp0 = OF(v3_reflect)(rp0, point, normal);
                }
                if (skip) continue;
                p = OF(v3_sub)(rp, ipos);
                q = OF(v3_sub)(rp0, ipos0);
                REAL dist = OF(v3_len)(p);
                if (dist < h) OF(contrib_apq)(p, q, OF(k_poly6)(dist, h), apq);
            }
        })
        REAL *r = s->rotation + 9 * (size_t)i;
        REAL *inter = s->intermediate + 9 * (size_t)i;
        for (int d = 0; d < 9; ++d) inter[d] = apq[d];
        OF(oracle_get_r)(inter, r, s->guards & 1);
        REAL rt[9], D[9];
        OF(transpose)(r, rt);
        for (int d = 0; d < 9; ++d) D[d] = 0;
        /* pass 2: D = sum (R^T p - q) m/rho0_i (x) gradW(-q) (+ mirrors) */
        O_FOR_NEIGHBOURS(s, i, j, {
            V3 jpos = OF(v3_load)(s->position, j), jpos0 = OF(v3_load)(s->originalpos, j);
            V3 p = OF(mul_mv)(rt, OF(v3_sub)(jpos, ipos));
            V3 q = OF(v3_sub)(jpos0, ipos0);
            V3 u = OF(v3_sub)(p, q);
            if (j != i)
                OF(add_outer)(OF(v3_div)(OF(v3_mul)(u, mass), s->density0[i]), OF(k_spiky_grad)(OF(v3_neg)(q), h, s->guards & 2), D);
            for (unsigned bits = 1; bits < (1u << nsp); ++bits) {
                V3 rp = jpos, rp0 = jpos0;
                int skip = 0;
                for (unsigned k = 0; k < nsp; ++k) {
                    if ((bits & (1u << k)) == 0) continue;
                    V3 point = O_PLANE_POINT(sp, k), normal = O_PLANE_NORMAL(sp, k);
                    if (OF(plane_skip)(ipos, jpos, point, normal, h)) { skip = 1; break; }
                    rp = OF(v3_reflect)(rp, point, normal);
                    rp0 = OF(v3_reflect)(rp0, point, normal);
                }
                if (skip) continue;
                p = OF(mul_mv)(rt, OF(v3_sub)(rp, ipos));
                q = OF(v3_sub)(rp0, ipos0);
                u = OF(v3_sub)(p, q);
                REAL dist = OF(v3_len)(p);
                if (dist < h)
                    OF(add_outer)(OF(v3_div)(OF(v3_mul)(u, mass), s->density0[i]), OF(k_spiky_grad)(OF(v3_neg)(q), h, s->guards & 2),
                                  D);
            }
        })
        /* computeCauchyStrain, solid_corotation.cl:1-8 */
        REAL *st = s->strain + 6 * (size_t)i;
        st[S00] = D[I00];
        st[S01] = (REAL)0.5f * (D[I01] + D[I10]);
        st[S02] = (REAL)0.5f * (D[I02] + D[I20]);
        st[S11] = D[I11];
        st[S12] = (REAL)0.5f * (D[I12] + D[I21]);
        st[S22] = D[I22];
    }
}

/* compute_stresses (isotropic Hooke), solid_corotation.cl:9-26,197-208 */
void OF(oracle_compute_stresses_corot)(OST *s) {
    const REAL E = s->youngs_modulus, nu = s->poisson;
    REAL lam = E * nu / ((REAL)1.0f + nu) / ((REAL)1 - (REAL)2.0f * nu);
    REAL mu = E / (REAL)2.0f / ((REAL)1.0f + nu);
    REAL c[36] = {0};
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) c[6 * r + k] = lam + (r == k ? (REAL)2.0f * mu : (REAL)0);
    for (int r = 3; r < 6; ++r) c[6 * r + r] = (REAL)2.0f * mu;
    /* the 6x6 diagonal block entries are lam+2mu (r==k) and lam, the lower
     * right block is 2mu on the diagonal (solid_corotation.cl:13-20) */
    long n = s->n;
#pragma omp parallel for schedule(static) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long i = 0; i < n; ++i) {
        const REAL *e = s->strain + 6 * i;
        REAL *o = s->stress + 6 * i;
        for (int r = 0; r < 6; ++r) {
            const REAL *cr = c + 6 * r;
            o[r] = cr[0] * e[0] + cr[1] * e[1] + cr[2] * e[2] + cr[3] * e[3] + cr[4] * e[4] + cr[5] * e[5];
        }
    }
}

/* compute_forces_solids, solid_corotation.cl:215-403 (corot != 0) and
 * solid_svk.cl:182-367 (corot == 0, no rotations). */
static void OF(forces_solids)(OST *s, int corot) {
    const REAL h = s->smoothingradius, mass = s->mass;
    const unsigned nsp = s->num_symmetry_planes;
    const REAL *sp = s->symmetry_planes;
    static const REAL ident[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    long n = s->n;
    /* a mixed scene's solids take their own viscosity */
    const REAL visc = s->has_solid_viscosity ? s->solid_viscosity : s->viscosity;
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long ii = 0; ii < n; ++ii) {
        unsigned i = (unsigned)ii;
        if (s->phase && !s->phase[i]) continue; /* a mixed scene's fluid particle */
        V3 ipos = OF(v3_load)(s->position, i), ivel = OF(v3_load)(s->velocity, i);
        V3 ipos0 = OF(v3_load)(s->originalpos, i);
        const REAL *ist = s->stress + 6 * (size_t)i;
        const REAL *irot = corot ? s->rotation + 9 * (size_t)i : ident;
        V3 fe_sum = OF(v3)(0, 0, 0), fv_sum = OF(v3)(0, 0, 0);
        V3 fec = OF(v3)(0, 0, 0), fvc = OF(v3)(0, 0, 0);
        O_FOR_NEIGHBOURS(s, i, j, {
            if (s->phase && !s->phase[j]) continue;
            V3 jpos0 = OF(v3_load)(s->originalpos, j);
            V3 x = OF(v3_sub)(ipos0, jpos0);
            V3 jpos = OF(v3_load)(s->position, j), jvel = OF(v3_load)(s->velocity, j);
            REAL vivj = mass * mass / s->density0[i] / s->density0[j];
            const REAL *jst = s->stress + 6 * (size_t)j;
            const REAL *jrot = corot ? s->rotation + 9 * (size_t)j : ident;
            if (j != i) {
                V3 f_ji = OF(v3_mul)(OF(mul_sv)(ist, OF(k_spiky_grad)(x, h, s->guards & 2)), -vivj);
                V3 f_ij = s->body_number[j] > 0 ? OF(v3_neg)(f_ji)
                                                 : OF(v3_mul)(OF(mul_sv)(jst, OF(k_spiky_grad)(OF(v3_neg)(x), h, s->guards & 2)), -vivj);
                V3 fe = corot ? OF(v3_add)(OF(v3_neg)(OF(mul_mv)(irot, f_ji)), OF(mul_mv)(jrot, f_ij))
                              : OF(v3_add)(OF(v3_neg)(f_ji), f_ij);
                V3 fv = OF(v3_mul)(OF(v3_mul)(OF(v3_sub)(jvel, ivel), mass / s->density[j]),
                                   OF(k_visc_lap)(OF(v3_len)(OF(v3_sub)(jpos, ipos)), h));
                fe_sum = OF(v3_add)(fe_sum, fe);
                fv_sum = OF(v3_add)(fv_sum, fv);
                fec = OF(v3_add)(fec, fe);
                fvc = OF(v3_add)(fvc, fv);
            }
            for (unsigned bits = 1; bits < (1u << nsp); ++bits) {
                V3 rp = jpos, rp0 = jpos0, rip0 = ipos0;
                V3 normal = OF(v3)(0, 0, 0);
                int skip = 0;
                for (unsigned k = 0; k < nsp; ++k) {
                    if ((bits & (1u << k)) == 0) continue;
                    V3 point = O_PLANE_POINT(sp, k);
                    normal = O_PLANE_NORMAL(sp, k);
                    if (OF(plane_skip)(ipos, jpos, point, normal, h)) { skip = 1; break; }
                    rp = OF(v3_reflect)(rp, point, normal);
                    rp0 = OF(v3_reflect)(rp0, point, normal);
                    rip0 = OF(v3_reflect)(rip0, point, normal);
                }
                if (skip) continue;
                V3 xm = OF(v3_sub)(ipos0, rp0);
                V3 refx = OF(v3_sub)(rip0, jpos0);
                V3 f_ji = OF(v3_mul)(OF(mul_sv)(ist, OF(k_spiky_grad)(xm, h, s->guards & 2)), -vivj);
                V3 f_ij = OF(v3_mul)(OF(mul_sv)(jst, OF(k_spiky_grad)(OF(v3_neg)(refx), h, s->guards & 2)), -vivj);
                if (corot) f_ij = OF(mul_mv)(jrot, f_ij);
                /* reflect f_ij back across the subset's planes, highest first;
                 * `normal` ends as the lowest plane's normal (used by refvel) */
                for (unsigned k = nsp; k > 0; --k) {
                    if ((bits & (1u << (k - 1))) == 0) continue;
                    normal = O_PLANE_NORMAL(sp, k - 1);
                    f_ij = OF(v3_sub)(f_ij, OF(v3_mul)(OF(v3_mul)(normal, (REAL)2), OF(v3_dot)(normal, f_ij)));
                }
                V3 fe = corot ? OF(v3_add)(OF(v3_neg)(OF(mul_mv)(irot, f_ji)), f_ij) : OF(v3_add)(OF(v3_neg)(f_ji), f_ij);
                fe_sum = OF(v3_add)(fe_sum, fe);
                V3 refvel = OF(v3_sub)(jvel, OF(v3_mul)(OF(v3_mul)(normal, (REAL)2), OF(v3_dot)(normal, jvel)));
                V3 fv = OF(v3_mul)(OF(v3_mul)(OF(v3_sub)(refvel, ivel), mass / s->density[j]),
                                   OF(k_visc_lap)(OF(v3_len)(OF(v3_sub)(rp, ipos)), h));
                fv_sum = OF(v3_add)(fv_sum, fv);
                if ((bits & 1u) == 0) { fec = OF(v3_add)(fec, fe); fvc = OF(v3_add)(fvc, fv); }
            }
        })
        fe_sum = OF(v3_mul)(fe_sum, (REAL)0.5f);
        fv_sum = OF(v3_mul)(fv_sum, visc);
        OF(v3_store)(OF(v3_add)(fe_sum, fv_sum), s->force, i);
        OF(v3_store)(fe_sum, s->force_elastic, i);
        OF(v3_store)(fv_sum, s->force_viscous, i);
        fec = OF(v3_mul)(fec, (REAL)0.5f);
        fvc = OF(v3_mul)(fvc, visc);
        OF(v3_store)(OF(v3_add)(fec, fvc), s->cutoff_force, i);
    }
}
void OF(oracle_compute_forces_solids_corot)(OST *s) { OF(forces_solids)(s, 1); }
void OF(oracle_compute_forces_solids_svk)(OST *s) { OF(forces_solids)(s, 0); }

/* ---- St. Venant-Kirchhoff, solid_svk.cl --------------------------------- */

/* compute_deformations, solid_svk.cl:82-175: F = Apq Aqq^-1 */
void OF(oracle_compute_deformations)(OST *s) {
    const REAL h = s->smoothingradius;
    const unsigned nsp = s->num_symmetry_planes;
    const REAL *sp = s->symmetry_planes;
    long n = s->n;
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long ii = 0; ii < n; ++ii) {
        unsigned i = (unsigned)ii;
        if (s->phase && !s->phase[i]) continue; /* a mixed scene's fluid particle */
        V3 ipos = OF(v3_load)(s->position, i), ipos0 = OF(v3_load)(s->originalpos, i);
        REAL apq[9] = {0}, aqq[6] = {0};
        O_FOR_NEIGHBOURS(s, i, j, {
            if (s->phase && !s->phase[j]) continue;
            V3 jpos = OF(v3_load)(s->position, j), jpos0 = OF(v3_load)(s->originalpos, j);
            V3 p = OF(v3_sub)(jpos, ipos), q = OF(v3_sub)(jpos0, ipos0);
            REAL w = OF(k_poly6)(OF(v3_len)(p), h);
            if (j != i) { OF(contrib_apq)(p, q, w, apq); OF(contrib_aqq)(q, w, aqq); }
            for (unsigned bits = 1; bits < (1u << nsp); ++bits) {
                V3 rp = jpos, rp0 = jpos0;
                int skip = 0;
                for (unsigned k = 0; k < nsp; ++k) {
                    if ((bits & (1u << k)) == 0) continue;
                    V3 point = O_PLANE_POINT(sp, k), normal = O_PLANE_NORMAL(sp, k);
                    if (OF(plane_skip)(ipos, jpos, point, normal, h)) { skip = 1; break; }
                    rp = OF(v3_reflect)(rp, point, normal);
                    rp0 = OF(v3_reflect)(rp0, point, normal);
                }
                if (skip) continue;
                p = OF(v3_sub)(rp, ipos);
                q = OF(v3_sub)(rp0, ipos0);
                REAL dist = OF(v3_len)(p);
                if (dist < h) {
                    w = OF(k_poly6)(dist, h);
                    OF(contrib_apq)(p, q, w, apq);
                    OF(contrib_aqq)(q, w, aqq);
                }
            }
        })
        REAL inv[6];
        OF(oracle_jacobi_invert)(aqq, inv, s->guards & 1);
        OF(mul_as)(apq, inv, s->deformation + 9 * (size_t)i);
    }
}

/* compute_stresses (SVK), solid_svk.cl:1-80: Green strain -> PK2 -> Cauchy.
 * The 0.5 / 1.0 / 2.0 literals are doubles in the source. */
void OF(oracle_compute_stresses_svk)(OST *s) {
    const REAL E = s->youngs_modulus, nu = s->poisson;
    /* E*nu is a float product before the double literals promote it */
    REAL lam = (REAL)((double)(E * nu) / (1.0 + (double)nu) / (1.0 - 2.0 * (double)nu));
    REAL mu = (REAL)((double)E / 2.0 / (1.0 + (double)nu));
    long n = s->n;
#pragma omp parallel for schedule(static) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long i = 0; i < n; ++i) {
        if (s->phase && !s->phase[i]) continue; /* a mixed scene's fluid particle */
        const REAL *F = s->deformation + 9 * i;
        REAL Ft[9], ftf[9], g[6], svk[6], tmp[9], cau[9];
        OF(transpose)(F, Ft);
        OF(mul_mm)(Ft, F, ftf);
        g[S00] = (REAL)(0.5 * (double)ftf[I00] - 0.5);
        g[S11] = (REAL)(0.5 * (double)ftf[I11] - 0.5);
        g[S22] = (REAL)(0.5 * (double)ftf[I22] - 0.5);
        g[S01] = (REAL)(0.5 * (double)ftf[I01]);
        g[S02] = (REAL)(0.5 * (double)ftf[I02]);
        g[S12] = (REAL)(0.5 * (double)ftf[I12]);
        REAL first = lam * (g[S00] + g[S11] + g[S22]);
        svk[S00] = (REAL)((double)first + 2.0 * (double)mu * (double)g[S00]);
        svk[S11] = (REAL)((double)first + 2.0 * (double)mu * (double)g[S11]);
        svk[S22] = (REAL)((double)first + 2.0 * (double)mu * (double)g[S22]);
        svk[S01] = (REAL)(2.0 * (double)mu * (double)g[S01]);
        svk[S02] = (REAL)(2.0 * (double)mu * (double)g[S02]);
        svk[S12] = (REAL)(2.0 * (double)mu * (double)g[S12]);
        OF(mul_as)(F, svk, tmp);
        OF(mul_mm)(tmp, Ft, cau);
        /* multiplyMatrixScalar(1.0/det, ...): the double reciprocal is
         * passed as a float argument (common.cl:239).  The source stores the
         * 9-entry product in a 6-entry array (solid_svk.cl:67); the
         * restatement gives it 9 entries. */
        REAL rdet = (REAL)(1.0 / (double)OF(det)(F));
        for (int k = 0; k < 9; ++k) cau[k] = rdet * cau[k];
        REAL *o = s->stress + 6 * i;
        o[S00] = cau[I00]; o[S11] = cau[I11]; o[S22] = cau[I22];
        o[S01] = cau[I01]; o[S02] = cau[I02]; o[S12] = cau[I12];
    }
}

/* ---- integration and constraints ---------------------------------------- */

/* step_forward, common.cl:691-722 (plus the optional reflective box, an
 * extension with no reference counterpart: a particle that leaves
 * wallbounds is mirrored back inside and its normal velocity reversed). */
void OF(oracle_step_forward)(OST *s) {
    const REAL m = s->mass, dt = s->timestep;
    V3 g = OF(v3)(s->gravity[0], s->gravity[1], s->gravity[2]);
    long n = s->n;
#pragma omp parallel for schedule(static) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long ii = 0; ii < n; ++ii) {
        unsigned i = (unsigned)ii;
        unsigned b = s->body_number[i];
        if (b > 0 && !s->body_dynamic[b - 1]) continue;
        /* rigid bodies (extension) are moved by oracle_rigid_step */
        if (b > 0 && s->rigid_state && b <= s->body_capacity && s->body_dynamic[b - 1] == ORACLE_BODY_RIGID)
            continue;
        V3 f = OF(v3_load)(s->force, i);
        V3 a = OF(v3_add)(OF(v3_div)(f, m), g);
        OF(v3_store)(a, s->acceleration, i);
        V3 v = OF(v3_load)(s->velocity, i);
        V3 vn = OF(v3_add)(v, OF(v3_mul)(a, dt));
        V3 p = OF(v3_load)(s->position, i);
        V3 pn = OF(v3_add)(p, OF(v3_mul)(vn, dt));
        if (s->has_wallbounds) {
            REAL *pc = &pn.x, *vc = &vn.x;
            for (int k = 0; k < 3; ++k) {
                REAL lo = s->wallbounds[2 * k], hi = s->wallbounds[2 * k + 1];
                if (pc[k] < lo) { pc[k] = lo + (lo - pc[k]); vc[k] = -vc[k]; }
                else if (pc[k] > hi) { pc[k] = hi - (pc[k] - hi); vc[k] = -vc[k]; }
            }
        }
        OF(v3_store)(pn, s->position, i);
        OF(v3_store)(vn, s->velocity, i);
    }
}

/* Rigid bodies: an extension with no reference counterpart (the
 * reference's bodies are only fixed or kinematic, rigidbody.cl).  A body b
 * with body_dynamic[b-1] == ORACLE_BODY_RIGID moves rigidly.  After the
 * material's step: its particles' forces are summed (FP64, in index order)
 * into the total force F and the torque about the centre; the body takes
 * the particles' semi-implicit Euler step (a = F/M + g, v += dt a,
 * c += dt v; L += dt tau, q += dt/2 (0, w) q normalised, w = R I0^-1 R^T L)
 * and its particles are placed at x = c + R r0, v = v_c + w x (R r0).  On
 * the body's first substep (or after a reset: flag 0) the centre, mean
 * velocity, inertia, angular momentum and offsets r0 = x - c0 are taken
 * from the particles.  The same algorithm as the CUDA kernels
 * (kernels_rigid.cuh), which sum in a different (blocked) order. */
static void OF(rigid_sym_inverse)(const double I[9], double out[9]) {
    double c00 = I[4] * I[8] - I[5] * I[7], c01 = I[5] * I[6] - I[3] * I[8], c02 = I[3] * I[7] - I[4] * I[6];
    double det = I[0] * c00 + I[1] * c01 + I[2] * c02, tr = I[0] + I[4] + I[8];
    for (int k = 0; k < 9; ++k) out[k] = 0.0;
    if (!(tr > 0.0) || !(fabs(det) > 1e-12 * tr * tr * tr)) return;
    double inv = 1.0 / det;
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

static void OF(rigid_quat_matrix)(const double q[4], double R[9]) {
    double w = q[0], x = q[1], y = q[2], z = q[3];
    R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - w * z);     R[2] = 2 * (x * z + w * y);
    R[3] = 2 * (x * y + w * z);     R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - w * x);
    R[6] = 2 * (x * z - w * y);     R[7] = 2 * (y * z + w * x);     R[8] = 1 - 2 * (x * x + y * y);
}

static void OF(rigid_omega)(const double R[9], const double Iinv0[9], const double L[3], double w[3]) {
    double a[3], b[3];
    for (int r = 0; r < 3; ++r) a[r] = R[r] * L[0] + R[3 + r] * L[1] + R[6 + r] * L[2];
    for (int r = 0; r < 3; ++r) b[r] = Iinv0[3 * r] * a[0] + Iinv0[3 * r + 1] * a[1] + Iinv0[3 * r + 2] * a[2];
    for (int r = 0; r < 3; ++r) w[r] = R[3 * r] * b[0] + R[3 * r + 1] * b[1] + R[3 * r + 2] * b[2];
}

void OF(oracle_rigid_step)(OST *s) {
    if (!s->rigid_state) return;
    const double m = (double)s->mass, dt = (double)s->timestep;
    unsigned nb = s->body_count < s->body_capacity ? s->body_count : s->body_capacity;
    for (unsigned b = 1; b <= nb; ++b) {
        if (s->body_dynamic[b - 1] != ORACLE_BODY_RIGID) continue;
        double *st = s->rigid_state + (size_t)(b - 1) * ORACLE_RIGID_STRIDE;
        unsigned lo = 0, hi = s->n;
        if (st[ORS_FLAG] != 0.0) {
            unsigned h1 = (unsigned)st[ORS_HI] + 1u;
            lo = (unsigned)st[ORS_LO];
            hi = h1 < s->n ? h1 : s->n;
        }
        double N = 0, X[3] = {0, 0, 0}, Vs[3] = {0, 0, 0}, XX[6] = {0, 0, 0, 0, 0, 0}, XV[3] = {0, 0, 0};
        double F[3] = {0, 0, 0}, XF[3] = {0, 0, 0}, mn = 4294967296.0, mx = -1.0;
        for (unsigned i = lo; i < hi; ++i) {
            if (s->body_number[i] != b) continue;
            double x = s->position[3 * i], y = s->position[3 * i + 1], z = s->position[3 * i + 2];
            double vx = s->velocity[3 * i], vy = s->velocity[3 * i + 1], vz = s->velocity[3 * i + 2];
            double fx = s->force[3 * i], fy = s->force[3 * i + 1], fz = s->force[3 * i + 2];
            N += 1.0;
            X[0] += x; X[1] += y; X[2] += z;
            Vs[0] += vx; Vs[1] += vy; Vs[2] += vz;
            XX[0] += x * x; XX[1] += y * y; XX[2] += z * z; XX[3] += x * y; XX[4] += x * z; XX[5] += y * z;
            XV[0] += y * vz - z * vy; XV[1] += z * vx - x * vz; XV[2] += x * vy - y * vx;
            F[0] += fx; F[1] += fy; F[2] += fz;
            XF[0] += y * fz - z * fy; XF[1] += z * fx - x * fz; XF[2] += x * fy - y * fx;
            if (i < mn) mn = i;
            if (i > mx) mx = i;
        }
        if (N == 0.0) { st[ORS_FLAG] = 0.0; continue; }
        if (st[ORS_FLAG] == 0.0) {
            double c[3], v[3];
            for (int k = 0; k < 3; ++k) { c[k] = X[k] / N; v[k] = Vs[k] / N; }
            double cxx = XX[0] - N * c[0] * c[0], cyy = XX[1] - N * c[1] * c[1], czz = XX[2] - N * c[2] * c[2];
            double cxy = XX[3] - N * c[0] * c[1], cxz = XX[4] - N * c[0] * c[2], cyz = XX[5] - N * c[1] * c[2];
            double I0[9] = {m * (cyy + czz), -m * cxy, -m * cxz, -m * cxy, m * (cxx + czz),
                            -m * cyz, -m * cxz, -m * cyz, m * (cxx + cyy)};
            OF(rigid_sym_inverse)(I0, st + ORS_IINV0);
            st[ORS_L] = m * (XV[0] - N * (c[1] * v[2] - c[2] * v[1]));
            st[ORS_L + 1] = m * (XV[1] - N * (c[2] * v[0] - c[0] * v[2]));
            st[ORS_L + 2] = m * (XV[2] - N * (c[0] * v[1] - c[1] * v[0]));
            for (int k = 0; k < 3; ++k) { st[ORS_C + k] = c[k]; st[ORS_C0 + k] = c[k]; st[ORS_V + k] = v[k]; }
            st[ORS_Q] = 1.0; st[ORS_Q + 1] = st[ORS_Q + 2] = st[ORS_Q + 3] = 0.0;
            st[ORS_N] = N; st[ORS_LO] = mn; st[ORS_HI] = mx;
            st[ORS_FLAG] = 1.0;
        } else if (st[ORS_FLAG] == 1.0) {
            st[ORS_FLAG] = 2.0;
        }
        double M = st[ORS_N] * m, c[3] = {st[ORS_C], st[ORS_C + 1], st[ORS_C + 2]};
        double tau[3] = {XF[0] - (c[1] * F[2] - c[2] * F[1]), XF[1] - (c[2] * F[0] - c[0] * F[2]),
                         XF[2] - (c[0] * F[1] - c[1] * F[0])};
        double v[3], L[3], q[4], R[9], w[3];
        for (int k = 0; k < 3; ++k) {
            double a = F[k] / M + (double)s->gravity[k];
            st[ORS_A + k] = a;
            v[k] = st[ORS_V + k] + dt * a;
            c[k] += dt * v[k];
            L[k] = st[ORS_L + k] + dt * tau[k];
        }
        for (int k = 0; k < 4; ++k) q[k] = st[ORS_Q + k];
        OF(rigid_quat_matrix)(q, R);
        OF(rigid_omega)(R, st + ORS_IINV0, L, w);
        double h = 0.5 * dt;
        double dq[4] = {-(w[0] * q[1] + w[1] * q[2] + w[2] * q[3]), w[0] * q[0] + w[1] * q[3] - w[2] * q[2],
                        w[1] * q[0] + w[2] * q[1] - w[0] * q[3], w[2] * q[0] + w[0] * q[2] - w[1] * q[1]};
        double nq = 0.0;
        for (int k = 0; k < 4; ++k) { q[k] += h * dq[k]; nq += q[k] * q[k]; }
        nq = 1.0 / sqrt(nq);
        for (int k = 0; k < 4; ++k) q[k] *= nq;
        OF(rigid_quat_matrix)(q, R);
        OF(rigid_omega)(R, st + ORS_IINV0, L, w);
        for (int k = 0; k < 3; ++k) { st[ORS_C + k] = c[k]; st[ORS_V + k] = v[k]; st[ORS_L + k] = L[k]; st[ORS_W + k] = w[k]; }
        for (int k = 0; k < 4; ++k) st[ORS_Q + k] = q[k];
        for (int k = 0; k < 9; ++k) st[ORS_R + k] = R[k];
        if (s->body_position)
            for (int k = 0; k < 3; ++k) s->body_position[3 * (b - 1) + k] = (REAL)c[k];
        /* place the particles on the body */
        unsigned slo = (unsigned)st[ORS_LO], sh1 = (unsigned)st[ORS_HI] + 1u;
        unsigned shi = sh1 < s->n ? sh1 : s->n;
        REAL a3[3] = {(REAL)st[ORS_A], (REAL)st[ORS_A + 1], (REAL)st[ORS_A + 2]};
        for (unsigned i = slo; i < shi; ++i) {
            if (s->body_number[i] != b) continue;
            double r0[3];
            if (st[ORS_FLAG] == 1.0) {
                for (int k = 0; k < 3; ++k) {
                    REAL o = (REAL)((double)s->position[3 * i + k] - st[ORS_C0 + k]);
                    s->rigid_offset[3 * i + k] = o;
                    r0[k] = o;
                }
            } else {
                for (int k = 0; k < 3; ++k) r0[k] = s->rigid_offset[3 * i + k];
            }
            double rr[3];
            for (int k = 0; k < 3; ++k) rr[k] = R[3 * k] * r0[0] + R[3 * k + 1] * r0[1] + R[3 * k + 2] * r0[2];
            s->position[3 * i] = (REAL)(c[0] + rr[0]);
            s->position[3 * i + 1] = (REAL)(c[1] + rr[1]);
            s->position[3 * i + 2] = (REAL)(c[2] + rr[2]);
            s->velocity[3 * i] = (REAL)(v[0] + (w[1] * rr[2] - w[2] * rr[1]));
            s->velocity[3 * i + 1] = (REAL)(v[1] + (w[2] * rr[0] - w[0] * rr[2]));
            s->velocity[3 * i + 2] = (REAL)(v[2] + (w[0] * rr[1] - w[1] * rr[0]));
            for (int k = 0; k < 3; ++k) s->acceleration[3 * i + k] = a3[k];
        }
    }
}

/* apply_plane_constraints, constraints.cl:1-30 */
void OF(oracle_apply_plane_constraints)(OST *s) {
    const unsigned nc = s->num_plane_constraints;
    const REAL *pc = s->plane_constraints;
    long n = s->n;
#pragma omp parallel for schedule(static) num_threads(s->nthreads > 0 ? s->nthreads : 1)
    for (long ii = 0; ii < n; ++ii) {
        unsigned i = (unsigned)ii;
        unsigned mask = s->plane_constraints_particles[i];
        if (mask == 0) continue;
        V3 ipos = OF(v3_load)(s->position, i), ivel = OF(v3_load)(s->velocity, i);
        for (unsigned c = 0; c < nc; ++c) {
            if ((mask & (1u << c)) == 0) continue;
            V3 point = O_PLANE_POINT(pc, c), normal = O_PLANE_NORMAL(pc, c);
            ipos = OF(v3_sub)(ipos, OF(v3_mul)(normal, OF(v3_dot)(normal, OF(v3_sub)(ipos, point))));
            ivel = OF(v3_sub)(ivel, OF(v3_mul)(normal, OF(v3_dot)(normal, ivel)));
        }
        OF(v3_store)(ipos, s->position, i);
        OF(v3_store)(ivel, s->velocity, i);
    }
}

/* set_body_position, rigidbody.cl:1-33 */
void OF(oracle_set_body_position)(OST *s, unsigned body, const REAL *newpos) {
    if (body >= s->body_count) return;
    V3 np = OF(v3)(newpos[0], newpos[1], newpos[2]);
    V3 old = OF(v3_load)(s->body_position, body);
    for (size_t i = 0; i < s->n; ++i) {
        if (s->body_number[i] != body + 1) continue;
        V3 pos = OF(v3_load)(s->position, i);
        OF(v3_store)(OF(v3_add)(OF(v3_sub)(pos, old), np), s->position, i);
        OF(v3_store)(OF(v3_div)(OF(v3_sub)(np, old), s->timestep), s->velocity, i);
    }
    OF(v3_store)(np, s->body_position, body);
}

/* get_matrix_from_euler (XYX), rigidbody.cl:35-68 */
static void OF(euler_xyx)(V3 e, REAL out[9]) {
    REAL cx = R_COS(e.x), sx = R_SIN(e.x), cy = R_COS(e.y), sy = R_SIN(e.y);
    REAL cx2 = R_COS(e.z), sx2 = R_SIN(e.z);
    REAL rx[9] = {1, 0, 0, 0, cx, -sx, 0, sx, cx};
    REAL ry[9] = {cy, 0, -sy, 0, 1, 0, sy, 0, cy};
    REAL rx2[9] = {1, 0, 0, 0, cx2, -sx2, 0, sx2, cx2};
    REAL ryx[9];
    OF(mul_mm)(ry, rx, ryx);
    OF(mul_mm)(rx2, ryx, out);
}
/* set_body_rotation, rigidbody.cl:70-120.  As in the source, the matrix
 * applied is built from the body's STORED Euler angles; the new angles are
 * only recorded. */
void OF(oracle_set_body_rotation)(OST *s, unsigned body, const REAL *euler) {
    if (body >= s->body_count) return;
    REAL binv[9], t[9], t2[9];
    OF(euler_xyx)(OF(v3_load)(s->body_euler_rotation, body), binv);
    OF(transpose)(binv, t);
    for (size_t i = 0; i < s->n; ++i) {
        if (s->body_number[i] != body + 1) continue;
        REAL *prot = s->rotation + 9 * i;
        REAL tmp2[9], tmp[9];
        OF(mul_mm)(t, prot, tmp2);
        V3 pos = OF(v3_load)(s->position, i);
        V3 rpos = OF(mul_mv)(tmp2, pos);
        OF(mul_mm)(tmp2, prot, tmp);
        for (int k = 0; k < 9; ++k) prot[k] = tmp[k];
        OF(v3_store)(rpos, s->position, i);
    }
    (void)t2;
    s->body_euler_rotation[3 * body] = euler[0];
    s->body_euler_rotation[3 * body + 1] = euler[1];
    s->body_euler_rotation[3 * body + 2] = euler[2];
}

/* populate_position_cuboid, common.cl:533-555: work item (i, j, k) of a
 * size[0] x size[1] x size[2] range writes particle p = i + size[0] j +
 * size[0] size[1] k at (i / (size[0] - 1)) (c2 - c1) + c1 per axis, unless
 * p >= pnum; the item p = pnum - 1 sets n = pnum, else the last item of the
 * range sets n = its size.  Items run in order; no two write one particle. */
void OF(oracle_populate_position_cuboid)(OST *s, unsigned pnum, const REAL *c1, const REAL *c2,
                                         const unsigned *size) {
    for (unsigned k = 0; k < size[2]; ++k)
        for (unsigned j = 0; j < size[1]; ++j)
            for (unsigned i = 0; i < size[0]; ++i) {
                unsigned p = i + size[0] * j + size[0] * size[1] * k;
                if (p >= pnum) continue;
                if (p == pnum - 1) s->n = pnum;
                else if (i == size[0] - 1 && j == size[1] - 1 && k == size[2] - 1) s->n = size[0] * size[1] * size[2];
                REAL q[3];
                const unsigned idx[3] = {i, j, k};
                for (int a = 0; a < 3; ++a)
                    q[a] = ((REAL)idx[a] / (REAL)(size[a] - 1)) * (c2[a] - c1[a]) + c1[a];
                OF(v3_store)(OF(v3)(q[0], q[1], q[2]), s->position, p);
            }
}

/* rotate_particles, common.cl:556-604: x <- Rx(ax) (Ry(ay) Rz(az)) x for
 * the first n particles, with the source's sign conventions (Ry has -sin
 * above the diagonal). */
void OF(oracle_rotate_particles)(OST *s, REAL ax, REAL ay, REAL az) {
    REAL cx = R_COS(ax), sx = R_SIN(ax), cy = R_COS(ay), sy = R_SIN(ay), cz = R_COS(az), sz = R_SIN(az);
    REAL rx[9] = {1, 0, 0, 0, cx, -sx, 0, sx, cx};
    REAL ry[9] = {cy, 0, -sy, 0, 1, 0, sy, 0, cy};
    REAL rz[9] = {cz, -sz, 0, sz, cz, 0, 0, 0, 1};
    REAL ryz[9], r[9];
    OF(mul_mm)(ry, rz, ryz);
    OF(mul_mm)(rx, ryz, r);
    for (size_t i = 0; i < s->n; ++i) OF(v3_store)(OF(mul_mv)(r, OF(v3_load)(s->position, i)), s->position, i);
}

#undef O_FOR_NEIGHBOURS
#undef O_PLANE_POINT
#undef O_PLANE_NORMAL
#undef O_PI
#undef V3
#undef OST
#undef OF
#undef S10
#undef S20
#undef S21
