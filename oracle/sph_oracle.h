/*
 * sph_oracle.h -- CPU restatement of the opencl-sph per-substep particle
 * pipeline, used ONLY as a test oracle and as the timed CPU baseline.
 *
 * This is test infrastructure: the product library never links, loads or
 * calls anything here. Every function restates one reference kernel
 * (the kernels/ OpenCL files of tauroid/opencl-sph) and cites the lines it
 * follows.
 *
 * The state struct is a flat table of field pointers laid out exactly like
 * the reference's psdata fields (AoS float[3] vectors, row-major 3x3
 * matrices, symmetric tensors as [xx,yy,zz,xy,xz,yz]); a field that a
 * kernel does not use may be NULL.  Two instantiations exist: _f32 (REAL =
 * float, the reference precision) and _f64 (REAL = double, the FP64 run
 * that errors are reported against).
 *
 * Deviations from the OpenCL source, all deliberate and shared with the
 * CUDA path:
 *   - float->uint conversion in find_particle_bins saturates (negative and
 *     NaN -> 0), the GPU's conversion rule; C leaves it undefined.
 *   - prefix_sum is a correct serial exclusive scan (the reference's
 *     cross-work-group fix-up is racy, common.cl:501-514).
 *   - insert_particles_in_bin_array is a stable scatter: particles of one
 *     cell appear in ascending index order (the reference's order is the
 *     nondeterministic atomic_inc order, common.cl:528).
 *   - set_body_position / set_body_rotation read the old body pose for
 *     every particle before it is overwritten (the reference relies on an
 *     unsynchronised global barrier, rigidbody.cl:13-17,30-32).
 *   - guards bit 0 defines the Givens angle as 0 when the pivot
 *     off-diagonal is exactly 0 (the reference evaluates atan(0/0) = NaN
 *     there when the two diagonal entries are equal, common.cl:124).
 *   - guards bit 1 makes a pair of distinct particles at exactly zero
 *     distance contribute nothing to the fluid pressure/viscosity force and
 *     gives a zero spiky gradient at zero distance (the reference divides
 *     by the distance there, fluids.cl:48 and common.cl:83, producing NaN;
 *     FP32 WCSPH under tension can merge two particles exactly).
 * With guards = 0 the oracle reproduces the reference bit for bit.
 *
 * Mixed fluid-solid scenes (phase != NULL) are an extension with no
 * reference counterpart: a solid particle's rest density, deformation
 * gradient, stress and elastic forces cover its solid neighbours only; the
 * fluid force pass gives every pair with a fluid particle the fluid pair
 * term (fluids.cl:1-63), which a solid particle adds to its elastic force.
 */
#ifndef SPH_ORACLE_H_
#define SPH_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ORACLE_STATE_FIELDS(REAL)                                          \
    unsigned int n;                 /* active particles */                     \
    unsigned int gridres[3];                                                   \
    REAL mass, timestep, smoothingradius;                                      \
    REAL restdens, stiffness, viscosity;                                       \
    REAL youngs_modulus, poisson;                                              \
    REAL gravity[3];                                                           \
    REAL gridbounds[6];                                                        \
    unsigned int num_symmetry_planes;   REAL *symmetry_planes;   /* [P][2][3] */\
    unsigned int num_plane_constraints; REAL *plane_constraints; /* [P][2][3] */\
    unsigned int *plane_constraints_particles;                                 \
    unsigned int body_count;                                                   \
    unsigned int *body_number, *body_dynamic;                                  \
    REAL *body_position, *body_euler_rotation;                                 \
    REAL *position, *velocity, *acceleration, *force;                          \
    REAL *density, *density0, *originalpos;                                    \
    REAL *rotation, *strain, *stress, *apq_temp, *intermediate, *deformation;  \
    REAL *cutoff_force, *force_elastic, *force_viscous;                        \
    unsigned int *num_neighbours;                                              \
    unsigned int *gridcell, *gridcount, *celloffset, *cellparticles;           \
    /* optional reflective box (extension, not in the reference): */          \
    unsigned int has_wallbounds; REAL wallbounds[6];                           \
    int guards; /* bit 0: Givens zero pivot, bit 1: zero-distance pairs */     \
    int nthreads;                                                              \
    /* rigid bodies (extension, not in the reference; oracle_rigid_step):  */ \
    /* body_dynamic[b-1] == 2 marks body b rigid; rigid_state holds        */ \
    /* ORACLE_RIGID_STRIDE doubles per body (zeroed = to set up), and     */ \
    /* rigid_offset[3 * n] the particles' body-frame offsets               */ \
    unsigned int body_capacity;                                                \
    double *rigid_state;                                                       \
    REAL *rigid_offset;                                                        \
    /* mixed fluid-solid scenes (extension, not in the reference): phase  */ \
    /* per particle (0 fluid, 1 SVK solid; NULL: one material) and the    */ \
    /* solids' own viscosity when has_solid_viscosity                     */ \
    unsigned int *phase;                                                       \
    unsigned int has_solid_viscosity; REAL solid_viscosity;

#define ORACLE_BODY_RIGID 2u
#define ORACLE_RIGID_STRIDE 64
/* slots of a body's rigid_state */
enum {
    ORS_FLAG = 0, /* 0: to set up, 1: set up this substep, 2: running */
    ORS_N = 1,    /* particle count */
    ORS_LO = 2,   /* lowest / highest particle index */
    ORS_HI = 3,
    ORS_C = 4,    /* centre (3) */
    ORS_V = 7,    /* linear velocity (3) */
    ORS_Q = 10,   /* orientation quaternion (w, x, y, z) */
    ORS_L = 14,   /* angular momentum (3) */
    ORS_IINV0 = 17, /* body-frame inverse inertia, 3x3 row-major */
    ORS_W = 26,   /* angular velocity (3) */
    ORS_A = 29,   /* linear acceleration of the last substep (3) */
    ORS_R = 32,   /* rotation matrix (3x3 row-major) */
    ORS_C0 = 41   /* centre at set-up (3) */
};

typedef struct { SPH_ORACLE_STATE_FIELDS(float)  } sph_oracle_state_f32;
typedef struct { SPH_ORACLE_STATE_FIELDS(double) } sph_oracle_state_f64;

#define SPH_ORACLE_DECLARE(SFX, REAL)                                                \
    void oracle_find_particle_bins##SFX(sph_oracle_state##SFX *s);             \
    void oracle_sort_particles##SFX(sph_oracle_state##SFX *s);                 \
    void oracle_compute_particle_bins##SFX(sph_oracle_state##SFX *s);          \
    void oracle_init_original_position##SFX(sph_oracle_state##SFX *s);         \
    void oracle_compute_original_density##SFX(sph_oracle_state##SFX *s);       \
    void oracle_compute_density##SFX(sph_oracle_state##SFX *s);                \
    void oracle_compute_forces_fluids##SFX(sph_oracle_state##SFX *s);          \
    void oracle_compute_rotations_and_strains##SFX(sph_oracle_state##SFX *s);  \
    void oracle_compute_stresses_corot##SFX(sph_oracle_state##SFX *s);         \
    void oracle_compute_forces_solids_corot##SFX(sph_oracle_state##SFX *s);    \
    void oracle_compute_deformations##SFX(sph_oracle_state##SFX *s);           \
    void oracle_compute_stresses_svk##SFX(sph_oracle_state##SFX *s);           \
    void oracle_compute_forces_solids_svk##SFX(sph_oracle_state##SFX *s);      \
    void oracle_step_forward##SFX(sph_oracle_state##SFX *s);                   \
    void oracle_rigid_step##SFX(sph_oracle_state##SFX *s);                     \
    void oracle_apply_plane_constraints##SFX(sph_oracle_state##SFX *s);        \
    void oracle_set_body_position##SFX(sph_oracle_state##SFX *s,               \
                                       unsigned int body, const REAL *pos);   \
    void oracle_set_body_rotation##SFX(sph_oracle_state##SFX *s,               \
                                       unsigned int body, const REAL *euler); \
    void oracle_populate_position_cuboid##SFX(sph_oracle_state##SFX *s,        \
                                              unsigned int pnum, const REAL *c1, \
                                              const REAL *c2, const unsigned int *size); \
    void oracle_rotate_particles##SFX(sph_oracle_state##SFX *s, REAL ax,       \
                                      REAL ay, REAL az);                       \
    void oracle_get_r##SFX(const REAL *apq, REAL *r, int guard);             \
    void oracle_jacobi_invert##SFX(const REAL *m6, REAL *out6, int guard);

SPH_ORACLE_DECLARE(_f32, float)
SPH_ORACLE_DECLARE(_f64, double)

#ifdef __cplusplus
}
#endif

#endif
