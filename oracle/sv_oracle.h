/*
 * sv_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * C API of the CPU oracle: a restatement, in C++, of the reference's MPM substep
 * (Squishy Volumes, rust/crates/cpu) and of its constitutive math
 * (rust/crates/util/src/elastic.rs).  It exists to check the CUDA library and to
 * serve as the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and
 * bench.py (cpu_baseline / --impl reference legs) may load it; the product never
 * links it.
 *
 * Parity status: the reference (Rust) cannot be built in this environment, so
 * this restatement is pinned by the reference's own test strategy re-derived:
 * finite-difference checks of every stress against its energy with the
 * reference's parameter sets (util/src/elastic.rs:679-696, util/src/tests.rs),
 * hand-computed known answers for the quadratic B-spline and the return maps,
 * and the conservation laws of the transfer.  Whole-substep results are
 * therefore "pinned by derivation", not by reference-produced vectors.
 */
#ifndef SV_ORACLE_H
#define SV_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-particle inputs use the reference's file_frame::Particles layout:
 * positions [n][3], position_gradients [n][9] column-major (nalgebra Matrix3),
 * velocities [n][3], velocity_gradients [n][9], flags u32 (ParticleFlags),
 * and ParticleParameters spread into arrays (file_frame/src/particles.rs:55-90).
 * model/xi/theta_c/theta_s/plastic_j are additions (not in the reference). */
typedef struct svo_particles {
    uint64_t n;
    uint32_t *flags;
    float *positions;
    float *position_gradients;
    float *velocities;
    float *velocity_gradients;
    float *elastic_energies;
    uint32_t *collider_bits;
    /* ParticleParameters */
    const float *mass;
    const float *initial_volume;
    const float *viscosity_dynamic; /* may be NULL when no particle has USE_VISCOSITY */
    const float *viscosity_bulk;
    const float *mu;
    const float *lambda;
    const float *sand_alpha;        /* may be NULL when no particle has USE_SAND_ALPHA */
    const int32_t *exponent;
    const float *bulk_modulus;
    /* additions: 0 = reference semantics, 1 = fixed-corotated, 2 = snow */
    const uint32_t *model;          /* may be NULL (all 0) */
    const float *hardening;         /* snow xi */
    const float *crit_compression;  /* snow theta_c */
    const float *crit_stretch;      /* snow theta_s */
    float *plastic_j;               /* snow hardening state J_p, may be NULL */
} svo_particles;

typedef struct svo_consts {
    float grid_node_size;   /* scaled */
    float domain_min[3];    /* scaled */
    float domain_max[3];
    /* addition: grid boundary plane on axis `ground_axis` at `ground_height`
     * (0 = off, 1 = sticky, 2 = slip) */
    int32_t ground_mode;
    int32_t ground_axis;
    float ground_height;
} svo_consts;

/* The inputs of frames a and b (xpu/src/frame_input.rs:33-65): gravity,
 * particle goals and collider meshes, interpolated linearly inside the
 * frame every substep (cpu/src/phase/interpolate_input.rs:18-106).
 * goal_flags_* are the frames' particle flags (only HAS_GOAL is read),
 * goal_positions_* [n][3]; both NULL for no goals.  Colliders: triangles
 * [n_triangles][3] into the vertex arrays [n_vertices][3], the collider
 * (0..15) of each triangle, per-triangle friction and damping.  Every *_b
 * array is ignored when has_b == 0 (b = a, as at the end of the input). */
typedef struct svo_frame_input {
    uint32_t frames_per_second;
    uint32_t frame;
    uint32_t has_b;
    float gravity_a[3], gravity_b[3];
    const uint32_t *goal_flags_a, *goal_flags_b;
    const float *goal_positions_a, *goal_positions_b;
    uint32_t n_vertices, n_triangles;
    const uint32_t *triangles;
    const uint32_t *triangle_collider;
    const float *vertex_positions_a, *vertex_positions_b;
    const float *friction_a, *friction_b;
    const float *damping_a, *damping_b;
    float leaf_size;
} svo_frame_input;

/* Scalar constitutive functions in double precision (util/src/elastic.rs). */
double svo_mu(double youngs_modulus, double poissons_ratio);
double svo_lambda(double youngs_modulus, double poissons_ratio);
double svo_kernel_quadratic(double x);
double svo_energy_neo_hookean(double mu, double lambda, const double F[9]);
void svo_piola_neo_hookean(double mu, double lambda, const double F[9], double P[9]);
double svo_energy_inviscid(double bulk_modulus, int32_t exponent, const double F[9]);
void svo_piola_inviscid(double bulk_modulus, int32_t exponent, const double F[9], double P[9]);
double svo_energy_fixed_corotated(double mu, double lambda, const double F[9]);
void svo_piola_fixed_corotated(double mu, double lambda, const double F[9], double P[9]);
void svo_cauchy_viscosity(double dynamic, double bulk, const double C[9], double S[9]);
void svo_svd3(const double F[9], double U[9], double S[3], double V[9]);
/* Plastic projections in double: sand (advance_particles.rs:48-71), fluid
 * (:77-85), snow (addition). F is updated in place.  svo_project_sand
 * returns 0, or -1 (F unchanged) on the compressive branch with mu <= 0,
 * where the reference asserts mu > 0 (advance_particles.rs:57). */
int svo_project_sand(double mu, double lambda, double alpha, double F[9]);
void svo_project_fluid(double F[9]);
void svo_project_snow(double theta_c, double theta_s, double F[9], double *plastic_j);
double svo_friction_angle_to_alpha(double friction_angle_rad);

/* Whole-state oracle.  fp64 != 0 runs the precision twin (T = double). */
void *svo_create(const svo_particles *p, const svo_consts *c, int fp64, int threads);
void svo_destroy(void *s);
/* Runs n_substeps substeps of the reference phase cycle with a fixed dt
 * (adaptive_time_steps = false).  Returns 0, or 1 when an energy error stopped
 * the run early (a particle got FAILED, advance_particles.rs:73-74), or 3
 * when a sand particle was compressed with mu <= 0 (the reference's assert at
 * advance_particles.rs:57; that substep's advance is complete, its cull is
 * not run). */
int svo_step(void *s, uint32_t n_substeps, float dt, const float gravity[3]);
/* With a frame input set (copied), every substep starts with the input
 * interpolation at the state's time and runs Collide; gravity then comes from
 * the input and the gravity arguments are ignored.  svo_step advances the
 * time by dt per substep.  Returns -2 from a substep whose time lies outside
 * the loaded frame (the reference's WrongFrameLoaded). */
int svo_set_frame_input(void *s, const svo_frame_input *in);
void svo_set_time(void *s, double time);
double svo_get_time(void *s);
/* Adaptive substeps while *time < target (cpu_state.rs:146-197 with
 * adaptive_time_steps = true); returns 0, 1 on an energy error, 2 on a zero
 * time step, 3 on a sand particle compressed with mu <= 0.  limits: the last substep's dt of external force, scatter and
 * advance, then the velocity, deformation, sound and isolated limits and the
 * allowed step (FLT_MAX = none). */
int svo_step_adaptive(void *s, double *time, double target, float max_dt, const float gravity[3],
                      uint32_t *substeps, float limits[8]);
/* Writes the state back in the caller's original particle order
 * (cpu_state.rs:71-135 to_io_state). */
void svo_download(void *s, svo_particles *out);
/* Grid after P2G + meld of the most recent substep: nodes with mass > 0 only,
 * sorted by (i, j, k, collider_bits).  Returns the node count; writes at most
 * capacity entries. */
/* The reference's P2G mass (scatter_momentum.rs:22-93) with every node's
 * fp32 sum taken in one canonical order: over the 27 base cells n - (i, j, k)
 * in lexicographic order, then the cell's particles in ascending index, left
 * to right.  Positions [n][3]; tombstoned particles skipped.  Writes the
 * nodes with mass > 0 in ascending (i, j, k) order (at most cap); returns
 * their count. */
uint64_t svo_deterministic_grid_mass(const float *pos, const float *mass, const uint32_t *flags, uint64_t n, float dx,
                                     int32_t *ids, float *masses, uint64_t cap);
uint64_t svo_grid(void *s, int32_t *node_ids, float *masses, float *velocities,
                  uint64_t capacity);
/* Runs the first half of a substep (sort, external force, grid nodes, P2G,
 * meld) without touching particle state; the grid is then readable through
 * svo_grid. */
void svo_p2g_only(void *s, float dt, const float gravity[3]);

/* Binning-key contract of the CUDA library: for each position
 * c = floor(x / dx - 0.5) (fp32), lc = c - origin, key =
 * (((lc.x>>2) * nb.y + (lc.y>>2)) * nb.z + (lc.z>>2)) << 6 | (lc&3 packed xyz),
 * 0xFFFFFFFF for tombstoned particles.  perm = stable sort of keys. */
void svo_binning_keys(uint64_t n, const float *positions, const uint32_t *flags, float dx,
                      const int32_t origin[3], const int32_t nblocks[3], uint32_t *keys);
void svo_stable_sort_perm(uint64_t n, const uint32_t *keys, uint32_t *perm);

#ifdef __cplusplus
}
#endif
#endif
