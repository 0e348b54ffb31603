/*
 * squishy_volumes_cuda.h -- C ABI of the GB300 MPM substep library
 * (libsquishy_volumes_cuda.so).
 *
 * It replaces the CPU backend of Squishy Volumes behind the backend switch
 * rust/crates/core/src/compute_thread.rs:101-117 (`enum ComputeState`):
 *
 *   reference call                                          | entry point here
 *   --------------------------------------------------------+---------------------------
 *   CpuState::from_io_state (cpu/src/cpu_state.rs:25-66)    | sv_create
 *   CpuState::produce_next_state (cpu/src/cpu_state.rs:146-197),
 *     its substep loop :167-194 with adaptive_time_steps off | sv_step
 *   CpuState::to_io_state (cpu/src/cpu_state.rs:68-135)     | sv_download, sv_download_grid
 *   drop(CpuState)                                          | sv_destroy
 *   error Display (cpu/src/errors.rs:9-36)                  | sv_last_error_string
 *
 * Conventions
 *  - Plain pointers and sizes; no callbacks.  The caller owns every host
 *    buffer; the handle owns all device memory.
 *  - Return value: 0 = success, negative = fatal (CUDA error, out of memory,
 *    invalid argument); the message is in sv_last_error_string() (per thread).
 *  - sv_step reports physics outcomes in *status_out as a bit mask that
 *    mirrors the reference GPU status word (rust/crates/gpu/src/status.rs:27-30):
 *    SV_STATUS_PARTICLE_INVERTED means a particle reached det F <= 0 and got
 *    the FAILED flag; like the reference's EnergyError the state is still
 *    valid and should be stored (compute_thread.rs:165-169).
 *  - One handle is driven from one host thread at a time (the reference calls
 *    its backend from its single compute thread, compute_thread.rs:78).
 *  - Particle arrays follow rust/crates/file_frame/src/particles.rs:92-109:
 *    positions [n][3], position_gradients [n][9] column-major (nalgebra),
 *    velocities [n][3], velocity_gradients [n][9], flags u32 (ParticleFlags,
 *    :21-33), and ParticleParameters (:55-90) spread into per-particle arrays.
 */
#ifndef SQUISHY_VOLUMES_CUDA_H
#define SQUISHY_VOLUMES_CUDA_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ParticleFlags, rust/crates/file_frame/src/particles.rs:21-33. */
#define SV_IS_SOLID (1u << 0)
#define SV_IS_FLUID (1u << 1)
#define SV_USE_VISCOSITY (1u << 2)
#define SV_USE_SAND_ALPHA (1u << 3)
#define SV_HAS_GOAL (1u << 4)
#define SV_TOMBSTONED (1u << 5)
#define SV_FAILED (1u << 6)

/* Status bits of sv_step (rust/crates/gpu/src/status.rs:27-30 meaning). */
#define SV_STATUS_CAPACITY_EXCEEDED (1u << 0) /* grid block capacity too small */
#define SV_STATUS_PARTICLE_INVERTED (1u << 3) /* det F <= 0: FAILED set */
#define SV_STATUS_CANCELED (1u << 8)          /* cancel flag seen between substeps */
/* A sand particle (SV_USE_SAND_ALPHA) with mu <= 0 reached the compressive
 * branch of the Drucker-Prager return map, where the reference asserts
 * mu > 0 (rust/crates/cpu/src/phase/advance_particles.rs:57) and its compute
 * thread panics.  That particle keeps its unprojected F for the substep, the
 * substeps after it do not run, and sv_step / sv_step_adaptive return -1
 * with this bit in *status_out.  In expansion mu <= 0 is valid: F becomes
 * U V^T as in the reference. */
#define SV_STATUS_SAND_INVALID_MU (1u << 11)

/* Material models.  SV_MODEL_REFERENCE selects what the reference does from
 * the flags: Neo-Hookean solid (plus the sand return map with
 * SV_USE_SAND_ALPHA) or the inviscid fluid.  The other two are additions
 * that the reference does not have. */
#define SV_MODEL_REFERENCE 0u
#define SV_MODEL_FIXED_COROTATED 1u
#define SV_MODEL_SNOW 2u

typedef struct sv_consts {
    /* InputConsts::scaled_grid_node_size / scaled_domain_{min,max}
     * (rust/crates/file_input/src/header.rs:36-58) */
    float grid_node_size;
    float domain_min[3];
    float domain_max[3];
    /* Addition (not in the reference): a grid boundary plane on axis
     * ground_axis at ground_height; 0 = off, 1 = sticky, 2 = slip. */
    int32_t ground_mode;
    int32_t ground_axis;
    float ground_height;
    /* Addition: 0 = fp32 positions; 1 = int32 cell index + fp32 in-cell offset. */
    uint32_t position_form;
    /* When the fp32 3x3 SVD is redone in fp64: 0 = never, 1 = det F < 0.05
     * (default), 2 = det F < 0.05 or min singular-value gap < 1e-4. */
    uint32_t svd_fp64_policy;
    /* Grid block (4^3 nodes) capacity; 0 = size it from the domain. */
    uint64_t block_capacity;
    /* Substeps between binning sorts: 0 = adaptive (at most 8), 1 = every
     * substep like the reference (cpu/src/phase/sort.rs, "only to optimize
     * memory access"), k = every k substeps.  Results do not depend on it
     * beyond fp32 summation order. */
    uint32_t sort_interval;
    /* How sv_create and sv_download move the particle arrays: 0 = kernels
     * that read and write the caller's host arrays directly where the
     * device can access pageable memory (a Grace host over NVLink-C2C), else
     * staged copies; 1 = staged copies always.  Same results either way. */
    uint32_t host_transfer;
    /* Addition: 1 = deterministic P2G.  Every substep bins the particles by
     * (cell, original index) and gathers each grid node's mass and momentum
     * in one fixed order: the 27 base cells around the node in lexicographic
     * order, then each cell's particles in ascending original index, left to
     * right in fp32.  The node masses then equal, bit for bit, the
     * reference's P2G mass (scatter_momentum.rs:22-93) summed in that order,
     * and every run of the same input gives the same bits.  Several times
     * slower than the default scatter; fp32 positions (position_form 0), no
     * frame input and no learned closure. */
    uint32_t deterministic_p2g;
    uint32_t reserved[3];
} sv_consts;

typedef struct sv_particles {
    uint64_t n;
    uint32_t *flags;
    float *positions;
    float *position_gradients;
    float *velocities;
    float *velocity_gradients;
    float *elastic_energies;       /* may be NULL */
    uint32_t *collider_bits;       /* may be NULL (all 0) */
    /* ParticleParameters (read by sv_create only) */
    const float *mass;
    const float *initial_volume;
    const float *viscosity_dynamic; /* NULL unless some particle has SV_USE_VISCOSITY */
    const float *viscosity_bulk;
    const float *mu;               /* solids */
    const float *lambda;
    const float *sand_alpha;       /* NULL unless some particle has SV_USE_SAND_ALPHA */
    const int32_t *exponent;       /* fluids */
    const float *bulk_modulus;
    /* additions (NULL = all SV_MODEL_REFERENCE) */
    const uint32_t *model;
    const float *hardening;        /* snow xi */
    const float *crit_compression; /* snow theta_c */
    const float *crit_stretch;     /* snow theta_s */
    float *plastic_j;              /* snow hardening state J_p (in and out), may be NULL */
} sv_particles;

typedef struct sv_handle sv_handle;

/* CpuState::from_io_state (cpu/src/cpu_state.rs:25-66): uploads the particles
 * and sizes the sparse grid.  Fails on invalid flags (neither or both of
 * IS_SOLID/IS_FLUID, like core/src/initialization.rs:197-201), on a domain
 * whose dense block index reaches 2^26 blocks, or on a CUDA error. */
int sv_create(const sv_consts *consts, const sv_particles *particles, sv_handle **out);

/* The substep loop of CpuState::produce_next_state (cpu_state.rs:167-194)
 * with adaptive_time_steps = false: n_substeps substeps of size dt with the
 * given (already interpolated) gravity.  `cancel` may be NULL; when it points
 * at a nonzero value the call stops (Harness::check, xpu/src/harness.rs:69-75)
 * and reports SV_STATUS_CANCELED.  Substeps are queued in chunks (16 when
 * `cancel` is given, 64 otherwise) and the host waits for each chunk by
 * polling it (yielding between polls), checking `cancel` meanwhile, like the reference's
 * GPU backend waits (gpu_state.rs:509-522): a cancel set from another thread
 * during a call takes effect once the chunk in flight has completed, and the
 * state stays that of the last completed substep.  The number of substeps
 * completed is written to *substeps_done when that is not NULL. */
int sv_step(sv_handle *h, uint32_t n_substeps, float dt, const float gravity[3],
            const volatile int32_t *cancel, uint32_t *status_out, uint32_t *substeps_done);

/* CpuState::to_io_state (cpu_state.rs:68-135): particle state in the
 * caller's original order.  Only the mutable arrays of `out` are written
 * (flags, positions, position_gradients, velocities, velocity_gradients,
 * elastic_energies, collider_bits, plastic_j); NULL arrays are skipped. */
int sv_download(sv_handle *h, sv_particles *out);

/* The grid of the most recent substep (to_io_state's store_grid part):
 * nodes with mass > 0, sorted by node id (i, j, k).  Writes up to `capacity`
 * entries; *count gets the total. */
int sv_download_grid(sv_handle *h, int32_t *node_ids, float *masses, float *velocities,
                     uint64_t capacity, uint64_t *count);

void sv_destroy(sv_handle *h);

/* Addition (not in the reference): many independent scenes advanced by the
 * same launches.  Scene s has its own consts[s] (domain, cull bounds) and
 * particles[s]; all scenes share grid_node_size, the ground plane (which must
 * be on axis 2) and the SVD policy, and are stepped together by sv_step with
 * one dt and gravity.  Scenes are placed side by side in x and y in one block
 * index and always use the int32-cell + fp32-offset position form, so their
 * placement is an exact whole-cell translation; sv_download and
 * sv_download_scene return positions in each scene's own coordinates, while
 * grid node ids from sv_download_grid are in the shared placement. */
int sv_create_batched(const sv_consts *consts, const sv_particles *particles, uint32_t n_scenes, sv_handle **out);
uint32_t sv_scene_count(sv_handle *h);
/* sv_download restricted to one scene (out->n must equal that scene's count). */
int sv_download_scene(sv_handle *h, uint32_t scene, sv_particles *out);

/* Message of the last failure on this thread ("" if none). */
const char *sv_last_error_string(void);

/* ---- inspection entry points used by the parity tests and the benchmark ---- */

/* Runs the first half of one substep (binning sort, external force, P2G,
 * grid update) on the current state without changing particle state; the
 * grid is then readable with sv_download_grid. */
int sv_p2g_only(sv_handle *h, float dt, const float gravity[3]);

/* Binning keys of the current particles (in device order) and the stable
 * sort permutation of those keys.  Key contract:
 * c = floor(x / dx - 0.5) in fp32, lc = c - origin,
 * key = (((lc.x>>2)*nb.y + (lc.y>>2))*nb.z + (lc.z>>2)) << 6
 *       | (lc.x&3)<<4 | (lc.y&3)<<2 | (lc.z&3), 0xFFFFFFFF when tombstoned.
 * Also returns the original particle index of each device slot. */
int sv_binning(sv_handle *h, uint32_t *keys, uint32_t *perm, uint32_t *original_index);

/* Grid layout: node origin and block counts of the dense block index. */
int sv_grid_layout(sv_handle *h, int32_t origin[3], int32_t nblocks[3]);

/* Stable LSD radix sort of n (key, index) pairs on the device: writes the
 * permutation that stably sorts `keys` (host buffers; allocates device
 * memory per call). */
int sv_sort_pairs(const uint32_t *keys, uint32_t *perm, uint64_t n);

/* No counterpart in the reference.  The same stable sort as sv_sort_pairs,
 * for callers that must not allocate device memory: a plugin running inside
 * a host application that hands out the whole device-memory budget from its
 * own pool (an allocation behind the pool's back breaks its accounting), or
 * a loop with a fixed time budget per iteration that cannot take the
 * device-wide synchronisation a cudaMalloc / cudaFree may cause.  It
 * allocates nothing: its scratch is one fixed array of
 * SV_NOALLOC_SCRATCH_BYTES (16,777,984 bytes, about 16.8 MB) compiled into
 * the library, which every GPU that loads the library holds until the
 * process exits.
 *  - keys and perm are DEVICE pointers to n uint32 each, owned by the
 *    caller; perm receives the permutation that stably sorts keys.
 *  - n may be at most SV_NOALLOC_MAX_KEYS; larger n is rejected with an
 *    error and nothing is launched.
 *  - The work is queued on `stream` (a cudaStream_t passed as void*, NULL for
 *    the default stream) and the call returns without waiting for it.
 *  - The first call on a device looks up the scratch array's device address
 *    (with that device current) and keeps it for later calls.
 *  - All calls share the one scratch array, so calls that can overlap on the
 *    GPU (other streams, other host threads) race: order them on one stream
 *    or synchronise between them.  The scratch needs no clearing between
 *    calls: every value in it is written before it is read.
 *  - Returns 0, or -1 with a message copied into error[0..error_capacity). */
#define SV_NOALLOC_MAX_KEYS (1u << 20)
#define SV_NOALLOC_SCRATCH_BYTES 16777984u
int sv_sort_pairs_noalloc(const uint32_t *keys, uint32_t *perm, uint64_t n, void *stream, char *error,
                          uint64_t error_capacity);

typedef struct sv_stats {
    uint64_t particles;
    uint64_t live_particles;
    uint64_t particle_blocks;   /* occupied 4^3 blocks in the last substep */
    uint64_t grid_blocks;       /* active grid blocks in the last substep */
    uint64_t fp64_svd;          /* particles that took the fp64 SVD, summed over substeps */
    uint64_t substeps;
    uint64_t device_bytes;      /* device memory held by the handle */
    uint64_t kernel_launches;   /* kernels launched by this handle so far */
    uint64_t sorts;             /* binning sorts run so far */
    uint64_t sort_interval;     /* current substeps between binning sorts */
    uint64_t tile_misses;       /* gathers that missed their block's shared tile (low 32 bits) */
    uint64_t graph_replays;     /* binning periods run as CUDA graph replays */
    uint64_t cta_per_sm;        /* CTAs per SM of the particle kernels other than the plain fused pass */
    uint64_t closure_learned;   /* snow/sand particle-substeps through the learned closure (low 32 bits) */
    uint64_t closure_fallbacks; /* of the learned mode's snow/sand particle-substeps: return-map fallbacks */
    uint64_t closure_mode;      /* 0 return maps, 1 learned closure */
    uint64_t adaptive_misses;   /* adaptive substeps whose speculative steps failed and were redone */
    uint64_t adaptive_split;    /* adaptive substeps queued in the split form */
    /* Conservation sums of the grid the last substep gathered from, taken
     * on the device in fp64 over its nodes in momentum form, before
     * momentum -> velocity (collider variants included): the total mass and
     * momentum that the P2G scattered.  Equal to the particles' sum of m and
     * m v + (the APIC term, which sums to zero) up to fp32 rounding of the
     * node values.  sv_step takes them on the last substep of each call
     * only (on every substep they would cost about 7 % of the substep's
     * time); a call that stops early leaves them 0.  The other stepping
     * calls take them on every substep. */
    double grid_mass;
    double grid_momentum[3];
    /* Device time of the plain fused particle pass (gather, advance,
     * scatter; its fp64 pass included), summed over its launches since
     * sv_create, and the number of those launches: from the start of the
     * pass's first CTA to the end of its last, read from the GPU's global
     * nanosecond timer by the kernels themselves, so CUDA-graph replays are
     * timed too.  Frame-input, learned-closure and adaptive passes are not
     * counted. */
    uint64_t pass_ns;
    uint64_t pass_count;
} sv_stats;

/* Adaptive time steps: CpuState::produce_next_state with
 * adaptive_time_steps = true (rust/crates/cpu/src/cpu_state.rs:146-197,
 * rust/crates/cpu/src/phase/limit_time_step.rs:25-224,
 * rust/crates/cpu/src/adaptive_time_step_state.rs:13-64).  Substeps run
 * while *time_inout < target_time; each takes the time step the reference's
 * AdaptiveTimeStepState allows at each phase (velocity, deformation, sound
 * speed and isolated-particle limits, the minimum over the last 11 pushed
 * limits, at most max_time_step).  The limit state persists in the handle
 * across calls, like the reference's.  *time_inout is advanced by the
 * substeps run.  Returns 0 (status bits as for sv_step), or -1 on a fatal
 * error, including a zero allowed time step (the reference's ZeroTimeStep).
 * sv_time_step_limits: the last substep's steps of external force, scatter
 * and advance, the velocity, deformation, sound and isolated limits, and the
 * step allowed now (FLT_MAX = no limit). */
int sv_step_adaptive(sv_handle *h, double *time_inout, double target_time, float max_time_step,
                     const float gravity[3], const volatile int32_t *cancel, uint32_t *status_out,
                     uint32_t *substeps_done);
int sv_time_step_limits(sv_handle *h, float out[8]);

/* ------------------------------------------------------------------ frame input and colliders
 * The inputs of frames a and b (rust/crates/xpu/src/frame_input.rs:33-65),
 * interpolated linearly inside the frame at the start of every substep
 * (rust/crates/cpu/src/phase/interpolate_input.rs:18-106):
 *   - gravity (replaces the gravity argument of sv_step / sv_step_adaptive);
 *   - particle goals: a particle whose flags carry HAS_GOAL in both frames
 *     gets v = (goal - x) / dt instead of gravity (external_force.rs:17-50);
 *     goal_flags_* [n], goal_positions_* [n][3] in the caller's particle
 *     order, NULL for no goals;
 *   - colliders: closed or open triangle meshes, up to 16 (the collider of
 *     each triangle in triangle_collider), vertices [n_vertices][3] at
 *     frames a and b, triangles [n_triangles][3], friction and damping per
 *     triangle.  Every substep runs the reference's Collide
 *     (rust/crates/cpu/src/phase/collide.rs:21-206) and keeps the grid's
 *     (node, collider bits) variants apart (update_grid_nodes.rs,
 *     meld_grid.rs).  leaf_size is the reference's InputConsts::leaf_size.
 * *_b arrays are ignored when has_b == 0 (frame b = a).  Substeps must start
 * inside `frame` (time * frames_per_second in [frame, frame + 1)), else
 * sv_step fails as the reference's WrongFrameLoaded; load the next frame
 * with another sv_set_frame_input.  NULL removes the frame input.  Not for
 * batched handles. */
typedef struct sv_frame_input {
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
} sv_frame_input;

int sv_set_frame_input(sv_handle *h, const sv_frame_input *in);
/* Simulation time of the state (CpuState::time); sv_step advances it by dt
 * per substep, sv_step_adaptive by its steps. */
int sv_set_time(sv_handle *h, double time);
int sv_get_time(sv_handle *h, double *time);

/* Whether sv_step runs whole binning periods as CUDA graphs (default on;
 * off, and while profiling, every kernel is launched directly). */
int sv_set_graphs(sv_handle *h, int enable);
/* sv_consts::host_transfer for the handle's later downloads; *direct (if
 * not NULL) tells whether the direct path is now in use. */
int sv_set_host_transfer(sv_handle *h, uint32_t mode, uint32_t *direct);
/* Maps the pages of `count` host arrays (bytes[k] bytes at arrays[k]) for a
 * later direct sv_download into them, without changing their contents.  A
 * page the GPU writes first is mapped through a device-side fault, much
 * slower; freshly allocated arrays can be prepared from another thread while
 * sv_step runs.  Touches no handle. */
int sv_prepare_host(void *const *arrays, const uint64_t *bytes, uint32_t count);
int sv_get_stats(sv_handle *h, sv_stats *out);

/* Addition: picks the substeps between binning sorts (2, 4, 6, 8, 12, 16, at
 * the handle's CTAs per SM) and then the CTAs per SM of the particle kernels
 * (8, 16, 32, 64, at the chosen interval) by timing each candidate from a
 * snapshot of the current state: two binning periods of
 * warm-up (first scatter, graph capture, steady binning), then three repeats
 * of at least max(substeps_per_trial, 48) substeps, ranked by the median
 * repeat.  The handle's own configuration is a candidate and is kept unless
 * another is more than 2 % faster.  The state is restored afterwards.  The
 * chosen values are written to the out pointers when not NULL.  One launch
 * covers all scenes of a batched handle, so these settings apply to all of
 * them alike.  The plain fused pass of sv_step always runs as one resident
 * wave taking segments from a queue; the CTAs-per-SM choice applies to the
 * other particle passes (standalone scatter, adaptive, frame-input and
 * learned forms). */
int sv_autotune(sv_handle *h, float dt, const float gravity[3], uint32_t substeps_per_trial,
                uint32_t *sort_interval_out, uint32_t *cta_per_sm_out);

/* Runs the handle's work on a caller-owned CUDA stream (a cudaStream_t passed
 * as void*; NULL returns to the handle's own stream).  The previous stream is
 * synchronised first; the caller keeps ownership of its stream. */
int sv_set_stream(sv_handle *h, void *stream);

/* Per-kernel timing with CUDA events on the handle's stream (off by
 * default).  sv_profile_report writes a JSON object
 * {"kernel": {"launches": L, "ms": T}, ...} and returns its length. */
int sv_set_profiling(sv_handle *h, int enable);
int sv_profile_report(sv_handle *h, char *buffer, uint64_t capacity);

/* ------------------------------------------------------------------ learned closure
 * Addition (not in the reference): a learned return map for snow and sand,
 * replacing rust/crates/cpu/src/phase/advance_particles.rs:48-71 when
 * switched on.  An MLP maps the principal Hencky strains and the material
 * parameters (normalised) to the plastic correction of the strains and the
 * principal Kirchhoff stress of the projected state (normalised), evaluated
 * on the tensor cores.
 * Network: x (16; input 15 is reserved and read as 0) -> 4 hidden layers of
 * width 64 with SiLU (bf16 operands, fp32 accumulation) -> an fp32 head of
 * 8 outputs, the first 6 used.  Parameters are an fp32 vector of
 * sv_mlp_param_count() = 14088 values: W1[64][16], b1[64], W2[64][64], b2,
 * W3[64][64], b3, W4[64][64], b4, W5[8][64], b5[8] (row-major, out x in).
 *
 * The two entry points below are stateless inspection calls on host
 * buffers (they allocate device memory per call) used to check the kernels:
 *   sv_mlp_forward: y[n][8] = network(x[n][16]);
 *   sv_mlp_grad:    loss = sum_r w[r] sum_{o<6} (y[r][o] - t[r][o])^2 / n
 *                   (t[n][8]), its gradient with respect to the parameters
 *                   into grad[], and y[n][8] when y is not NULL. */
int sv_mlp_param_count(void);
int sv_mlp_forward(const float *params, const float *x, uint64_t n, float *y);
int sv_mlp_grad(const float *params, const float *x, const float *t, const float *w, uint64_t n, float *y,
                float *grad, float *loss);

/* The closure of a handle's snow and sand particles.
 *
 * In sv_step with the learned closure on, a snow/sand particle's principal
 * stretches come from a closed-form eigen-decomposition of F^T F; the yield
 * test (closed form) keeps elastic particles on their stretches, and the
 * network decides the yielding ones.  A yielding particle outside the
 * training hull, or whose network stress disagrees with the closed-form
 * stress of its projected stretches by more than 1e-3 mu h, takes the SVD +
 * return map.
 *
 * sv_closure_harvest: adds up to max_samples trial deformation gradients
 *   F + dt C F of the live snow/sand particles of the current state (states
 *   the plain solver produced) to the handle's training pool (at most 2^26);
 *   with augment > 0 half of them are multiplied by I + augment R, R
 *   symmetric with entries in [-1, 1).  *total_out = pool size.
 * sv_closure_harvest_from: the same from the current state of another
 *   handle `src` into h's pool (the samples carry their material
 *   parameters), so that one pool gathers several workloads' states.
 * sv_closure_train: labels the pool with the fp64 SVD + return map, keeps
 *   the yielding samples, records the range of their features (the hull)
 *   and the normalisation of inputs and outputs, and runs `iterations` Adam
 *   steps (minibatches of `batch`, 0 = 65536; learning rate lr with a cosine
 *   decay to 1 %) on the GPU from the current weights (He-initialised from
 *   `seed` on the first call).  *loss_out = mean squared error (normalised
 *   units) over the yielding samples afterwards.
 * sv_closure_set_material_ranges: from the next sv_closure_train on, each
 *   sample keeps its harvested deformation and shear modulus but is labelled
 *   with a Poisson's ratio drawn uniformly from [nu_lo, nu_hi] and, for
 *   sand, a friction angle from [phi_lo_deg, phi_hi_deg] (degrees), so that
 *   the pool covers those material ranges evenly whichever scenes the
 *   samples came from.  All four 0: the harvested materials (default).
 * sv_closure_copy: gives dst the trained network, hull and normalisation of
 *   src (e.g. trained on a batched handle, used on another).
 * sv_closure_set_mode: 0 = return maps (default), 1 = learned closure in
 *   sv_step (needs a trained network).
 * sv_closure_evaluate: on the trial F of the current state, out[0] / out[1]
 *   = relative Kirchhoff-stress error (Frobenius, over all snow/sand
 *   particles) of the learned closure (with its fallbacks) / of the fp32
 *   return map, both against the fp64 return map; out[2] / out[3] the same
 *   for the projected F; out[4] particles evaluated, out[5] fallbacks,
 *   out[6] |tau_fp64|, out[7] |F_fp64|, out[8] particles handed to the
 *   network (yielding, inside the hull), out[9] of which failed the
 *   residual check, out[10] / out[11] the parts of out[0] from the
 *   particles the network decided / from the elastic ones (out[0]^2 =
 *   out[10]^2 + out[11]^2 + the fallbacks' part).
 * sv_closure_phase_times: per-phase costs on the trial F of the current
 *   state (mean of 5 launches, ms): out[0] SVD + return map + stress (the
 *   plain path), out[1] eigen-decomposition + yield test + closed-form
 *   stress (the learned path without its network), out[2] the network over
 *   every snow/sand particle, out[3] snow/sand particles, out[4] of which
 *   yield inside the hull, out[5] the network over those only.
 * sv_closure_pool: the pool size and the yielding samples of the last
 *   sv_closure_train (0 before).
 * sv_closure_get_pool: rows [first, first + count) of the normalised
 *   training pool of the last sv_closure_train (the yielding samples in
 *   their shuffled order: X[count][16], Y[count][8]) and the hull (80
 *   floats: lo[16], hi[16], xm[16], xs[16], ym[8], ys[8]); NULL skips one.
 * sv_closure_get_params: the fp32 master weights (sv_mlp_param_count()). */
int sv_closure_harvest(sv_handle *h, float dt, uint32_t max_samples, float augment, uint32_t seed,
                       uint64_t *total_out);
int sv_closure_harvest_from(sv_handle *h, sv_handle *src, float dt, uint32_t max_samples, float augment,
                            uint32_t seed, uint64_t *total_out);
int sv_closure_train(sv_handle *h, uint32_t iterations, uint32_t batch, float lr, uint32_t seed, float *loss_out);
int sv_closure_set_mode(sv_handle *h, int mode);
int sv_closure_copy(sv_handle *dst, sv_handle *src);
int sv_closure_set_material_ranges(sv_handle *h, float nu_lo, float nu_hi, float phi_lo_deg, float phi_hi_deg);
int sv_closure_phase_times(sv_handle *h, float dt, double out[6]);
int sv_closure_pool(sv_handle *h, uint64_t *pairs, uint64_t *yielding);
int sv_closure_get_pool(sv_handle *h, uint64_t first, uint64_t count, float *X, float *Y, float *hull);

/* No counterpart in the reference: a failure-detection check.  Runs the
 * learned closure's bounded tensor-core wait on a CTA whose MMA commit is
 * never issued, with a limit of max_cycles SM clocks (1 .. 4e9): the kernel
 * gives up, frees its TMEM and raises the closure's timeout counter, as a
 * particle pass whose MMA never completed would; the next sv_step then fails
 * with "a tensor-core wait of the learned closure timed out".  The GPU
 * context stays usable.  Returns 0 once the kernel has returned. */
int sv_debug_closure_wait_timeout(sv_handle *h, uint64_t max_cycles);
int sv_closure_evaluate(sv_handle *h, float dt, double out[12]);
int sv_closure_get_params(sv_handle *h, float *params);

/* ---- Frame files and the frame cache ----------------------------------
 *
 *   reference                                                  | entry point here
 *   -----------------------------------------------------------+-----------------------------
 *   IoState::write / IoState::read (file_frame/src/io_state.rs:31-75),
 *     magic and version (file_util/src/lib.rs:27-99)            | sv_frame_write, sv_frame_read
 *   StoreThread::new / store / check / drop
 *     (cache/src/store_thread.rs:27-110), frame_path (cache/src/util.rs:9-11) |
 *                                                              | sv_cache_open, sv_cache_store,
 *                                                              | sv_cache_store_frame, sv_cache_check,
 *                                                              | sv_cache_flush, sv_cache_close
 *
 * A frame file is the reference's: 32 magic bytes, 64 version bytes (the
 * version string, zero padded; the reader demands the same string), then
 * IoState { time, particles, grid_nodes } serialised by bincode 1.3.3 with
 * its default options (little endian, fixed-width integers, u64 sequence
 * lengths, u32 enum variant indices, u8 Option tags).  `version` NULL means
 * SV_FRAME_VERSION, the reference's file_util crate version.
 *
 * sv_frame describes one IoState.  ParticleParameters (particles.rs:55-90) is
 * spread into arrays: viscosity is Some where flags has SV_USE_VISCOSITY,
 * the variant is Fluid { exponent, bulk_modulus } where flags has
 * SV_IS_FLUID and Solid { mu, lambda, sand_alpha } otherwise, sand_alpha
 * Some where flags has SV_USE_SAND_ALPHA.  (The file has no room for this
 * library's additional models: it stores their mu and lambda as a Solid.)
 * Unused arrays may be NULL when writing (their entries are written as 0).
 * node_* arrays describe GridNodes (grid_nodes.rs:10-15) when has_grid.
 *
 * sv_frame_read: with every array pointer NULL it fills time, n, has_grid
 * and n_nodes only; otherwise n and n_nodes must equal the file's and every
 * array is filled (the parameter arrays with 0 where the variant or the
 * Option leaves them unused). */
#define SV_FRAME_VERSION "0.3.4"
typedef struct sv_frame {
    double time;
    uint64_t n;
    uint32_t *flags;
    float *mass, *initial_volume;
    float *viscosity_dynamic, *viscosity_bulk;
    float *mu, *lambda, *sand_alpha;
    int32_t *exponent;
    float *bulk_modulus;
    float *elastic_energies;
    uint32_t *collider_bits;
    float *positions, *position_gradients, *velocities, *velocity_gradients, *initial_positions;
    uint32_t has_grid;
    uint64_t n_nodes;
    int32_t *node_ids;
    uint32_t *node_collider_bits;
    float *node_masses, *node_velocities;
} sv_frame;

int sv_frame_write(const char *path, const sv_frame *frame, const char *version, uint64_t *bytes_written);
int sv_frame_read(const char *path, const char *version, sv_frame *frame);

/* The frame cache: frames go to <dir>/frame_%05u.bin, numbered from
 * first_frame, by a writer thread.  `statics` gives what the substep never
 * changes and every frame repeats: n, the parameter arrays and
 * initial_positions, in the original particle order (NULL arrays are
 * written as 0; the stored flags select the variants as above).
 *
 * sv_cache_store queues a device snapshot of the handle's current state
 * (and, when store_grid, of the grid its last substep gathered, with the
 * collider variants) on the handle's stream, and its copy to pinned host
 * memory on the cache's own stream, and returns without waiting.  The
 * handle's next kernels wait only for the device snapshot; the host copy
 * overlaps them.  The writer thread waits for the host copy, restores the
 * original particle order and writes the file.  At most `depth` frames are
 * in flight (each holds a device and a pinned copy of the state); a further
 * store waits for the oldest.  sv_cache_store_frame queues a copy of a host
 * frame.
 * sv_cache_check returns -1 with the message once the writer has failed
 * (StoreThread::check); sv_cache_flush waits until every queued frame is
 * on disk; sv_cache_info reports frames written and their bytes
 * (total_bytes_on_disk, available_frames).  sv_cache_close flushes and
 * ends the thread. */
typedef struct sv_cache sv_cache;
int sv_cache_open(const char *dir, const char *version, const sv_frame *statics, uint32_t first_frame, uint32_t depth,
                  sv_cache **out);
int sv_cache_store(sv_cache *c, sv_handle *h, int store_grid);
int sv_cache_store_frame(sv_cache *c, const sv_frame *frame);
int sv_cache_check(sv_cache *c);
int sv_cache_flush(sv_cache *c);
int sv_cache_info(sv_cache *c, uint64_t *frames_written, uint64_t *bytes_written);
int sv_cache_close(sv_cache *c);

#ifdef __cplusplus
}
#endif
#endif
