// sv_internal.h -- device state of one handle and the launchers of the
// substep kernels (sv_substep.cu), shared with the C ABI (sv_api.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/squishy_volumes_cuda.h"
#include "sv_math.cuh"

namespace sv {

// Particle flag bits (file_frame/src/particles.rs:21-33) live in the low 8
// bits of the packed word; the material index in the upper 24.
constexpr uint32_t FLAG_MASK = 0xFFu;
constexpr uint32_t MATERIAL_SHIFT = 8;
constexpr uint32_t MAX_MATERIALS = 1u << 24;
constexpr uint32_t SENTINEL_KEY = 0xFFFFFFFFu;

// Device status word bits.  Any bit in STOP_MASK makes every later kernel of
// the run leave the particle state untouched.
constexpr uint32_t ST_CAPACITY = SV_STATUS_CAPACITY_EXCEEDED;
constexpr uint32_t ST_INVERTED = SV_STATUS_PARTICLE_INVERTED;
constexpr uint32_t ST_OUT_OF_GRID = 1u << 4;  // a live particle left the block index
constexpr uint32_t ST_MOVED_FAR = 1u << 5;    // a particle left the blocks claimed at binning
constexpr uint32_t ST_TIME_REACHED = 1u << 6; // adaptive steps: the target time is reached
constexpr uint32_t ST_ZERO_DT = 1u << 7;      // adaptive steps: the allowed time step is 0
constexpr uint32_t ST_VARIANT_FULL = 1u << 9; // the collider-variant table or a node's variant slots are full
constexpr uint32_t ST_WRONG_FRAME = 1u << 10; // a substep's time lies outside the loaded frame input
constexpr uint32_t ST_SAND_MU = SV_STATUS_SAND_INVALID_MU;  // sand with mu <= 0 under compression
constexpr uint32_t STOP_MASK = ST_CAPACITY | ST_INVERTED | ST_OUT_OF_GRID | ST_MOVED_FAR | ST_TIME_REACHED | ST_ZERO_DT |
                               ST_VARIANT_FULL | ST_WRONG_FRAME | ST_SAND_MU;

// Device counters (one array so one copy reads them all).
enum Counter : int {
    C_STATUS = 0,
    C_NSEG = 1,      // particle blocks (segments) of the last binning
    C_NSLOT0 = 2,    // grid blocks claimed in block map 0
    C_NSLOT1 = 3,    // grid blocks claimed in block map 1
    C_NLIVE = 4,     // live particles at the last binning (segments cover [0, n_live))
    C_SUBSTEPS = 5,  // substeps completed
    C_FP64 = 6,      // particles that took the fp64 SVD
    C_STOP = 7,      // STOP_MASK bits latched for the kernels that follow
    C_FALLBACK = 8,  // gathers that missed their segment's shared tile
    C_CLOSURE = 9,       // snow/sand particle-substeps through the learned closure
    C_CLOSURE_FB = 10,   // snow/sand particle-substeps that fell back to the return map
    C_CLOSURE_ERR = 11,  // a tensor-core wait of the learned closure gave up
    C_CTA_DONE = 12,     // CTAs of a self-latching particle pass that have finished
    C_TRANSFER_BAD = 13, // a direct download met an original index out of range or repeated
    C_ADT_MISS = 14,     // adaptive substeps whose speculative steps failed (fused form)
    C_SUMS_AT = 15,      // the grid updates take the fp64 conservation sums from this substep on
    C_DEFER = 16,        // particles of this substep's fused pass left for its fp64 pass (defer_list)
    C_SEGQ = 17,         // next segment for the fused pass's CTAs to take
    C_COUNT = 18,
};

// One side of the particle state (ping-pong).  Structure of arrays: pos and
// vel as float4 so one 16-byte load brings a vector and its companion word;
// the two 3x3 matrices as nine planar float arrays each (fully coalesced).
struct ParticleArrays {
    float4 *pos;     // fp32 form: x, y, z, packed flags|material
                     // cell form: offset x, y, z in [0,1) cell units, packed
    int4 *cell;      // cell form only: cell x, y, z, unused
    float4 *vel;     // vx, vy, vz, plastic J (snow)
    float *C;        // [9][n] velocity gradient, column-major element planes
    float *F;        // [9][n] position gradient
    float *energy;   // [n]
    uint32_t *orig;  // [n] original particle index (the reference's sort_map)
    // collider bits (allocated once a frame input is set): the bits in
    // effect for the next gather (after the pending scatter's Collide) and
    // the bits after the last completed substep
    uint32_t *cbits = nullptr, *cbits_done = nullptr;
};

struct GridLayout {
    int32_t origin[3];  // node/cell index of local cell 0
    int32_t nb[3];      // blocks per axis
    uint64_t total_blocks;
    float dx;
    float domain_min[3], domain_max[3];
    double dmin_cells[3], dmax_cells[3];  // domain in cell units (cell form cull)
    int32_t ground_mode, ground_axis;
    float ground_height;
    uint32_t position_form;
    uint32_t svd_policy;
    int key_bits;
};

// Grid node velocity from its momentum (meld_grid.rs:61-66: v = p / m, or 0
// when m <= 0), then the boundary plane (an addition, not in the reference)
// at global node (x, y, z).  Shared by the grid update and the variant meld.
__host__ __device__ inline float4 node_velocity(float4 g, int x, int y, int z, const GridLayout &L) {
    const float m = g.w;
    float vx = 0.f, vy = 0.f, vz = 0.f;
    if (m > 0.f) vx = g.x / m, vy = g.y / m, vz = g.z / m;
    if (L.ground_mode != 0) {
        const int node[3] = {x, y, z};
        if ((float)node[L.ground_axis] * L.dx <= L.ground_height) {
            if (L.ground_mode == 1) vx = vy = vz = 0.f;
            else if (L.ground_axis == 0) vx = fmaxf(vx, 0.f);
            else if (L.ground_axis == 1) vy = fmaxf(vy, 0.f);
            else vz = fmaxf(vz, 0.f);
        }
    }
    return make_float4(vx, vy, vz, m);
}

struct KernelTimer {
    std::vector<std::pair<std::string, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::map<std::string, std::pair<uint64_t, double>> totals;  // launches, ms
};

}  // namespace sv

struct sv_handle {
    sv::GridLayout layout;
    uint64_t n = 0;
    int cur = 0;  // particle side holding the state
    sv::ParticleArrays side[2] = {};
    sv::Material *materials = nullptr;
    uint32_t n_materials = 0;
    std::vector<sv::Material> host_materials;
    // independent scenes sharing the handle (one unless created batched)
    sv::SceneInfo *scenes = nullptr;
    std::vector<sv::SceneInfo> host_scenes;
    std::vector<uint64_t> scene_first;  // first particle of each scene (+ total at the end)
    bool batched = false;

    uint32_t *keys = nullptr;         // [n] binning keys in device order (valid when keys_valid)
    bool keys_valid = false;
    uint32_t *sorted_keys = nullptr;  // [n]
    uint32_t *perm = nullptr;         // [n] device slot of each sorted position
    uint32_t *defer_list = nullptr;   // [n] sorted positions the fused pass left for its fp64 pass
    uint32_t kind_set = 0x1F;         // 1 << kind of every material in use
    void *sort_temp = nullptr;
    size_t sort_temp_bytes = 0;

    uint32_t *seg_start = nullptr;  // [n + 1]
    uint32_t *seg_block = nullptr;  // [n]
    uint32_t *tile_counts = nullptr;
    void *scan_temp = nullptr;

    // Two grids (the one gathered from and the one scattered into) and two
    // block maps (dense block index -> slot), swapped when the binning is redone.
    int32_t *blockmap[2] = {nullptr, nullptr};
    uint32_t *active[2] = {nullptr, nullptr};
    float4 *grid[2] = {nullptr, nullptr};  // [capacity * 64] (px, py, pz, m) -> (vx, vy, vz, m)
    uint64_t capacity = 0;
    int gcur = 0;      // grid holding the pending scatter (momentum form)
    int map_cur = 0;   // block map of grid[gcur]
    int map_next = 0;  // block map of the grid being scattered into
    int vel_side = -1, vel_map = 0;  // grid with the last velocities (for sv_download_grid)

    // The pending grid is the scatter of the current state for the next
    // substep, made with these dt and gravity.
    bool pending_valid = false;
    float pending_dt = 0.f;
    float pending_g[3] = {0.f, 0.f, 0.f};
    bool need_perm = true;   // state not yet in the order of the last binning
    uint32_t since_sort = 0;
    uint32_t sort_interval = 8;  // current interval between binning sorts
    uint32_t max_interval = 8;
    bool adaptive_interval = true;

    // Deterministic P2G (sv_consts::deterministic_p2g): binning keys in
    // original-index order, the sort's original indices, per sorted particle
    // records (4 float4), per segment cell starts [65] and the segment of
    // each grid slot; det_seg_cap segments and slots fit.
    bool deterministic = false;
    uint32_t *det_kbo = nullptr, *det_orig = nullptr, *det_cstart = nullptr;
    int32_t *det_slot_seg = nullptr;
    float4 *det_rec = nullptr;
    uint64_t det_seg_cap = 0;
    // device [2][4] fp64 sums (mass, px, py, pz) of grid[0] and grid[1] in
    // momentum form, taken by the grid update; zeroed where a grid is cleared
    double *grid_sums = nullptr;
    uint64_t *pass_timer = nullptr;     // device [3]: start of the current fused pass, ns summed, passes (globaltimer)
    uint32_t *counters = nullptr;       // device [C_COUNT]
    uint32_t *host_counters = nullptr;  // pinned mirror

    // Upload and download by kernels that access the caller's pageable host
    // arrays (sv_transfer.cu), where the device can; else staged copies.
    bool direct_host = false;
    uint32_t *inv = nullptr;  // [n] slot of each original particle (direct download)
    void *arena = nullptr;    // the one allocation the fixed-size device buffers are carved from
    // C_STOP will hold the stop bits of every kernel queued so far (the last
    // status-setting launch was a latch or a self-latching particle pass)
    bool stop_latched = false;

    cudaEvent_t wait_event = nullptr;   // marks the counter copy the substep loops poll for
    cudaStream_t stream = nullptr;      // stream all work is queued on
    cudaStream_t own_stream = nullptr;  // the handle's own stream
    uint64_t device_bytes = 0;
    uint64_t fp64_total = 0;
    uint64_t substeps_total = 0;
    uint64_t launches = 0;  // kernels launched by this handle
    uint64_t sorts = 0;     // binning sorts run

    // host-side copies of what the substep never changes: the collider bits
    // the particles were created with (empty when all are 0)
    std::vector<uint32_t> collider_bits;

    bool profiling = false;
    sv::KernelTimer timer;

    // CTAs per SM of the particle kernels' grid (tuned by sv_autotune).  Five
    // are resident per SM; the rest wait in the hardware block scheduler,
    // which balances segments of uneven size better than a fixed stride.
    uint32_t cta_per_sm = 32;

    // CUDA graphs of one binning period (a binning substep and the substeps
    // up to the next binning), keyed by everything their launches bake in.
    // A run of `count` substeps captured from host state (cur, gcur, map_cur,
    // map_next, since_sort, keys_valid, need_perm, stop_latched) with the
    // binning interval `period`: whole binning periods, or the part of one
    // that a call's substep count leaves.
    struct GraphKey {
        int cur, gcur, map_cur, map_next;
        uint32_t period, since_sort, count;
        bool keys_valid, need_perm, stop_latched;
        float dt, g[3];
        bool operator<(const GraphKey &o) const {
            return std::tie(cur, gcur, map_cur, map_next, period, since_sort, count, keys_valid, need_perm, stop_latched, dt,
                            g[0], g[1], g[2]) < std::tie(o.cur, o.gcur, o.map_cur, o.map_next, o.period, o.since_sort,
                                                         o.count, o.keys_valid, o.need_perm, o.stop_latched, o.dt, o.g[0],
                                                         o.g[1], o.g[2]);
        }
    };
    struct GraphState {  // host-side state after the period
        cudaGraphExec_t exec = nullptr;
        int cur, gcur, map_cur, map_next, vel_side, vel_map;
        bool keys_valid, need_perm, stop_latched;
        uint32_t since_sort;
        uint64_t launches, sorts;
    };
    std::map<GraphKey, GraphState> graphs;
    std::set<GraphKey> partial_seen;  // partial periods run once directly, captured when they recur
    bool use_graphs = true;
    uint64_t graph_launches = 0;  // graph replays issued

    // Adaptive time steps (adaptive::State in device memory, sv_adaptive.cuh);
    // adaptive_active while sv_step_adaptive runs.
    void *adt = nullptr;
    void *adt_backup = nullptr;  // the state at the start of the running substep
    bool adaptive_active = false;
    // the particle state is still the one the last sv_step_adaptive left, so
    // the force limits its last advance reduced (adaptive::State::force_ready)
    // still apply; any other pass that writes particles clears it
    bool force_limits_valid = false;
    // the next adaptive substep queues k_limits_force: the first of a call and
    // the redo of a stopped one, whose state may predate any advance
    bool limits_pass_pending = false;
    // batches of adaptive substeps still to run in the split form, after a
    // batch whose speculative steps failed too often
    uint32_t adt_split_batches = 0;
    uint64_t adt_split_substeps = 0;  // adaptive substeps queued in the split form

    // Simulation time of the completed state (the reference's CpuState::time),
    // used to interpolate the frame input.
    double time = 0.0;

    // Frame input and colliders (sv_collide.cuh, set by sv_set_frame_input).
    bool fin_active = false;
    uint32_t fin_fps = 24, fin_frame = 0;
    bool fin_has_b = false;
    float fin_g_a[3] = {0, 0, 0}, fin_g_b[3] = {0, 0, 0};
    uint32_t fin_nv = 0, fin_nt = 0;
    float *fin_scalars = nullptr;    // device: gravity[3], factor
    uint32_t *fin_goal_both = nullptr;
    float *fin_goal_a = nullptr, *fin_goal_b = nullptr;
    uint32_t *fin_tri = nullptr, *fin_tri_col = nullptr, *fin_opp = nullptr;
    float *fin_va = nullptr, *fin_vb = nullptr, *fin_vvel = nullptr;
    float *fin_fr_a = nullptr, *fin_fr_b = nullptr, *fin_dm_a = nullptr, *fin_dm_b = nullptr;
    uint32_t *fin_vt_start = nullptr, *fin_vt_list = nullptr;  // vertex -> triangles (CSR)
    uint32_t *fin_leaf_start = nullptr, *fin_leaf_list = nullptr;
    int32_t fin_leaf_lo[3] = {0, 0, 0}, fin_leaf_dim[3] = {0, 0, 0};
    float fin_leaf_size = 1.f;
    float *fin_vpos = nullptr, *fin_vnorm = nullptr, *fin_tnorm = nullptr, *fin_fric = nullptr, *fin_damp = nullptr;
    // collider-variant tables (two, swapped with the grids)
    unsigned long long *var_key[2] = {nullptr, nullptr};
    uint32_t *var_bits[2] = {nullptr, nullptr};
    float4 *var_acc[2] = {nullptr, nullptr}, *var_vel[2] = {nullptr, nullptr};
    uint32_t var_cap = 0;

    // Learned stress closure of snow and sand (sv_closure.cu).
    int closure_mode = 0;  // 0 return maps (SVD), 1 learned closure
    bool cl_trained = false;
    float *cl_params = nullptr, *cl_grad = nullptr, *cl_m = nullptr, *cl_v = nullptr;  // fp32 master + Adam
    uint8_t *cl_img = nullptr;      // packed bf16 weight image
    void *cl_hull = nullptr;        // closure::Hull of the training features
    float *cl_samples = nullptr;    // [cl_cap][CL_SAMPLE]: trial F, plastic J, material kind and parameters
    uint64_t cl_n = 0, cl_cap = 0;  // harvested samples
    float *cl_X = nullptr, *cl_Y = nullptr;  // normalised features and targets of the yielding samples
    uint64_t cl_xy_cap = 0;
    int cl_step = 0;                // Adam steps taken
    uint64_t cl_yielding = 0;       // yielding (weighted) samples of the last labelling
    int cl_ranges_on = 0;           // labels draw nu / the friction angle from cl_ranges
    float cl_ranges[4] = {0, 0, 0, 0};  // nu_lo, nu_hi, phi_lo, phi_hi (radians)
    float *cl_loss = nullptr;       // device scalar
    uint32_t *cl_err = nullptr;     // device flag
    uint64_t *cl_count = nullptr;   // device counter of the harvest
    double *cl_sums = nullptr;      // device sums of the error evaluation
};

namespace sv {

// Launchers (sv_substep.cu).  All run on h->stream and read counts from
// device memory, so a substep needs no host synchronisation.
cudaError_t launch_keys(sv_handle *h);
cudaError_t launch_sort_and_segments(sv_handle *h);
cudaError_t launch_activate(sv_handle *h, int which);
cudaError_t launch_clear(sv_handle *h, int grid_side, int which);
// latches the status word's stop bits for the kernels that follow
cudaError_t launch_latch(sv_handle *h);
cudaError_t launch_p2g(sv_handle *h, float dt, float3 gravity);
// deterministic P2G: the binning by (cell, original index), then the
// records, cell tables and fixed-order node gather into grid[gcur]
cudaError_t launch_det_binning(sv_handle *h);
cudaError_t launch_det_p2g(sv_handle *h, float dt, float3 gravity);
// latch = false: the stop bits are already latched (by the particle pass
// before it, or by the binning's block claims)
cudaError_t launch_grid_update(sv_handle *h, bool clear_next, bool latch = true);
// Without a frame input the pass latches the stop bits and counts the
// substep itself (its last CTA), so no k_latch / k_finish launches follow.
cudaError_t launch_g2p2g(sv_handle *h, float dt, float3 gravity, bool write_keys, bool use_perm);
// adaptive time steps (the unfused substep)
// k_dt_force, after k_limits_force when `reduce` (the pass returns at once
// when the last advance reduced the force limits already)
cudaError_t launch_limits_force(sv_handle *h, bool reduce);
cudaError_t launch_g2p_only(sv_handle *h);
cudaError_t launch_advance(sv_handle *h);
// The fused pass of an adaptive substep (no frame input): advance at the
// speculative step, scatter of the next substep at its speculative steps,
// the checks, the redo of either when a limit bound, and k_adaptive_finish
cudaError_t launch_g2p2g_adaptive(sv_handle *h, float3 g, bool write_keys, bool use_perm);
// latches the stop bits and keeps the adaptive state for a redo
cudaError_t launch_adaptive_begin(sv_handle *h);
// frame input: interpolation at `time` (adaptive: the device time), the
// gather + advance without the scatter of the next substep, clearing the
// variant table the next scatter fills
cudaError_t launch_interpolate(sv_handle *h, double time);
cudaError_t launch_g2p_advance(sv_handle *h, float dt);
cudaError_t launch_clear_variants(sv_handle *h, int which);

// Reads the device counters into h->host_counters (waits for the stream);
// -1 with the last error set on failure.
int refresh_counters(sv_handle *h);

// ---- direct host transfers (sv_transfer.cu) ----
// whether the current device reads and writes pageable host memory
bool pageable_access();
// side 0 from the caller's arrays (h->scenes uploaded first); waits for it
cudaError_t upload_direct(sv_handle *h, const sv_particles *ps, uint32_t n_scenes, const uint64_t *first,
                          const uint32_t *mat_index);
// the current side into the caller's arrays in the original order; -1 with
// the last error set on failure
// particles first .. first + count (original order) into the caller's arrays
int download_direct(sv_handle *h, sv_particles *out, uint64_t first, uint64_t count);

// ---- host copies of the device state (sv_cache.cu) ----
// One particle side copied to the host in device (binning) order.
struct HostParticles {
    uint64_t n = 0;
    float4 *pos = nullptr, *vel = nullptr;
    int4 *cell = nullptr;                                  // cell form only
    float *C = nullptr, *F = nullptr, *energy = nullptr;   // C and F as [9][n] element planes
    uint32_t *orig = nullptr, *cbits = nullptr;            // cbits: with a frame input only
};
// What turning such a copy back into the reference's layout needs from the
// handle (copied, so a queued copy outlives changes to the handle).
struct UnpackInfo {
    bool cell = false;
    double dx = 0.0;
    std::vector<SceneInfo> scenes;
    std::vector<Material> materials;
    bool stepped = false;                      // a substep ran: Collide cleared the live particles' bits
    const uint32_t *initial_bits = nullptr;    // collider bits the particles were created with
    std::vector<uint32_t> initial_bits_copy;   // owned copy (own_bits)
};
// Queues the copies of the current particle side into `dst` (n elements
// each; cell and cbits only where the handle has them) on h->stream.
cudaError_t copy_particles_async(sv_handle *h, const HostParticles &dst);
// own_bits: copy the handle's initial collider bits instead of pointing at them
UnpackInfo unpack_info(const sv_handle *h, bool own_bits);
// Original particle order (the reference's reverse_sort_map restore,
// cpu_state.rs:71-104); false on a corrupt original index.
bool unpack_particles(const HostParticles &src, const UnpackInfo &u, sv_particles *out);

// Grid nodes with mass > 0, keyed (node, collider bits).
struct GridNode {
    int32_t id[3];
    uint32_t bits;
    float4 v;  // vx, vy, vz, m
};
// The grid gathered by the last substep (and its collider variants).
struct HostGrid {
    uint64_t slots = 0;
    uint32_t *active = nullptr;  // [slots]
    float4 *grid = nullptr;      // [slots * 64]
    uint64_t var_cap = 0;        // 0: no variants
    unsigned long long *var_key = nullptr;
    uint32_t *var_bits = nullptr;
    float4 *var_vel = nullptr;
};
// sizes of that grid from the last counter read-back (the stream idle)
void grid_sizes(const sv_handle *h, uint64_t &slots, uint64_t &var_cap);
cudaError_t copy_grid_async(sv_handle *h, const HostGrid &dst);
// sorted like the reference's GridKey (node id, then collider bits)
std::vector<GridNode> grid_nodes(const HostGrid &g, const GridLayout &L);

// Per-kernel timing hooks.
void timer_begin(sv_handle *h, const char *name, cudaEvent_t *start);
void timer_end(sv_handle *h, const char *name, cudaEvent_t start);

int sm_count();

// Sets the string sv_last_error_string returns (this thread).
void set_last_error(const std::string &msg);

// Drops the handle's captured CUDA graphs (their launches are stale).
void drop_graphs(sv_handle *h);

// Frees the learned closure's device buffers (sv_closure.cu).
void free_closure(sv_handle *h);

// Frees the frame input, the collider bits and the variant tables (sv_frame.cu).
void free_frame(sv_handle *h);

}  // namespace sv
