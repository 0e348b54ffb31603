// sv_substep.cu -- the MPM substep on the GPU.
//
// Reference: Squishy Volumes rust/crates/cpu, one pass of the phase cycle
// (cpu/src/phase/mod.rs:27-41) with adaptive time steps off:
//   Sort -> ExternalForce -> UpdateGridNodes -> ScatterMomentum -> MeldGrid
//   -> CollectVelocity -> AdvanceParticles -> CullParticles.
//
// GB300 design.  Substep t+1's scatter is fused into substep t's gather, so
// each particle is read once and written once per substep and its 3x3 SVD is
// computed once:
//
//   grid      momentum -> velocity on grid G_t (MeldGrid, meld_grid.rs:16-69,
//             plus the optional boundary plane), and clears G_t+1
//   g2p2g     one CTA per 4^3 particle block ("segment"): the 8^3-node velocity
//             tile of G_t staged in shared memory; thread per particle: gather
//             v and C (collect_velocity.rs:19-75), advance x and F, plasticity
//             and energy (advance_particles.rs:17-93), cull
//             (cull_particles.rs:17-41), write the new state; then the external
//             force of substep t+1 (external_force.rs:17-50) and its stress
//             (scatter_momentum.rs:22-93) into a per-particle scatter record.
//             Warps then replay the records with one lane per stencil node,
//             summing the records of each cell in registers, and add each
//             cell's sums to G_t+1 with one float4 reduction per node (the
//             segment's 27 blocks of G_t+1 stay resident in L2).
//   sort      every `sort_interval` substeps: binning keys, a stable radix sort
//             (bit-exact against a CPU stable sort) and the 4^3-block
//             segments; the grid blocks of the next substeps are claimed for
//             the 27-block neighbourhood of every particle block.
// Particles that drift out of their segment's tile take a global-memory path;
// a particle that leaves the claimed blocks makes the host redo the binning.
#include <cstddef>
#include <cstdio>

#include <type_traits>

#include "sv_adaptive.cuh"
#include "sv_closure.cuh"
#include "sv_collide.cuh"
#include "sv_internal.h"
#include "sv_mlp.cuh"
#include "sv_sort.cuh"

namespace sv {

namespace {

constexpr int PT = 128;  // threads (and particles per chunk) of the particle kernels
constexpr int ELEM_THREADS = 256;
constexpr int SEG_TILE = 2048;
constexpr int SEG_ITEMS = SEG_TILE / ELEM_THREADS;
constexpr int TN = 8;  // tile edge in nodes: block nodes 4b..4b+3 plus 1 below, 3 above
constexpr int TILE_NODES = TN * TN * TN;
constexpr uint32_t REC_NONE = 0xFFFFFFFFu;
constexpr uint32_t REC_GLOBAL = 0x80000000u;
constexpr uint32_t REC_VARIANT = 0x80000001u;  // non-zero collider bits: the variant table

// Scatter record of one particle: for stencil offset (i, j, k) the node gets
// mass w m and momentum w (p0[i] + p1[j] + p2[k]) with w = p0[i].w p1[j].w
// p2[k].w -- the APIC/MLS momentum m v + A (x_i - x_p) split by axis.
struct Rec {
    float4 p[9];
};

// Momentum (x, y, z) and weight (w) of stencil node (li, lj, lk) of a record.
__device__ __forceinline__ float4 rec_node(const Rec &r, int li, int lj, int lk) {
    const float4 p0 = r.p[li], p1 = r.p[3 + lj], p2 = r.p[6 + lk];
    const float2 sxy = __fadd2_rn(__fadd2_rn(make_float2(p0.x, p0.y), make_float2(p1.x, p1.y)), make_float2(p2.x, p2.y));
    return make_float4(sxy.x, sxy.y, p0.z + p1.z + p2.z, p0.w * p1.w * p2.w);
}

// MODE_G2P2G_LEARNED is MODE_G2P2G with the learned closure for snow and
// sand.  Adaptive time steps: MODE_G2P2G_ADAPTIVE is the fused pass at the
// speculative steps of the adaptive state, reducing the G2P's limits and the
// next substep's force limits as it goes; with a frame input loaded the
// substep is split instead (MODE_G2P_ONLY gathers v and C, written back in
// place, MODE_ADVANCE advances from them).
enum Mode {
    MODE_P2G = 0,
    MODE_G2P2G = 1,
    MODE_G2P2G_LEARNED = 2,
    MODE_G2P_ONLY = 3,
    MODE_ADVANCE = 4,
    MODE_G2P_ADVANCE = 5,  // the fused pass without the next scatter (the next substep's input is not loaded)
    MODE_G2P2G_ADAPTIVE = 6,
};

struct StepArgs {
    ParticleArrays in, out;
    const Material *mats;
    const SceneInfo *scenes;
    uint32_t *counters;
    const uint32_t *perm;  // nullptr: identity
    const uint32_t *seg_start;
    const uint32_t *seg_block;
    const int32_t *map_cur;   // block -> slot of the grid being gathered (G2P2G)
    const int32_t *map_next;  // block -> slot of the grid being scattered into
    const float4 *grid_cur;
    float4 *grid_next;
    uint32_t *keys_out;  // nullptr: keys not needed after this substep
    uint32_t *defer_list;  // sorted positions left by the fused pass for its fp64 pass ([C_DEFER] of them)
    uint64_t *pass_timer;  // plain fused pass only: [start ns, ns summed, passes] (else nullptr)
    const uint8_t *closure_img;          // packed network weights (learned mode)
    const closure::Hull *closure_hull;   // training hull of the features (learned mode)
    adaptive::State *adt;                // adaptive time steps: device dt and reductions (else nullptr)
    col::FrameArgs fa;                   // frame input (kernels instantiated with FIN only)
    col::VariantTable vcur, vnext;       // collider variants gathered from / scattered into
    bool self_latch;                     // the last CTA latches the stop bits and counts the substep
    // Adaptive passes (their steps come from the adaptive state):
    //   2  G2P_ADVANCE redoing a G2P2G_ADAPTIVE pass's advance at dt_c, only
    //      when the G2P's limits bound (redo)
    //   3  G2P2G_ADAPTIVE: advance at dt_spec, the next substep's scatter at
    //      dt_spec (its external force) and dt_spec_b (its stress)
    //   4  P2G of the next substep redone at its exact steps, only when a
    //      speculation failed (p2g_redo)
    uint32_t adt_pass;
    uint64_t n;
    GridLayout L;
    float dt;
    float3 gravity;
};

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t stopped(const uint32_t *counters) {
    return *(volatile const uint32_t *)&counters[C_STOP];
}

__device__ __forceinline__ void block_coords(uint32_t b, const GridLayout &L, int &bx, int &by, int &bz) {
    bz = (int)(b % (uint32_t)L.nb[2]);
    uint32_t r = b / (uint32_t)L.nb[2];
    by = (int)(r % (uint32_t)L.nb[1]);
    bx = (int)(r / (uint32_t)L.nb[1]);
}

// Neighbour t in [0, 27) of block b: offsets (t/9 - 1, (t/3)%3 - 1, t%3 - 1).
__device__ __forceinline__ uint32_t neighbour27(uint32_t b, int t, const GridLayout &L) {
    int dxb = t / 9 - 1, dyb = (t / 3) % 3 - 1, dzb = t % 3 - 1;
    return (uint32_t)((int64_t)b + (int64_t)dxb * L.nb[1] * L.nb[2] + (int64_t)dyb * L.nb[2] + dzb);
}

// Binning key of a base cell (global node coordinates); valid particles keep
// one spare block on every side of their own for the 27-neighbourhood.
__device__ __forceinline__ uint32_t cell_key(int cx, int cy, int cz, const GridLayout &L, bool &ok) {
    int lx = cx - L.origin[0], ly = cy - L.origin[1], lz = cz - L.origin[2];
    ok = lx >= 4 && ly >= 4 && lz >= 4 && (lx >> 2) < L.nb[0] - 1 && (ly >> 2) < L.nb[1] - 1 && (lz >> 2) < L.nb[2] - 1;
    if (!ok) return SENTINEL_KEY;
    uint32_t block = ((uint32_t)(lx >> 2) * (uint32_t)L.nb[1] + (uint32_t)(ly >> 2)) * (uint32_t)L.nb[2] + (uint32_t)(lz >> 2);
    return block << 6 | (uint32_t)((lx & 3) << 4 | (ly & 3) << 2 | (lz & 3));
}

// Slot of the block holding global node (x, y, z), or -1.
__device__ __forceinline__ int32_t node_slot(const int32_t *map, int x, int y, int z, const GridLayout &L, int &local) {
    int lx = x - L.origin[0], ly = y - L.origin[1], lz = z - L.origin[2];
    if (lx < 0 || ly < 0 || lz < 0 || (lx >> 2) >= L.nb[0] || (ly >> 2) >= L.nb[1] || (lz >> 2) >= L.nb[2]) return -1;
    local = (lx & 3) * 16 + (ly & 3) * 4 + (lz & 3);
    return map[((uint32_t)(lx >> 2) * (uint32_t)L.nb[1] + (uint32_t)(ly >> 2)) * (uint32_t)L.nb[2] + (uint32_t)(lz >> 2)];
}

// Base cell (floor(x/dx - 0.5), kernels.rs:46-49) and fx = x/dx - base in
// [0.5, 1.5) of a particle.
template <bool CELL>
__device__ __forceinline__ void grid_position(const float4 &pos, const int4 &cell, float dx, int base[3], float fx[3]) {
    if (!CELL) {
        float q[3] = {pos.x / dx, pos.y / dx, pos.z / dx};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float b = floorf(q[k] - 0.5f);
            base[k] = (int)b;
            fx[k] = q[k] - b;
        }
    } else {
        float o[3] = {pos.x, pos.y, pos.z};
        int ci[3] = {cell.x, cell.y, cell.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            bool hi = o[k] >= 0.5f;
            base[k] = ci[k] - (hi ? 0 : 1);
            fx[k] = o[k] + (hi ? 0.f : 1.f);
        }
    }
}

__device__ __forceinline__ void load_mat9(const float *planes, uint64_t n, uint32_t p, m3f &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) m.a[k] = planes[(uint64_t)k * n + p];
}
__device__ __forceinline__ void store_mat9(float *planes, uint64_t n, uint64_t i, const m3f &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) planes[(uint64_t)k * n + i] = m.a[k];
}

__device__ __forceinline__ void copy_particle(const ParticleArrays &in, const ParticleArrays &out, uint64_t n,
                                              uint64_t src, uint64_t dst, bool cell) {
    out.pos[dst] = in.pos[src];
    if (cell) out.cell[dst] = in.cell[src];
    out.vel[dst] = in.vel[src];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        out.C[(uint64_t)k * n + dst] = in.C[(uint64_t)k * n + src];
        out.F[(uint64_t)k * n + dst] = in.F[(uint64_t)k * n + src];
    }
    out.energy[dst] = in.energy[src];
    out.orig[dst] = in.orig[src];
    if (in.cbits) out.cbits[dst] = in.cbits[src], out.cbits_done[dst] = in.cbits_done[src];
}

// P F^T of the particle's model (the part of scatter_momentum.rs:46-90 that
// multiplies F^T (x_i - x_p)):
//   Neo-Hookean (util/src/elastic.rs:299-311): mu F F^T + (lambda ln J - mu) I
//   inviscid (elastic.rs:582-592):             K (1 - J^-gamma) J I
//   fixed-corotated / snow (additions):        2 mu U (S^2 - S) U^T + lambda (J-1) J I
// U and S are only read by the corotated kinds.
__device__ __forceinline__ m3f stress_times_ft(const Material &m, uint32_t kind, const m3f &F, float J,
                                               const m3f &U, const float S[3], float hard) {
    m3f r;
    float iso;
    if (kind == KIND_FLUID) {
#pragma unroll
        for (int k = 0; k < 9; ++k) r.a[k] = 0.f;
        iso = m.bulk_modulus * (1.f - 1.f / powi_f(J, m.exponent)) * J;
    } else if (kind == KIND_FIXED_COROTATED || kind == KIND_SNOW) {
        const float mu = m.mu * hard, la = m.lambda * hard;
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k] = 2.f * mu * (S[k] * S[k] - S[k]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                r.a[j * 3 + i] = U.a[i] * d[0] * U.a[j] + U.a[3 + i] * d[1] * U.a[3 + j] + U.a[6 + i] * d[2] * U.a[6 + j];
        iso = la * (J - 1.f) * J;
    } else {
        const m3f FFt = mat_mul_bt(F, F);
#pragma unroll
        for (int k = 0; k < 9; ++k) r.a[k] = m.mu / 2.f * 2.f * FFt.a[k];
        iso = m.lambda * logf(J) - m.mu;
    }
    r.a[0] += iso, r.a[4] += iso, r.a[8] += iso;
    return r;
}

// Builds the scatter record of a particle at base cell/fx with velocity v
// (external force already applied), velocity gradient C and stress P F^T.
__device__ __forceinline__ void make_record(const Material &m, const m3f &C, const m3f &PFt, float J, const float v[3],
                                            const float fx[3], float dx, float dt, Rec &rec) {
    const float scaling = dt * 4.f / (dx * dx);  // scatter_momentum.rs:24-25
    const float sv0 = scaling * m.initial_volume;
    m3f A;
#pragma unroll
    for (int k = 0; k < 9; ++k) A.a[k] = m.mass * C.a[k] - sv0 * PFt.a[k];
    if (m.use_viscosity) {
        // util/src/elastic.rs:659-677: 2 mu_d sym(C) + mu_b tr(C) I, times s J V0
        const float sj = sv0 * J;
        const float tr = C.a[0] + C.a[4] + C.a[8];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float s = m.visc_dynamic * (C.a[c * 3 + r] + C.a[r * 3 + c]) + (r == c ? m.visc_bulk * tr : 0.f);
                A.a[c * 3 + r] -= sj * s;
            }
    }
    float w[3][3];
    bspline_weights(fx[0], w[0]);
    bspline_weights(fx[1], w[1]);
    bspline_weights(fx[2], w[2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float dX = ((float)k - fx[0]) * dx, dY = ((float)k - fx[1]) * dx, dZ = ((float)k - fx[2]) * dx;
        rec.p[k] = make_float4(m.mass * v[0] + A.a[0] * dX, m.mass * v[1] + A.a[1] * dX, m.mass * v[2] + A.a[2] * dX, w[0][k]);
        rec.p[3 + k] = make_float4(A.a[3] * dY, A.a[4] * dY, A.a[5] * dY, w[1][k]);
        rec.p[6 + k] = make_float4(A.a[6] * dZ, A.a[7] * dZ, A.a[8] * dZ, w[2][k]);
    }
}

// The material kinds a handle's particles use, as a set of 1 << KIND_*.  The
// plain fused pass is compiled for two common sets (fixed-corotated, snow and
// sand; fluid and Neo-Hookean) as well as for all kinds: without the other
// kinds' code the compiler allocates the pass's registers for what runs
// (1M three-box scene +2 %, 8M dam break +4 %, 64 batched scenes +1.6 %).
constexpr uint32_t KSET_ALL = 0x1Fu;
constexpr uint32_t KSET_SOLID_PLASTIC = (1u << KIND_FIXED_COROTATED) | (1u << KIND_SNOW) | (1u << KIND_SAND);
constexpr uint32_t KSET_FLUID_NH = (1u << KIND_FLUID) | (1u << KIND_NEO_HOOKEAN);
// A particle's kind, known to lie in KSET.
template <uint32_t KSET> __device__ __forceinline__ uint32_t kind_in(uint32_t k) {
    if constexpr (KSET == KSET_SOLID_PLASTIC)
        return k == KIND_SAND ? (uint32_t)KIND_SAND : k == KIND_SNOW ? (uint32_t)KIND_SNOW : (uint32_t)KIND_FIXED_COROTATED;
    else if constexpr (KSET == KSET_FLUID_NH)
        return k == KIND_FLUID ? (uint32_t)KIND_FLUID : (uint32_t)KIND_NEO_HOOKEAN;
    else
        return k;
}

// ------------------------------------------------------------------ keys
template <bool CELL> __global__ void __launch_bounds__(ELEM_THREADS) k_keys(StepArgs A) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += (uint64_t)gridDim.x * blockDim.x) {
        float4 pos = A.in.pos[i];
        uint32_t packed = __float_as_uint(pos.w);
        uint32_t key = SENTINEL_KEY;
        if (!(packed & SV_TOMBSTONED)) {
            int base[3];
            float fx[3];
            grid_position<CELL>(pos, CELL ? A.in.cell[i] : make_int4(0, 0, 0, 0), A.L.dx, base, fx);
            bool ok;
            key = cell_key(base[0], base[1], base[2], A.L, ok);
            if (!ok) atomicOr(&A.counters[C_STATUS], ST_OUT_OF_GRID);
        }
        A.keys_out[i] = key;
    }
}

// ------------------------------------------------------------------ segments
__device__ __forceinline__ bool is_head(const uint32_t *sk, uint64_t i) {
    uint32_t k = sk[i];
    if (k == SENTINEL_KEY) return false;
    return i == 0 || (sk[i - 1] >> 6) != (k >> 6);
}

__global__ void __launch_bounds__(ELEM_THREADS)
    k_seg_count(const uint32_t *sk, uint64_t n, uint32_t *tile_counts, uint32_t *counters) {
    uint64_t base = (uint64_t)blockIdx.x * SEG_TILE;
    uint32_t c = 0;
#pragma unroll
    for (int j = 0; j < SEG_ITEMS; ++j) {
        uint64_t i = base + (uint64_t)j * ELEM_THREADS + threadIdx.x;
        if (i < n) {
            c += is_head(sk, i);
            uint32_t k = sk[i];
            if (k == SENTINEL_KEY && (i == 0 || sk[i - 1] != SENTINEL_KEY)) counters[C_NLIVE] = (uint32_t)i;
            if (i == n - 1 && k != SENTINEL_KEY) counters[C_NLIVE] = (uint32_t)n;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ uint32_t red[ELEM_THREADS / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < ELEM_THREADS / 32; ++w) t += red[w];
        tile_counts[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(ELEM_THREADS)
    k_seg_write(const uint32_t *sk, uint64_t n, const uint32_t *tile_offsets, uint32_t tiles, uint32_t *seg_start,
                uint32_t *seg_block, uint32_t *counters) {
    __shared__ uint32_t warp_sums[ELEM_THREADS / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * SEG_TILE + (uint64_t)threadIdx.x * SEG_ITEMS;
    bool head[SEG_ITEMS];
    uint32_t c = 0;
#pragma unroll
    for (int j = 0; j < SEG_ITEMS; ++j) {
        uint64_t i = base + j;
        head[j] = i < n && is_head(sk, i);
        c += head[j];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int w = 0; w < ELEM_THREADS / 32; ++w) {
            uint32_t t = warp_sums[w];
            warp_sums[w] = run;
            run += t;
        }
        warp_sums[ELEM_THREADS / 32] = run;
    }
    __syncthreads();
    uint32_t out = tile_offsets[blockIdx.x] + warp_sums[warp] + inc - c;
#pragma unroll
    for (int j = 0; j < SEG_ITEMS; ++j) {
        if (head[j]) {
            seg_start[out] = (uint32_t)(base + j);
            seg_block[out] = sk[base + j] >> 6;
            ++out;
        }
    }
    if (blockIdx.x == tiles - 1 && threadIdx.x == 0) {
        uint32_t nseg = tile_offsets[blockIdx.x] + warp_sums[ELEM_THREADS / 32];
        counters[C_NSEG] = nseg;
        seg_start[nseg] = counters[C_NLIVE];
    }
}

// ------------------------------------------------------------------ block maps
__global__ void __launch_bounds__(ELEM_THREADS)
    k_map_reset(int32_t *map, const uint32_t *active, uint32_t *counters, int which, uint64_t capacity) {
    uint64_t cnt = counters[C_NSLOT0 + which];
    if (cnt > capacity) cnt = capacity;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < cnt; s += (uint64_t)gridDim.x * blockDim.x)
        map[active[s]] = -1;
}

// Latches the stop bits; optionally zeroes (reset_which) or clamps to the
// capacity (clamp_which) a slot counter.
__global__ void k_latch(uint32_t *counters, int reset_which, int clamp_which, uint64_t capacity) {
    if (reset_which >= 0) counters[C_NSLOT0 + reset_which] = 0;
    if (clamp_which >= 0 && counters[C_NSLOT0 + clamp_which] > capacity) counters[C_NSLOT0 + clamp_which] = (uint32_t)capacity;
    counters[C_STOP] = counters[C_STATUS] & STOP_MASK;
}

// Claims a slot for each block in the 27-neighbourhood of every segment.
__global__ void __launch_bounds__(ELEM_THREADS)
    k_activate(const uint32_t *seg_block, int32_t *map, uint32_t *active, uint64_t capacity, GridLayout L,
               uint32_t *counters, int which) {
    if (stopped(counters)) return;
    uint32_t nseg = counters[C_NSEG];
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (uint64_t)nseg * 27;
         t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = neighbour27(seg_block[t / 27], (int)(t % 27), L);
        if (atomicCAS(&map[b], -1, -2) == -1) {
            uint32_t slot = atomicAdd(&counters[C_NSLOT0 + which], 1u);
            if (slot < capacity) {
                active[slot] = b;
                map[b] = (int32_t)slot;
            } else {
                map[b] = -1;
                atomicOr(&counters[C_STATUS], ST_CAPACITY);
            }
        }
    }
}

__global__ void __launch_bounds__(ELEM_THREADS)
    k_clear_grid(float4 *grid, uint64_t capacity, uint32_t *counters, int which, double *sums,
                 const uint32_t *only_if = nullptr) {
    if (only_if && !*only_if) return;
    if (blockIdx.x == 0 && threadIdx.x < 4) sums[threadIdx.x] = 0.0;
    uint64_t slots = counters[C_NSLOT0 + which];
    if (slots > capacity) slots = capacity;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < slots * 64; i += (uint64_t)gridDim.x * blockDim.x)
        grid[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ------------------------------------------------------------------ grid update
// Momentum -> velocity of grid node i (block index `block`): the
// compatible collider variants' momentum first (meld_grid.rs:29-58: bits 0 is
// compatible with every variant), the fp64 sums on the way.
__device__ __forceinline__ float4 grid_node(float4 g, uint64_t i, uint32_t block, const GridLayout &L,
                                            const col::VariantTable &var, bool want_sums, double s[4]) {
    int bx = 0, by = 0, bz = 0;
    if (var.key || L.ground_mode != 0) block_coords(block, L, bx, by, bz);
    const int l = (int)(i & 63);
    const int x = L.origin[0] + 4 * bx + (l >> 4), y = L.origin[1] + 4 * by + ((l >> 2) & 3), z = L.origin[2] + 4 * bz + (l & 3);
    if (var.key) {
        const int64_t e = col::node_entry(var, x, y, z);
        if (e >= 0)
            for (int j = 0; j < col::VK; ++j)
                if (var.bits[e * col::VK + j]) {
                    const float4 a = var.acc[e * col::VK + j];
                    g.x += a.x, g.y += a.y, g.z += a.z, g.w += a.w;
                }
    }
    if (want_sums) s[0] += (double)g.w, s[1] += (double)g.x, s[2] += (double)g.y, s[3] += (double)g.z;
    return node_velocity(g, x, y, z, L);
}

// Momentum -> velocity on grid_cur (slots of map `wc`), and zeroes grid_next
// (slots of map `wn`) for the scatter that follows.  On the way it adds the
// fp64 sums of mass and momentum over grid_cur's nodes (variants included)
// into sums_cur -- from substep counters[C_SUMS_AT] on (sv_step sets it to
// the last substep of the call: the fp64 work costs 7 % of a substep) --
// and zeroes sums_next with grid_next.  Launched as one wave of resident
// CTAs, each thread takes two nodes a stride apart with both loads in
// flight: the 1M-particle scene's 0.3M nodes then take one pass of memory
// latency instead of two waves of one node per thread.
__global__ void __launch_bounds__(ELEM_THREADS, 4)
    k_grid_update(float4 *grid_cur, const uint32_t *active_cur, float4 *grid_next, uint64_t capacity, GridLayout L,
                  uint32_t *counters, int wc, int wn, col::VariantTable var, double *sums_cur, double *sums_next) {
    if (stopped(counters)) return;
    uint64_t sc = counters[C_NSLOT0 + wc], sn = grid_next ? counters[C_NSLOT0 + wn] : 0;
    if (sc > capacity) sc = capacity;
    if (sn > capacity) sn = capacity;
    if (grid_next && blockIdx.x == 0 && threadIdx.x < 4) sums_next[threadIdx.x] = 0.0;
    const bool want_sums = counters[C_SUBSTEPS] >= counters[C_SUMS_AT];
    const bool need_block = var.key || L.ground_mode != 0;
    const uint64_t total = (sc > sn ? sc : sn) * 64, nc = sc * 64, nn = sn * 64;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += 2 * stride) {
        const uint64_t j = i + stride;
        const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 gi = i < nc ? grid_cur[i] : zero, gj = j < nc ? grid_cur[j] : zero;
        const uint32_t bi = need_block && i < nc ? active_cur[i >> 6] : 0u;
        const uint32_t bj = need_block && j < nc ? active_cur[j >> 6] : 0u;
        if (i < nc) grid_cur[i] = grid_node(gi, i, bi, L, var, want_sums, s);
        if (j < nc) grid_cur[j] = grid_node(gj, j, bj, L, var, want_sums, s);
        if (i < nn) grid_next[i] = zero;
        if (j < nn) grid_next[j] = zero;
    }
    double sm = s[0], sx = s[1], sy = s[2], sz = s[3];
    if (!want_sums) return;  // uniform over the grid
    // The block's sum in fp64 with few fp64 instructions (about 16 clocks
    // per warp instruction on this part): every thread's partial sums go
    // to shared memory and warp 0 alone adds them up, rather than eight
    // warps running a shuffle tree each.
    __shared__ double red[4][ELEM_THREADS];
    red[0][threadIdx.x] = sm, red[1][threadIdx.x] = sx, red[2][threadIdx.x] = sy, red[3][threadIdx.x] = sz;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int j = 0; j < ELEM_THREADS / 32; ++j)
#pragma unroll
            for (int c = 0; c < 4; ++c) t[c] += red[c][threadIdx.x + 32 * j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < 4; ++c) t[c] += __shfl_xor_sync(0xffffffffu, t[c], o);
        if (threadIdx.x < 4) {
            const double v = threadIdx.x == 0 ? t[0] : threadIdx.x == 1 ? t[1] : threadIdx.x == 2 ? t[2] : t[3];
            if (v != 0.0) atomicAdd(&sums_cur[threadIdx.x], v);
        }
    }
}

// Melds the collider variants (meld_grid.rs:16-69): variant (node, bits) gets
// its own momentum, the node's bits-0 momentum from the dense grid (still
// raw: this runs before k_grid_update) and every compatible variant's; then
// v = p / m and the boundary plane as in k_grid_update.
__global__ void __launch_bounds__(ELEM_THREADS)
    k_variant_meld(col::VariantTable var, const float4 *grid_raw, const int32_t *map, GridLayout L,
                   const uint32_t *counters) {
    if (stopped(counters)) return;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < var.cap; e += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = var.key[e];
        if (k == 0ull) continue;
        const unsigned long long q = k - 1ull;
        const int node[3] = {(int)((q >> 42) & 0x1FFFFFull) - (1 << 20), (int)((q >> 21) & 0x1FFFFFull) - (1 << 20),
                             (int)(q & 0x1FFFFFull) - (1 << 20)};
        int local;
        const int32_t slot = node_slot(map, node[0], node[1], node[2], L, local);
        const float4 base = slot >= 0 ? grid_raw[(uint64_t)slot * 64 + local] : make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t b[col::VK];
        float4 a[col::VK];
        for (int j = 0; j < col::VK; ++j) b[j] = var.bits[e * col::VK + j], a[j] = var.acc[e * col::VK + j];
        for (int j = 0; j < col::VK; ++j) {
            if (!b[j]) continue;
            float4 g = make_float4(a[j].x + base.x, a[j].y + base.y, a[j].z + base.z, a[j].w + base.w);
            for (int o = 0; o < col::VK; ++o)
                if (o != j && b[o] && col::compatible(b[j], b[o])) g.x += a[o].x, g.y += a[o].y, g.z += a[o].z, g.w += a[o].w;
            var.vel[e * col::VK + j] = node_velocity(g, node[0], node[1], node[2], L);
        }
    }
}

// ------------------------------------------------------------------ frame input interpolation
// interpolate_input.rs:18-106 at `time` (or the adaptive state's time):
// factor of frame b, gravity, vertex positions, frictions, dampings.
struct FinDev {
    uint32_t fps, frame, nv, nt;
    float g_a[3], g_b[3];
    const float *va, *vb, *fr_a, *fr_b, *dm_a, *dm_b;
    const uint32_t *tri, *vt_start, *vt_list;
    float *scalars;  // gravity[3], factor
    float *vpos, *vnorm, *tnorm, *fric, *damp;
};

__global__ void k_interp_factor(FinDev f, double time, const adaptive::State *st, uint32_t *counters) {
    if (st && stopped(counters)) return;
    const double t = st ? st->time : time;
    const double ft = t * (double)f.fps;
    if ((long long)floor(ft) != (long long)f.frame) {  // frame_input.rs:266-278 WrongFrameLoaded
        atomicOr(&counters[C_STATUS], ST_WRONG_FRAME);
        return;
    }
    const float fb = (float)fmod(ft, 1.0), fa = 1.f - fb;
    for (int a = 0; a < 3; ++a) f.scalars[a] = fa * f.g_a[a] + fb * f.g_b[a];
    f.scalars[3] = fb;
}

__global__ void __launch_bounds__(ELEM_THREADS) k_interp_vertices(FinDev f, const uint32_t *counters) {
    const float fb = f.scalars[3], fa = 1.f - fb;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < 3ull * f.nv; k += (uint64_t)gridDim.x * blockDim.x)
        f.vpos[k] = fa * f.va[k] + fb * f.vb[k];
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < f.nt; t += (uint64_t)gridDim.x * blockDim.x)
        f.fric[t] = fa * f.fr_a[t] + fb * f.fr_b[t], f.damp[t] = fa * f.dm_a[t] + fb * f.dm_b[t];
}

__device__ inline void normalize_or_zero(float a[3]) {  // nalgebra try_normalize(1e-5)
    const float nn = sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (nn <= col::EPS) a[0] = a[1] = a[2] = 0.f;
    else a[0] /= nn, a[1] /= nn, a[2] /= nn;
}

__global__ void __launch_bounds__(ELEM_THREADS) k_interp_triangles(FinDev f) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < f.nt; t += (uint64_t)gridDim.x * blockDim.x) {
        const float *A = f.vpos + 3 * f.tri[3 * t], *B = f.vpos + 3 * f.tri[3 * t + 1], *C = f.vpos + 3 * f.tri[3 * t + 2];
        const float ab[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]}, ac[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
        float n[3];
        col::cross3(ab, ac, n);
        normalize_or_zero(n);
        for (int a = 0; a < 3; ++a) f.tnorm[3 * t + a] = n[a];
    }
}

// angle-weighted vertex normals (interpolate_input.rs:56-79)
__global__ void __launch_bounds__(ELEM_THREADS) k_interp_vertex_normals(FinDev f) {
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < f.nv; v += (uint64_t)gridDim.x * blockDim.x) {
        float s[3] = {0.f, 0.f, 0.f};
        const float *P = f.vpos + 3 * v;
        for (uint32_t k = f.vt_start[v]; k < f.vt_start[v + 1]; ++k) {
            const uint32_t t = f.vt_list[k];
            uint32_t others[2] = {0, 0}, m = 0;
            for (int c = 0; c < 3; ++c)
                if (f.tri[3 * t + c] != (uint32_t)v && m < 2) others[m++] = f.tri[3 * t + c];
            const float *A = f.vpos + 3 * others[0], *B = f.vpos + 3 * others[1];
            const float pa[3] = {A[0] - P[0], A[1] - P[1], A[2] - P[2]}, pb[3] = {B[0] - P[0], B[1] - P[1], B[2] - P[2]};
            const float na = sqrtf(col::dot3(pa, pa)), nb = sqrtf(col::dot3(pb, pb));
            float ang = 0.f;
            if (na != 0.f && nb != 0.f) {
                const float c = col::dot3(pa, pb) / (na * nb);
                ang = c > 1.f ? 0.f : (c < -1.f ? 3.14159265358979f : acosf(c));
            }
            for (int a = 0; a < 3; ++a) s[a] += ang * f.tnorm[3 * t + a];
        }
        normalize_or_zero(s);
        for (int a = 0; a < 3; ++a) f.vnorm[3 * v + a] = s[a];
    }
}

// ------------------------------------------------------------------ particle kernel
// Scatter tile layout: node (tx, ty, tz) at tx*PX + ty*PY + tz.  With PX = 3
// and PY = 9 (mod 32) the 27 stencil offsets 9i + 3j + k of any cell fall in
// 27 distinct shared-memory banks, so a warp's lane-per-node lookups of the
// nodes' grid indices never conflict.  A grid index is slot * 64 + node, below
// 2^32 - 1 (NO_NODE) because the block index holds fewer than 2^26 blocks.
constexpr uint32_t NO_NODE = 0xFFFFFFFFu;
constexpr int PY = 9, PX = 99;
constexpr int PLANE = 7 * PX + 7 * PY + 8;  // 764 floats

struct Shared {
    float4 gv[TILE_NODES];      // velocity tile of grid_cur (G2P2G), tx*64 + ty*8 + tz
    uint32_t gidx[PLANE];       // float4 index in grid_next of each tile node (NO_NODE: no claimed block)
    Rec rec[PT];
    float2 meta[PT];            // (record cell as bits: REC_NONE, tile index or REC_GLOBAL; mass)
    int4 gbase[PT];             // global base cell of REC_GLOBAL records
    int32_t slot_cur[27];
    int32_t slot_next[27];
    int raised;                 // a thread of the CTA set a status bit (see cta_done)
};

// Tile node (tx, ty, tz) in [0, 8)^3 of block (bx, by, bz): global node
// 4b - 1 + t, in neighbour block (t + 3) / 4 - 1 along each axis.
__device__ __forceinline__ int tile_neighbour(int tx, int ty, int tz) {
    return ((tx + 3) / 4) * 9 + ((ty + 3) / 4) * 3 + (tz + 3) / 4;
}
__device__ __forceinline__ int tile_local(int tx, int ty, int tz) {
    return ((tx + 3) & 3) * 16 + ((ty + 3) & 3) * 4 + ((tz + 3) & 3);
}

// Adds one cell's summed contributions (mass, px | py, pz) to tile node t:
// one float4 reduction into grid_next, which the 27 blocks of a segment keep
// resident in L2.
__device__ __forceinline__ void flush_node(Shared &sh, const StepArgs &A, int t, float2 amx, float2 ayz) {
    const uint32_t g = sh.gidx[t];
    if (g != NO_NODE)
        atomicAdd(&A.grid_next[g], make_float4(amx.y, ayz.x, ayz.y, amx.x));
    else
        atomicOr(&A.counters[C_STATUS], ST_MOVED_FAR), sh.raised = 1;
}

// Replays the chunk's scatter records: warp w owns records [32w, 32w + 32);
// lane l < 27 is stencil offset (l/9, (l/3)%3, l%3).  The records of one
// tile cell (found with a match over the warp's keys, wherever they sit in
// the chunk) are summed in registers and leave once per lane, so each
// distinct cell of the warp's records costs one float4 reduction per node
// however far the particles drifted since the binning sort.  Two records per
// step keep two sets of shared loads in flight.
__device__ __forceinline__ void scatter_records(Shared &sh, int count, const StepArgs &A) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int li = lane / 9, lj = (lane / 3) % 3, lk = lane % 3;
    const bool active = lane < 27;
    const int off = li * PX + lj * PY + lk;
    const int r0 = warp * 32;
    if (r0 >= count) return;
    const float2 me = lane < count - r0 ? sh.meta[r0 + lane] : make_float2(__uint_as_float(REC_NONE), 0.f);
    const uint32_t key = __float_as_uint(me.x);
    const bool valid = key < REC_GLOBAL;  // a tile index
    const uint32_t gmask = __ballot_sync(0xffffffffu, key == REC_GLOBAL);
    const uint32_t cmask = __ballot_sync(0xffffffffu, key == REC_VARIANT);
    // lanes with the same key; the lowest valid lane of each group leads it
    const uint32_t grp = __match_any_sync(0xffffffffu, key);
    const uint32_t lead = __ballot_sync(0xffffffffu, valid && (grp & ((1u << lane) - 1u)) == 0u);
    const Rec *rp = &sh.rec[r0];
    for (uint32_t lb = lead; lb; lb &= lb - 1) {
        const int s = __ffs(lb) - 1;
        uint32_t mm = __shfl_sync(0xffffffffu, grp, s);
        float2 amx = make_float2(0.f, 0.f), ayz = make_float2(0.f, 0.f);
        while (mm) {
            const int ra = __ffs(mm) - 1;
            mm &= mm - 1;
            const float4 na = rec_node(rp[ra], li, lj, lk);
            const float ma = __shfl_sync(0xffffffffu, me.y, ra);
            if (mm) {
                const int rb = __ffs(mm) - 1;
                mm &= mm - 1;
                const float4 nb = rec_node(rp[rb], li, lj, lk);
                const float mb = __shfl_sync(0xffffffffu, me.y, rb);
                amx = __ffma2_rn(make_float2(na.w, na.w), make_float2(ma, na.x), amx);
                ayz = __ffma2_rn(make_float2(na.w, na.w), make_float2(na.y, na.z), ayz);
                amx = __ffma2_rn(make_float2(nb.w, nb.w), make_float2(mb, nb.x), amx);
                ayz = __ffma2_rn(make_float2(nb.w, nb.w), make_float2(nb.y, nb.z), ayz);
            } else {
                amx = __ffma2_rn(make_float2(na.w, na.w), make_float2(ma, na.x), amx);
                ayz = __ffma2_rn(make_float2(na.w, na.w), make_float2(na.y, na.z), ayz);
            }
        }
        const int t = (int)__shfl_sync(0xffffffffu, key, s) + off;
        if (active) flush_node(sh, A, t, amx, ayz);
    }
    // records outside the tile: straight to global memory
    for (uint32_t g = gmask; g; g &= g - 1) {
        const int r = __ffs(g) - 1;
        const float4 nd = rec_node(sh.rec[r0 + r], li, lj, lk);
        const float w = nd.w;
        const float m = sh.meta[r0 + r].y;
        const int4 gb = sh.gbase[r0 + r];
        if (active) {
            int local;
            const int32_t slot = node_slot(A.map_next, gb.x + li, gb.y + lj, gb.z + lk, A.L, local);
            if (slot >= 0)
                atomicAdd(&A.grid_next[(uint64_t)slot * 64 + local], make_float4(w * nd.x, w * nd.y, w * nd.z, w * m));
            else
                atomicOr(&A.counters[C_STATUS], ST_MOVED_FAR), sh.raised = 1;
        }
    }
    // records of particles with collider bits: their (node, bits) variants
    // (update_grid_nodes.rs:94-118)
    for (uint32_t g = cmask; g; g &= g - 1) {
        const int r = __ffs(g) - 1;
        const float4 nd = rec_node(sh.rec[r0 + r], li, lj, lk);
        const float w = nd.w;
        const float m = sh.meta[r0 + r].y;
        const int4 gb = sh.gbase[r0 + r];
        if (active) {
            const int64_t s = col::variant_slot(A.vnext, gb.x + li, gb.y + lj, gb.z + lk, (uint32_t)gb.w, true);
            if (s >= 0)
                atomicAdd(&A.vnext.acc[s], make_float4(w * nd.x, w * nd.y, w * nd.z, w * m));
            else
                atomicOr(&A.counters[C_STATUS], ST_VARIANT_FULL), sh.raised = 1;
        }
    }
}

// G2P of a particle with collider bits from its (node, bits) variants.
__device__ __forceinline__ void gather_variant(const StepArgs &A, const int base[3], uint32_t bits, const float w[3][3],
                                               const float d[3][3], float v[3], m3f &C) {
    v[0] = v[1] = v[2] = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) C.a[k] = 0.f;
    for (int ii = 0; ii < 3; ++ii)
        for (int jj = 0; jj < 3; ++jj)
            for (int kk = 0; kk < 3; ++kk) {
                const float wt = w[0][ii] * w[1][jj] * w[2][kk];
                const int64_t s = col::variant_slot(A.vcur, base[0] + ii, base[1] + jj, base[2] + kk, bits, false);
                const float4 g = s >= 0 ? A.vcur.vel[s] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float gx = g.x * wt, gy = g.y * wt, gz = g.z * wt;
                v[0] += gx, v[1] += gy, v[2] += gz;
                C.a[0] += gx * d[0][ii], C.a[1] += gy * d[0][ii], C.a[2] += gz * d[0][ii];
                C.a[3] += gx * d[1][jj], C.a[4] += gy * d[1][jj], C.a[5] += gz * d[1][jj];
                C.a[6] += gx * d[2][kk], C.a[7] += gy * d[2][kk], C.a[8] += gz * d[2][kk];
            }
}

// Record key for a particle scattering from base cell `base` into the tile
// whose node 0 is global node `org`.
__device__ __forceinline__ uint32_t tile_cell(const int base[3], const int org[3], int4 &gb) {
    const int tx = base[0] - org[0], ty = base[1] - org[1], tz = base[2] - org[2];
    if (tx >= 0 && ty >= 0 && tz >= 0 && tx <= TN - 3 && ty <= TN - 3 && tz <= TN - 3) return (uint32_t)(tx * PX + ty * PY + tz);
    gb = make_int4(base[0], base[1], base[2], 0);
    return REC_GLOBAL;
}

// G2P gather (collect_velocity.rs:40-72) of v and the unscaled C from the
// shared velocity tile, factorised over the separable weights:
// a_ij = sum_k wz_k g_ijk, b_ij = sum_k wz_k dZ_k g_ijk, then over j and i.
__device__ __forceinline__ void gather_tile(const float4 *gv, int t0, const float w[3][3], const float d[3][3],
                                            float v[3], m3f &C) {
    float3 c[3], dd[3], e[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        c[i] = dd[i] = e[i] = make_float3(0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float3 a = make_float3(0.f, 0.f, 0.f), b = make_float3(0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float4 g = gv[t0 + i * 64 + j * 8 + k];
                const float wz = w[2][k], wzd = w[2][k] * d[2][k];
                a.x += wz * g.x, a.y += wz * g.y, a.z += wz * g.z;
                b.x += wzd * g.x, b.y += wzd * g.y, b.z += wzd * g.z;
            }
            const float wy = w[1][j], wyd = w[1][j] * d[1][j];
            c[i].x += wy * a.x, c[i].y += wy * a.y, c[i].z += wy * a.z;
            dd[i].x += wyd * a.x, dd[i].y += wyd * a.y, dd[i].z += wyd * a.z;
            e[i].x += wy * b.x, e[i].y += wy * b.y, e[i].z += wy * b.z;
        }
    }
    v[0] = v[1] = v[2] = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) C.a[k] = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float wx = w[0][i], wxd = w[0][i] * d[0][i];
        v[0] += wx * c[i].x, v[1] += wx * c[i].y, v[2] += wx * c[i].z;
        C.a[0] += wxd * c[i].x, C.a[1] += wxd * c[i].y, C.a[2] += wxd * c[i].z;
        C.a[3] += wx * dd[i].x, C.a[4] += wx * dd[i].y, C.a[5] += wx * dd[i].z;
        C.a[6] += wx * e[i].x, C.a[7] += wx * e[i].y, C.a[8] += wx * e[i].z;
    }
}

// The same gather from global memory for particles outside their tile.
__device__ __forceinline__ void gather_global(const StepArgs &A, const int base[3], const float w[3][3],
                                              const float d[3][3], float v[3], m3f &C) {
    v[0] = v[1] = v[2] = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) C.a[k] = 0.f;
    for (int ii = 0; ii < 3; ++ii)
        for (int jj = 0; jj < 3; ++jj)
            for (int kk = 0; kk < 3; ++kk) {
                const float wt = w[0][ii] * w[1][jj] * w[2][kk];
                int local;
                const int32_t slot = node_slot(A.map_cur, base[0] + ii, base[1] + jj, base[2] + kk, A.L, local);
                const float4 g = slot >= 0 ? A.grid_cur[(uint64_t)slot * 64 + local] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float gx = g.x * wt, gy = g.y * wt, gz = g.z * wt;
                v[0] += gx, v[1] += gy, v[2] += gz;
                C.a[0] += gx * d[0][ii], C.a[1] += gy * d[0][ii], C.a[2] += gz * d[0][ii];
                C.a[3] += gx * d[1][jj], C.a[4] += gy * d[1][jj], C.a[5] += gz * d[1][jj];
                C.a[6] += gx * d[2][kk], C.a[7] += gy * d[2][kk], C.a[8] += gz * d[2][kk];
            }
}

// Shared state of the learned closure (feature hull, TMEM and MMA-completion
// control).  The network image (its forward part) sits in dynamic shared
// memory; the two operand buffers overlay the records, their metadata and
// global bases, which are free between the previous chunk's replay and this
// chunk's record writes.
struct SharedLearned {
    closure::Hull hull;
    mlp::Ctl ctl;
};
constexpr int LEARNED_SMEM_BYTES = tc::IMG_FWD_BYTES;
static_assert(offsetof(Shared, meta) == offsetof(Shared, rec) + sizeof(Rec) * PT &&
                  offsetof(Shared, gbase) == offsetof(Shared, meta) + sizeof(float2) * PT &&
                  sizeof(Rec) * PT + (sizeof(float2) + sizeof(int4)) * PT >= (tc::NIN + tc::NH) * PT * 2 &&
                  offsetof(Shared, rec) % 16 == 0,
              "closure operands overlay the records");

// End of a self-latching pass (one call per CTA, by all its threads): the
// last CTA to finish latches the stop bits for the kernels that follow and
// counts the substep unless the pass started stopped -- the work of k_latch
// and k_finish without their launches.  Threads that set a status bit fence
// it (only when one did: `raised`), then thread 0's fence orders everything
// before its ticket.
__device__ __forceinline__ void cta_done(const StepArgs &A, uint32_t stop_at_start, const volatile int *raised) {
    if (!A.self_latch) return;
    __syncthreads();
    if (raised && *raised) __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t ticket = atomicAdd(&A.counters[C_CTA_DONE], 1u);
        if (ticket == gridDim.x - 1) {
            __threadfence();
            const uint32_t status = *(volatile uint32_t *)&A.counters[C_STATUS];
            A.counters[C_STOP] = status & STOP_MASK;
            if (!stop_at_start) A.counters[C_SUBSTEPS] += 1;
            A.counters[C_CTA_DONE] = 0;
            A.counters[C_DEFER] = 0;  // the fused pass's fp64 list has been served
            A.counters[C_SEGQ] = 0;
            if (A.pass_timer && !stop_at_start) {
                // the plain fused pass and its fp64 pass, first CTA start to here
                A.pass_timer[1] += global_ns() - A.pass_timer[0];
                A.pass_timer[2] += 1;
            }
        }
    }
}

// Five CTAs per SM (at most 102 registers): measured faster than the
// unconstrained 150-register build despite a few spilled values.  The
// learned-closure variant holds the network image as well: three CTAs; the
// frame-input variant four.
// FIN: a frame input is loaded -- interpolated gravity and goals, Collide
// (collide.rs:21-206) before the scatter, collider bits and their variants.
// REDO (with MODE_G2P2G): the fused pass's fp64 pass.  The plain fused pass
// holds no fp64 SVD code: inlined, that rarely taken path gave the pass a
// 256-byte stack frame and four times the register spills of the fp32 path
// (0.66M against 0.20M local loads per 1M-particle launch).  A particle whose
// fp32 SVD is degenerate or flagged by the fp64 policy is left out of the
// fused pass and listed; the REDO pass then runs the whole substep for the
// listed particles (from the same input state and grid, the gather and
// scatter through global memory) with the fp64 SVD, and latches the stop
// bits for both.
#ifndef SV_PARTICLE_CTAS_PER_SM
#define SV_PARTICLE_CTAS_PER_SM 5
#endif
template <bool CELL, int MODE, bool FIN = false, bool REDO = false, uint32_t KSET = KSET_ALL>
__global__ void __launch_bounds__(PT, MODE == MODE_G2P2G_LEARNED ? 3 : FIN ? 4 : SV_PARTICLE_CTAS_PER_SM)
    k_particles(StepArgs A) {
    static_assert(!REDO || (MODE == MODE_G2P2G && !FIN), "the fp64 pass follows the plain fused pass");
    constexpr bool LEARNED = MODE == MODE_G2P2G_LEARNED;
    constexpr bool DEFER64 = MODE == MODE_G2P2G && !FIN && !REDO;
    // the pass's start for its timer (CTA 0 is among the first to run)
    if (DEFER64 && A.pass_timer && blockIdx.x == 0 && threadIdx.x == 0) A.pass_timer[0] = global_ns();
    // what the pass does: gather from the grid, advance the particles (and
    // write them out in sorted order), scatter into the next grid
    constexpr bool ADT_FUSED = MODE == MODE_G2P2G_ADAPTIVE;
    constexpr bool GATHER = MODE == MODE_G2P2G || LEARNED || ADT_FUSED || MODE == MODE_G2P_ONLY || MODE == MODE_G2P_ADVANCE;
    constexpr bool G2P = MODE == MODE_G2P2G || LEARNED || ADT_FUSED || MODE == MODE_ADVANCE || MODE == MODE_G2P_ADVANCE;  // advances
    constexpr bool SCATTER = MODE == MODE_P2G || MODE == MODE_G2P2G || LEARNED || ADT_FUSED;
    constexpr bool LOAD_VC = MODE == MODE_P2G || MODE == MODE_ADVANCE;  // v and C from the state
    __shared__ Shared sh;
    __shared__ typename std::conditional<LEARNED, SharedLearned, int>::type shl;
    if (MODE == MODE_G2P_ADVANCE && A.adt_pass == 2 && !*(volatile const uint32_t *)&A.adt->redo) return;
    if (MODE == MODE_P2G && A.adt_pass == 4 && !*(volatile const uint32_t *)&A.adt->p2g_redo) return;
    const uint32_t stop_at_start = stopped(A.counters);
    if (stop_at_start) {
        if (G2P && !REDO) {
            // Keep the state as it is (identity copy) so the buffer swap is a no-op.
            for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += (uint64_t)gridDim.x * blockDim.x)
                copy_particle(A.in, A.out, A.n, i, i, CELL);
        }
        cta_done(A, stop_at_start, nullptr);
        return;
    }
    if (threadIdx.x == 0) sh.raised = 0;
    mlp::Phase ph;
    uint32_t n_learned = 0, n_closure_fb = 0;
    extern __shared__ __align__(128) uint8_t learned_img[];
    if constexpr (LEARNED) {
        for (int t = threadIdx.x * 16; t < LEARNED_SMEM_BYTES; t += PT * 16)
            *reinterpret_cast<uint4 *>(learned_img + t) = *reinterpret_cast<const uint4 *>(A.closure_img + t);
        for (int t = threadIdx.x; t < (int)(sizeof(closure::Hull) / 4); t += PT)
            reinterpret_cast<float *>(&shl.hull)[t] = reinterpret_cast<const float *>(A.closure_hull)[t];
        mlp::ctl_init(shl.ctl, mlp::TMEM_COLS_INFER);
    }
    const uint32_t nseg = A.counters[C_NSEG];
    const uint32_t nlive = A.counters[C_NLIVE];
    const float dx = A.L.dx;
    // time steps of the external force, the scatter and the advance: one dt,
    // or the three of the adaptive state's phases
    float dt_force = A.dt, dt_scatter = A.dt, dt_adv = A.dt;
    if (A.adt) {
        dt_force = A.adt->dt_a, dt_scatter = A.adt->dt_b, dt_adv = A.adt->dt_c;
        if (A.adt_pass == 3) dt_adv = dt_force = A.adt->dt_spec, dt_scatter = A.adt->dt_spec_b;
        if (A.adt_pass == 4) dt_force = A.adt->dt_c, dt_scatter = A.adt->dt_b_next;
    }
    // G2P_ONLY and the speculative G2P_ADVANCE: max |v| and max |C_ij| of live particles
    constexpr bool G2P_LIMITS_MODE = MODE == MODE_G2P_ONLY || MODE == MODE_G2P_ADVANCE || ADT_FUSED;
    const bool g2p_limits = MODE == MODE_G2P_ONLY || ADT_FUSED;
    float red_v = 0.f, red_c = 0.f;
    bool red_live = false;
    // ADVANCE, adaptive G2P_ADVANCE: the next substep's sound and isolated
    // limits of the advanced state
    constexpr bool FORCE_LIMITS_MODE = MODE == MODE_ADVANCE || MODE == MODE_G2P_ADVANCE || ADT_FUSED;
    float lim_sound = adaptive::NONE, lim_iso = adaptive::NONE;
    if (G2P && !REDO) {
        // particles that were tombstoned at binning time are carried over
        for (uint64_t i = nlive + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += (uint64_t)gridDim.x * blockDim.x) {
            copy_particle(A.in, A.out, A.n, A.perm ? A.perm[i] : i, i, CELL);
            if (A.keys_out) A.keys_out[i] = SENTINEL_KEY;
        }
    }
    uint32_t fp64_count = 0, fallback = 0;
    // One chunk of up to PT particles: thread t takes the particle at sorted
    // position i (has: there is one), org is the tile's node origin.
    auto chunk = [&](const uint32_t i, const bool has, const int count, const int *org) {
        uint32_t rcell = REC_NONE;
        float rmass = 0.f;
        // this thread's particle; live across the closure network pass
        bool work = false;
        uint32_t p = 0, packed = 0, orig_p = 0;
        float vel_w = 1.f;
        float4 pos = make_float4(0.f, 0.f, 0.f, 0.f);
        int4 cell = make_int4(0, 0, 0, 0);
        m3f F, C;
        float v[3] = {0.f, 0.f, 0.f};
        float plastic_j = 1.f;
        // collider bits in effect for this pass (FIN): for a gather the
        // bits the particle scattered with, for a standalone scatter the
        // bits after the last completed substep
        uint32_t bits_in = 0;
        if (has) {
            p = A.perm ? A.perm[i] : i;
            pos = A.in.pos[p];
            packed = __float_as_uint(pos.w);
            if (CELL) cell = A.in.cell[p];
            // issued with the position: neither waits for the material
            // table, and the copy of orig does not wait behind this
            // particle's stores
            if (!LOAD_VC) vel_w = A.in.vel[p].w;
            if (G2P) orig_p = A.in.orig[p];
            if (packed & SV_TOMBSTONED) {
                if (G2P) {
                    copy_particle(A.in, A.out, A.n, p, i, CELL);
                    if (A.keys_out) A.keys_out[i] = SENTINEL_KEY;
                }
            } else {
                work = true;
                const uint32_t kind = kind_in<KSET>(A.mats[packed >> MATERIAL_SHIFT].kind);
                if constexpr (FIN) bits_in = MODE == MODE_P2G ? A.in.cbits_done[p] : A.in.cbits[p];
                if (MODE != MODE_G2P_ONLY) load_mat9(A.in.F, A.n, p, F);
                if (LOAD_VC) {
                    load_mat9(A.in.C, A.n, p, C);
                    const float4 vel = A.in.vel[p];
                    v[0] = vel.x, v[1] = vel.y, v[2] = vel.z;
                    plastic_j = vel.w;
                } else {
                    plastic_j = (kind == KIND_SNOW || MODE == MODE_G2P_ONLY) ? vel_w : 1.f;
                    // ---- G2P (collect_velocity.rs:40-72)
                    int base[3];
                    float fx[3];
                    grid_position<CELL>(pos, cell, dx, base, fx);
                    float w[3][3];
                    bspline_weights(fx[0], w[0]);
                    bspline_weights(fx[1], w[1]);
                    bspline_weights(fx[2], w[2]);
                    float d[3][3];
#pragma unroll
                    for (int a = 0; a < 3; ++a)
#pragma unroll
                        for (int k = 0; k < 3; ++k) d[a][k] = ((float)k - fx[a]) * dx;
                    const int tx = base[0] - org[0], ty = base[1] - org[1], tz = base[2] - org[2];
                    const bool in_tile = tx >= 0 && ty >= 0 && tz >= 0 && tx <= TN - 3 && ty <= TN - 3 && tz <= TN - 3;
                    if (FIN && bits_in != 0u) {
                        gather_variant(A, base, bits_in, w, d, v, C);  // collect_velocity.rs:61-62 keyed by bits
                    } else if (in_tile) {
                        gather_tile(sh.gv, tx * 64 + ty * 8 + tz, w, d, v, C);
                    } else {
                        if (!REDO) ++fallback;
                        gather_global(A, base, w, d, v, C);
                    }
                    const float cscale = 4.f / dx / dx;
#pragma unroll
                    for (int k = 0; k < 9; ++k) C.a[k] *= cscale;
                }
                if constexpr (MODE == MODE_G2P_ONLY) {
                    // v and C back into the state, in place
                    A.in.vel[p] = make_float4(v[0], v[1], v[2], plastic_j);
                    store_mat9(A.in.C, A.n, p, C);
                }
                if constexpr (G2P_LIMITS_MODE) {
                    // the limits of limit_time_step.rs:189-222 reduce over v and C
                    if (g2p_limits) {
                        red_v = fmaxf(red_v, sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
#pragma unroll
                        for (int k = 0; k < 9; ++k) red_c = fmaxf(red_c, fabsf(C.a[k]));
                        red_live = true;
                    }
                }
                if (G2P) {
                    // ---- advance (advance_particles.rs:39-41): x += v dt, F += C F dt
                    {
                        const m3f CF = mat_mul(C, F);
#pragma unroll
                        for (int k = 0; k < 9; ++k) F.a[k] += CF.a[k] * dt_adv;
                    }
                    if (!CELL) {
                        pos.x += v[0] * dt_adv, pos.y += v[1] * dt_adv, pos.z += v[2] * dt_adv;
                    } else {
                        float o[3] = {pos.x + v[0] * dt_adv / dx, pos.y + v[1] * dt_adv / dx, pos.z + v[2] * dt_adv / dx};
                        int ci[3] = {cell.x, cell.y, cell.z};
#pragma unroll
                        for (int k = 0; k < 3; ++k) {
                            const float fl = floorf(o[k]);
                            ci[k] += (int)fl;
                            o[k] -= fl;
                            if (o[k] >= 1.f) o[k] = 0.f, ci[k] += 1;
                        }
                        pos.x = o[0], pos.y = o[1], pos.z = o[2];
                        cell = make_int4(ci[0], ci[1], ci[2], 0);
                    }
                }
            }
        }
        // ---- learned closure (snow, sand): closed-form principal
        // stretches, then one network pass for the whole chunk on the
        // tensor cores (all threads take part)
        int l_class = closure::L_PLAIN;  // after the network: L_PLAIN, L_ELASTIC or L_NET
        float l_sig[3], l_V[9], l_y[tc::NOUT];
        if constexpr (LEARNED) {
            float x[tc::NIN];
            if (work) {
                const Material &lm = A.mats[packed >> MATERIAL_SHIFT];
                if (closure::applies(lm.kind)) l_class = closure::learned_features(lm, F, shl.hull, l_sig, l_V, x);
            }
            const bool want = l_class == closure::L_NET;
            if (!want)
#pragma unroll
                for (int k = 0; k < tc::NIN; ++k) x[k] = 0.f;
            if (__syncthreads_or(want)) {
                bool ok = false;
                if (!shl.ctl.abort) {
                    uint8_t *a0 = reinterpret_cast<uint8_t *>(sh.rec);
                    ok = mlp::infer_tile(shl.ctl, ph, learned_img, a0, a0 + tc::NIN * PT * 2, x, l_y);
                }
                if (want && !ok) l_class = closure::L_PLAIN;
            }
        }
        // ---- SVD (advance_particles.rs:42-44); in the plain fused pass the
        // fp32 SVD only, a particle it cannot serve going to the fp64 pass
        m3f U, V;
        float S[3] = {1.f, 1.f, 1.f};
        if constexpr (DEFER64) {
            if (work && kind_in<KSET>(A.mats[packed >> MATERIAL_SHIFT].kind) != KIND_NEO_HOOKEAN) {
                const bool degenerate = svd3_fast_f32(F, U, S, V);
                if (svd_needs_fp64(F, S, degenerate, A.L.svd_policy)) {
                    A.defer_list[atomicAdd(&A.counters[C_DEFER], 1u)] = i;
                    work = false;
                }
            }
        }
        if (work && (G2P || SCATTER)) {
            const Material mat = A.mats[packed >> MATERIAL_SHIFT];
            const uint32_t kind = kind_in<KSET>(mat.kind);
            // ---- plasticity (advance_particles.rs:45-86), energy
            float energy = 0.f;
            m3f tau_l{};  // learned path: Kirchhoff stress P F^T
            bool use_l = false;
            if constexpr (LEARNED) {
                if (l_class != closure::L_PLAIN) {
                    m3f Fn;
                    float e_l, jp_l, J_l;
                    if (closure::learned_apply(mat, F, l_sig, l_V, l_class == closure::L_NET ? l_y : nullptr, shl.hull,
                                               plastic_j, Fn, tau_l, e_l, jp_l, J_l)) {
                        use_l = true;
                        F = Fn;
                        plastic_j = jp_l;
                        energy = e_l;
                    }
                }
                if (closure::applies(kind)) {
                    if (use_l) ++n_learned;
                    else ++n_closure_fb;
                }
            }
            if (!use_l) {
                const bool need_svd = G2P ? kind != KIND_NEO_HOOKEAN : (kind == KIND_FIXED_COROTATED || kind == KIND_SNOW);
                if (need_svd && !DEFER64) particle_svd(F, U, S, V, A.L.svd_policy | (REDO ? SVD_ALWAYS_FP64 : 0u), fp64_count);
                if (G2P) {
                    if (kind == KIND_SAND) {
                        // Drucker-Prager return map in Hencky strain (advance_particles.rs:48-71)
                        const float e[3] = {logf(S[0]), logf(S[1]), logf(S[2])};
                        const float e_tr = e[0] + e[1] + e[2];
                        const float eh[3] = {e[0] - e_tr / 3.f, e[1] - e_tr / 3.f, e[2] - e_tr / 3.f};
                        const float ehn = sqrtf(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]);
                        if (e_tr < 0.f && ehn > 0.f) {
                            if (!(mat.mu > 0.f)) {
                                // the reference asserts mu > 0 here (:57)
                                atomicOr(&A.counters[C_STATUS], ST_SAND_MU), sh.raised = 1;
                            } else {
                                const float dg = ehn + (3.f * mat.lambda + 2.f * mat.mu) / 2.f / mat.mu * e_tr * mat.alpha;
                                if (dg > 0.f) {
#pragma unroll
                                    for (int k = 0; k < 3; ++k) S[k] = expf(e[k] - dg / ehn * eh[k]);
                                    F = recompose(U, S, V);
                                }
                            }
                        } else {
                            // expansion: U V^T whatever mu is
                            S[0] = S[1] = S[2] = 1.f;
                            F = mat_mul_bt(U, V);
                        }
                    } else if (kind == KIND_FLUID) {
                        // advance_particles.rs:77-85: singular values -> geometric mean
                        const float g = powf(S[0] * S[1] * S[2], 1.f / 3.f);
                        S[0] = S[1] = S[2] = g;
                        F = recompose(U, S, V);
                    } else if (kind == KIND_SNOW) {
                        // addition: Stomakhin et al. 2013 clamp + hardening state
                        float s[3];
#pragma unroll
                        for (int k = 0; k < 3; ++k) s[k] = fminf(fmaxf(S[k], 1.f - mat.theta_c), 1.f + mat.theta_s);
                        plastic_j = plastic_j * (S[0] * S[1] * S[2]) / (s[0] * s[1] * s[2]);
#pragma unroll
                        for (int k = 0; k < 3; ++k) S[k] = s[k];
                        F = recompose(U, S, V);
                    }
                }
            }
            const float J = det3(F);
            const float hard = kind == KIND_SNOW ? expf(mat.xi * (1.f - plastic_j)) : 1.f;
            bool alive = true;
            if (G2P) {
                if (use_l) {
                    // energy of the learned projected stretches (J > 0 by construction)
                } else if (kind == KIND_FLUID) {
                    // util/src/elastic.rs:546-553
                    const float K = mat.bulk_modulus, gm = (float)mat.exponent;
                    const float at_rest = K * (1.f - 1.f / (1.f - gm));
                    energy = K * (J - powi_f(J, 1 - mat.exponent) / (1.f - gm)) - at_rest;
                } else if (!(J > 0.f)) {
                    // try_elastic_energy_neo_hookean: J <= 0 -> FAILED (advance_particles.rs:73-74)
                    packed |= SV_FAILED;
                    atomicOr(&A.counters[C_STATUS], ST_INVERTED), sh.raised = 1;
                } else if (kind == KIND_FIXED_COROTATED || kind == KIND_SNOW) {
                    // mu |F - R|^2 + lambda/2 (J - 1)^2 = mu sum (s - 1)^2 + ...
                    const float d2 = (S[0] - 1.f) * (S[0] - 1.f) + (S[1] - 1.f) * (S[1] - 1.f) + (S[2] - 1.f) * (S[2] - 1.f);
                    energy = mat.mu * hard * d2 + mat.lambda * hard / 2.f * (J - 1.f) * (J - 1.f);
                } else {
                    // util/src/elastic.rs:233-241
                    float I2 = 0.f;
#pragma unroll
                    for (int k = 0; k < 9; ++k) I2 += F.a[k] * F.a[k];
                    const float lj = logf(J);
                    energy = mat.mu / 2.f * (I2 - 3.f) - mat.mu * lj + mat.lambda / 2.f * lj * lj;
                }
                // cull (cull_particles.rs:17-41): strict domain bounds
                bool inside;
                if (!CELL) {
                    inside = pos.x > A.L.domain_min[0] && pos.x < A.L.domain_max[0] && pos.y > A.L.domain_min[1] &&
                             pos.y < A.L.domain_max[1] && pos.z > A.L.domain_min[2] && pos.z < A.L.domain_max[2];
                } else {
                    // scene-local cell coordinates against the scene's domain
                    const SceneInfo &sc = A.scenes[mat.scene];
                    const double q[3] = {(double)(cell.x - sc.off[0]) + pos.x, (double)(cell.y - sc.off[1]) + pos.y,
                                         (double)(cell.z - sc.off[2]) + pos.z};
                    inside = q[0] > sc.dmin[0] && q[0] < sc.dmax[0] && q[1] > sc.dmin[1] && q[1] < sc.dmax[1] &&
                             q[2] > sc.dmin[2] && q[2] < sc.dmax[2];
                }
                if (!inside) packed |= SV_TOMBSTONED;
                alive = !(packed & (SV_TOMBSTONED | SV_FAILED));
                if constexpr (FORCE_LIMITS_MODE) {
                    // LimitTimeStepBeforeForce of the next substep
                    // (limit_time_step.rs:25-178) over the state just
                    // written: the singular values come from this pass's
                    // SVD (after the plastic projection, which sets them);
                    // Neo-Hookean solids took none and take one here.
                    if (A.adt && !(packed & SV_TOMBSTONED)) {
                        float s[3] = {S[0], S[1], S[2]};
                        if (kind == KIND_NEO_HOOKEAN) {
                            uint32_t none = 0;
                            particle_svd(F, U, s, V, 0, none);
                        }
                        if (s[0] < s[1]) { const float t = s[0]; s[0] = s[1], s[1] = t; }
                        if (s[1] < s[2]) { const float t = s[1]; s[1] = s[2], s[2] = t; }
                        if (s[0] < s[1]) { const float t = s[0]; s[0] = s[1], s[1] = t; }
                        const bool fluid = kind == KIND_FLUID;
                        const float a = adaptive::sound_limit<float>(fluid, mat.mu, mat.lambda, mat.bulk_modulus,
                                                                     mat.exponent, mat.mass, mat.initial_volume, s, dx);
                        const float b = fluid ? adaptive::isolated_limit<float>(true, mat.mu, mat.lambda, mat.bulk_modulus,
                                                                                mat.exponent, mat.mass, mat.initial_volume, J, dx)
                                              : mat.iso_limit;
                        if (a > 0.f && a < adaptive::NONE) lim_sound = fminf(lim_sound, a);
                        if (b > 0.f && b < adaptive::NONE) lim_iso = fminf(lim_iso, b);
                    }
                }
                // write the advanced state in sorted order
                pos.w = __uint_as_float(packed);
                A.out.pos[i] = pos;
                if (CELL) A.out.cell[i] = cell;
                A.out.vel[i] = make_float4(v[0], v[1], v[2], plastic_j);
                store_mat9(A.out.C, A.n, i, C);
                store_mat9(A.out.F, A.n, i, F);
                A.out.energy[i] = energy;
                A.out.orig[i] = orig_p;
                if constexpr (FIN) {
                    // the bits of the completed substep; the next
                    // scatter's Collide (below) replaces the ones in effect
                    A.out.cbits_done[i] = bits_in;
                    A.out.cbits[i] = bits_in;
                }
            }
            int nbase[3];
            float nfx[3];
            grid_position<CELL>(pos, cell, dx, nbase, nfx);
            if (G2P && A.keys_out) {
                uint32_t key = SENTINEL_KEY;
                if (!(packed & SV_TOMBSTONED)) {
                    bool ok;
                    key = cell_key(nbase[0], nbase[1], nbase[2], A.L, ok);
                    if (!ok) atomicOr(&A.counters[C_STATUS], ST_OUT_OF_GRID), sh.raised = 1;
                }
                A.keys_out[i] = key;
            }
            if (SCATTER && alive) {
                // ---- scatter record of the next substep: Collide
                // (collide.rs:21-206), external force (external_force.rs:17-50),
                // then the momentum of scatter_momentum.rs:38-90
                uint32_t bits_new = 0u;
                if constexpr (FIN) {
                    const float P[3] = {CELL ? ((float)cell.x + pos.x) * dx : pos.x,
                                        CELL ? ((float)cell.y + pos.y) * dx : pos.y,
                                        CELL ? ((float)cell.z + pos.z) * dx : pos.z};
                    bits_new = bits_in;
                    if (A.fa.nt) col::collide_particle(A.fa, P, v, bits_new, dt_force);
                    else bits_new = 0u;  // nothing to check (collide.rs:53-56)
                    const uint32_t o = A.in.orig[p];
                    if (A.fa.goal_both && A.fa.goal_both[o]) {
                        // both frames give a goal: reach it in one step
                        const float fb = A.fa.factor[0], fa_ = 1.f - fb;
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            v[a] = (fa_ * A.fa.goal_a[3 * o + a] + fb * A.fa.goal_b[3 * o + a] - P[a]) / dt_force;
                    } else {
#pragma unroll
                        for (int a = 0; a < 3; ++a) v[a] += dt_force * A.fa.gravity[a];
                    }
                    if (G2P) A.out.cbits[i] = bits_new;
                    else A.in.cbits[p] = bits_new;
                } else {
                    v[0] += dt_force * A.gravity.x, v[1] += dt_force * A.gravity.y, v[2] += dt_force * A.gravity.z;
                }
                const m3f PFt = use_l ? tau_l : stress_times_ft(mat, kind, F, J, U, S, hard);
                make_record(mat, C, PFt, J, v, nfx, dx, dt_scatter, sh.rec[threadIdx.x]);
                rmass = mat.mass;
                int4 gb;
                rcell = tile_cell(nbase, org, gb);
                if (FIN && bits_new != 0u) {
                    rcell = REC_VARIANT;
                    gb = make_int4(nbase[0], nbase[1], nbase[2], (int)bits_new);
                }
                if (rcell == REC_GLOBAL || rcell == REC_VARIANT) sh.gbase[threadIdx.x] = gb;
            }
        }
        if (SCATTER) {
            sh.meta[threadIdx.x] = make_float2(__uint_as_float(rcell), rmass);
            // Warp w replays only its own threads' records, so warp
            // barriers would do here; measured 1-2 % slower than keeping
            // the CTA's warps in step, so the CTA barriers stay.
            __syncthreads();
            scatter_records(sh, count, A);
            __syncthreads();
        }
    };
    if constexpr (REDO) {
        // one pass per CTA over its share of the list, with no tile: every
        // listed particle takes the global gather and scatter
        const uint32_t end = A.counters[C_DEFER];
        const int org[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
        for (uint32_t c0 = blockIdx.x * PT; c0 < end; c0 += gridDim.x * PT) {
            const uint32_t slot = c0 + threadIdx.x;
            chunk(slot < end ? A.defer_list[slot] : 0u, slot < end, (int)min((uint32_t)PT, end - c0), org);
        }
    } else {
        // The plain fused pass: one resident wave of CTAs takes segments
        // from a queue, so segments of uneven size balance without the
        // oversubscribed grid the other passes use (which pays each CTA's
        // start and end per segment).
        constexpr bool QUEUE = DEFER64;
        __shared__ uint32_t next_seg;
        uint32_t seg = blockIdx.x;
        if (QUEUE) {
            if (threadIdx.x == 0) next_seg = atomicAdd(&A.counters[C_SEGQ], 1u);
            __syncthreads();
            seg = next_seg;
        }
        while (seg < nseg) {
            const uint32_t b = A.seg_block[seg];
            const uint32_t start = A.seg_start[seg], end = A.seg_start[seg + 1];
            int bx, by, bz;
            block_coords(b, A.L, bx, by, bz);
            const int org[3] = {A.L.origin[0] + 4 * bx - 1, A.L.origin[1] + 4 * by - 1, A.L.origin[2] + 4 * bz - 1};
            if (threadIdx.x < 27) {
                const uint32_t nbk = neighbour27(b, threadIdx.x, A.L);
                sh.slot_next[threadIdx.x] = A.map_next[nbk];
                if (GATHER) sh.slot_cur[threadIdx.x] = A.map_cur[nbk];
            }
            __syncthreads();
            if (SCATTER)
                for (int t = threadIdx.x; t < TILE_NODES; t += PT) {
                    const int tx = t >> 6, ty = (t >> 3) & 7, tz = t & 7;
                    const int32_t slot = sh.slot_next[tile_neighbour(tx, ty, tz)];
                    sh.gidx[tx * PX + ty * PY + tz] = slot >= 0 ? (uint32_t)slot * 64u + (uint32_t)tile_local(tx, ty, tz) : NO_NODE;
                }
            if (GATHER) {
                for (int t = threadIdx.x; t < TILE_NODES; t += PT) {
                    const int tx = t >> 6, ty = (t >> 3) & 7, tz = t & 7;
                    const int32_t slot = sh.slot_cur[tile_neighbour(tx, ty, tz)];
                    sh.gv[t] = slot >= 0 ? A.grid_cur[(uint64_t)slot * 64 + tile_local(tx, ty, tz)] : make_float4(0.f, 0.f, 0.f, 0.f);
                }
                __syncthreads();
            }
            for (uint32_t c0 = start; c0 < end; c0 += PT)
                chunk(c0 + threadIdx.x, c0 + threadIdx.x < end, (int)min((uint32_t)PT, end - c0), org);
            if (QUEUE) {
                // (every thread read next_seg before this segment's barriers)
                if (threadIdx.x == 0) next_seg = atomicAdd(&A.counters[C_SEGQ], 1u);
                __syncthreads();
                seg = next_seg;
            } else {
                seg += gridDim.x;
            }
            __syncthreads();
        }
    }
    if (G2P_LIMITS_MODE && g2p_limits) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            red_v = fmaxf(red_v, __shfl_xor_sync(0xffffffffu, red_v, o));
            red_c = fmaxf(red_c, __shfl_xor_sync(0xffffffffu, red_c, o));
        }
        const bool any = __any_sync(0xffffffffu, red_live);
        if ((threadIdx.x & 31) == 0 && any) {
            atomicMax(&A.adt->red_max_v, __float_as_uint(red_v));
            atomicMax(&A.adt->red_max_c, __float_as_uint(red_c));
            atomicOr(&A.adt->red_live, 1u);
        }
    }
    if constexpr (FORCE_LIMITS_MODE) {
        if (A.adt) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lim_sound = fminf(lim_sound, __shfl_xor_sync(0xffffffffu, lim_sound, o));
                lim_iso = fminf(lim_iso, __shfl_xor_sync(0xffffffffu, lim_iso, o));
            }
            if ((threadIdx.x & 31) == 0) {
                if (lim_sound < adaptive::NONE) atomicMin(&A.adt->red_sound, __float_as_uint(lim_sound));
                if (lim_iso < adaptive::NONE) atomicMin(&A.adt->red_iso, __float_as_uint(lim_iso));
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fp64_count += __shfl_xor_sync(0xffffffffu, fp64_count, o);
        fallback += __shfl_xor_sync(0xffffffffu, fallback, o);
        if (LEARNED) {
            n_learned += __shfl_xor_sync(0xffffffffu, n_learned, o);
            n_closure_fb += __shfl_xor_sync(0xffffffffu, n_closure_fb, o);
        }
    }
    if ((threadIdx.x & 31) == 0) {
        if (fp64_count) atomicAdd(&A.counters[C_FP64], fp64_count);
        if (fallback) atomicAdd(&A.counters[C_FALLBACK], fallback);
        if (n_learned) atomicAdd(&A.counters[C_CLOSURE], n_learned);
        if (n_closure_fb) atomicAdd(&A.counters[C_CLOSURE_FB], n_closure_fb);
    }
    if constexpr (LEARNED) mlp::ctl_finish(shl.ctl, mlp::TMEM_COLS_INFER, &A.counters[C_CLOSURE_ERR]);
    cta_done(A, 0u, &sh.raised);
}

__global__ void k_finish(uint32_t *counters) {
    if (!counters[C_STOP]) counters[C_SUBSTEPS] += 1;
}

// ------------------------------------------------------------------ adaptive time steps
// limit_time_step.rs:25-33 (LimitTimeStepBeforeForce): the sound-speed and
// isolated-particle limits over the live particles' current F, reduced as
// float bits (positive values order like their bits).
__global__ void __launch_bounds__(ELEM_THREADS)
    k_limits_force(ParticleArrays s, const Material *mats, uint64_t n, float dx, adaptive::State *st,
                   const uint32_t *counters) {
    // the last substep's advance reduced them over the same state already
    if (stopped(counters) || st->force_ready) return;
    float ls = adaptive::NONE, li = adaptive::NONE;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t packed = __float_as_uint(s.pos[i].w);
        if (packed & SV_TOMBSTONED) continue;
        const Material m = mats[packed >> MATERIAL_SHIFT];
        m3f F, U, V;
        load_mat9(s.F, n, i, F);
        float S[3];
        uint32_t dummy = 0;
        particle_svd(F, U, S, V, 0, dummy);
        // descending, as the reference's SVD returns them
        if (S[0] < S[1]) { const float t = S[0]; S[0] = S[1], S[1] = t; }
        if (S[1] < S[2]) { const float t = S[1]; S[1] = S[2], S[2] = t; }
        if (S[0] < S[1]) { const float t = S[0]; S[0] = S[1], S[1] = t; }
        const bool fluid = m.kind == KIND_FLUID;
        const float a = adaptive::sound_limit<float>(fluid, m.mu, m.lambda, m.bulk_modulus, m.exponent, m.mass,
                                                     m.initial_volume, S, dx);
        const float b = !fluid ? m.iso_limit : adaptive::isolated_limit<float>(true, m.mu, m.lambda, m.bulk_modulus, m.exponent, m.mass,
                                                        m.initial_volume, det3(F), dx);
        if (a > 0.f && a < adaptive::NONE) ls = fminf(ls, a);
        if (b > 0.f && b < adaptive::NONE) li = fminf(li, b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ls = fminf(ls, __shfl_xor_sync(0xffffffffu, ls, o));
        li = fminf(li, __shfl_xor_sync(0xffffffffu, li, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (ls < adaptive::NONE) atomicMin(&st->red_sound, __float_as_uint(ls));
        if (li < adaptive::NONE) atomicMin(&st->red_iso, __float_as_uint(li));
    }
}

// ExternalForce takes the step allowed before LimitTimeStepBeforeForce
// pushes its limits; ScatterMomentum the one after (limit_time_step.rs:25-33,
// adaptive_time_step_state.rs:35-63).
__global__ void k_dt_force(adaptive::State *st, uint32_t *counters) {
    if (counters[C_STOP]) return;
    st->dt_a = adaptive::allowed(*st);
    st->sound = __uint_as_float(st->red_sound);
    st->iso = __uint_as_float(st->red_iso);
    adaptive::push(*st);
    st->dt_b = adaptive::allowed(*st);
    st->red_max_v = 0u, st->red_max_c = 0u, st->red_live = 0u;
    // consumed: the advance of this substep reduces the next ones
    st->red_sound = __float_as_uint(adaptive::NONE), st->red_iso = __float_as_uint(adaptive::NONE);
    st->force_ready = 0;
    st->dt_spec = adaptive::step_without_g2p_limits(*st);
    st->dt_spec_b = adaptive::next_scatter_step_without_new_limits(*st);
    st->redo = 0, st->p2g_redo = 0;
    if (!(st->dt_a > 0.f) || !(st->dt_b > 0.f)) counters[C_STATUS] |= ST_ZERO_DT;
}

// limit_time_step.rs:181-222 (LimitTimeStepBeforeIntegrate) from the
// reductions of the G2P pass; AdvanceParticles takes the step after the push.
__global__ void k_dt_integrate(adaptive::State *st, uint32_t *counters, float dx) {
    if (counters[C_STOP]) return;
    const float mv = __uint_as_float(st->red_max_v), mc = __uint_as_float(st->red_max_c);
    st->vel = mv != 0.f ? 0.5f * dx / mv : adaptive::NONE;
    st->def = st->red_live ? 0.2f / fmaxf(mc, 1e-8f) : adaptive::NONE;
    adaptive::push(*st);
    st->dt_c = adaptive::allowed(*st);
    // a speculative advance at dt_spec (adaptive G2P_ADVANCE) is redone when
    // the G2P's limits bind; the redo reduces the force limits again
    st->redo = st->dt_c != st->dt_spec;
    if (st->redo) st->red_sound = st->red_iso = __float_as_uint(adaptive::NONE);
    if (!(st->dt_c > 0.f)) counters[C_STATUS] |= ST_ZERO_DT;
}

// cpu_state.rs:186-189: the substep's time step is added to the time; the
// run stops (ST_TIME_REACHED latches) once the target time is reached.
// `next_scatter`: the substep's pass also scattered the next substep, whose
// failure (a particle outside the claimed blocks, the block capacity) is
// redone by the host without undoing this one.
__global__ void k_adaptive_finish(adaptive::State *st, uint32_t *counters, bool next_scatter = false) {
    const uint32_t mask = next_scatter ? STOP_MASK & ~(ST_MOVED_FAR | ST_CAPACITY) : STOP_MASK;
    if (counters[C_STOP] || (counters[C_STATUS] & mask)) return;
    st->force_ready = 1;  // the advance completed its reduction of the next force limits
    st->time += (double)st->dt_c;
    st->substeps += 1;
    counters[C_SUBSTEPS] += 1;
    if (st->time >= st->target) counters[C_STATUS] |= ST_TIME_REACHED;
}

// ------------------------------------------------------------------ deterministic P2G
// (sv_consts::deterministic_p2g)  The particles are binned by (cell, original
// index) -- the binning keys written in original-index order, then the
// stable radix sort -- and every grid node gathers its mass and momentum in
// one fixed order: the 27 base cells around it in lexicographic order, each
// cell's particles in ascending original index.  The mass of each pair is
// the reference's (scatter_momentum.rs:22-93): w = kernel(n - x/dx) per axis
// (kernels.rs:17-26), product over x, y, z, times m, summed left to right --
// every operation rounded on its own, as the CPU computes it.

// keys in original-index order; inv = slot of each original particle
__global__ void __launch_bounds__(ELEM_THREADS)
    k_det_order(const uint32_t *orig, const uint32_t *keys, uint64_t n, uint32_t *kbo, uint32_t *inv) {
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t o = orig[s];
        kbo[o] = keys[s];
        inv[o] = (uint32_t)s;
    }
}

// sorted position -> device slot, from the sort's original indices
__global__ void __launch_bounds__(ELEM_THREADS)
    k_det_perm(const uint32_t *sorted_orig, const uint32_t *inv, uint64_t n, uint32_t *perm) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        perm[i] = inv[sorted_orig[i]];
}

// grid slot -> segment of its block (-1: no particles), cleared per binning
__global__ void __launch_bounds__(ELEM_THREADS)
    k_det_slot_reset(int32_t *slot_seg, const uint32_t *counters, int which, uint64_t capacity) {
    uint64_t cnt = counters[C_NSLOT0 + which];
    if (cnt > capacity) cnt = capacity;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < cnt; s += (uint64_t)gridDim.x * blockDim.x)
        slot_seg[s] = -1;
}

// First sorted index of each of the 64 cells of each segment (entry 64: the
// segment's end), and the segment of each claimed block's slot.
__global__ void __launch_bounds__(ELEM_THREADS)
    k_det_cells(const uint32_t *sk, const uint32_t *seg_start, const uint32_t *seg_block, const int32_t *map,
                const uint32_t *counters, uint32_t *cstart, int32_t *slot_seg, uint64_t max_seg) {
    uint64_t nseg = counters[C_NSEG];
    if (nseg > max_seg) nseg = max_seg;  // more segments than claimed blocks: the claim failed (ST_CAPACITY)
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nseg * 65; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t seg = (uint32_t)(t / 65), c = (uint32_t)(t % 65);
        const uint32_t b = seg_block[seg];
        uint32_t lo = seg_start[seg], hi = seg_start[seg + 1];
        if (c < 64) {
            const uint32_t key = b << 6 | c;
            while (lo < hi) {  // first position whose key is not below `key`
                const uint32_t mid = lo + (hi - lo) / 2;
                if (sk[mid] < key) lo = mid + 1;
                else hi = mid;
            }
        }
        cstart[t] = c < 64 ? lo : hi;  // entry 64: the segment's end
        if (c == 0) {
            const int32_t slot = map[b];
            if (slot >= 0) slot_seg[slot] = (int32_t)seg;
        }
    }
}

// Per sorted particle: x/dx, the mass, m v after the external force and
// A = m C - s V0 P F^T (- viscosity), the affine momentum of the scatter
// (as the fused pass builds it, scatter_momentum.rs:38-90).
template <bool CELL>
__global__ void __launch_bounds__(ELEM_THREADS) k_det_records(StepArgs A, float4 *rec) {
    const uint32_t nlive = A.counters[C_NLIVE];
    if (stopped(A.counters)) return;
    uint32_t fp64_dummy = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nlive; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t p = A.perm ? A.perm[i] : (uint32_t)i;
        const float4 pos = A.in.pos[p];
        const uint32_t packed = __float_as_uint(pos.w);
        const Material mat = A.mats[packed >> MATERIAL_SHIFT];
        m3f F, C, U, V;
        load_mat9(A.in.F, A.n, p, F);
        load_mat9(A.in.C, A.n, p, C);
        const float4 vel = A.in.vel[p];
        float v[3] = {vel.x + A.dt * A.gravity.x, vel.y + A.dt * A.gravity.y, vel.z + A.dt * A.gravity.z};
        float S[3] = {1.f, 1.f, 1.f};
        if (mat.kind == KIND_FIXED_COROTATED || mat.kind == KIND_SNOW) particle_svd(F, U, S, V, A.L.svd_policy, fp64_dummy);
        const float J = det3(F);
        const float hard = mat.kind == KIND_SNOW ? expf(mat.xi * (1.f - vel.w)) : 1.f;
        const m3f PFt = stress_times_ft(mat, mat.kind, F, J, U, S, hard);
        const float sv0 = A.dt * 4.f / (A.L.dx * A.L.dx) * mat.initial_volume;
        m3f Am;
#pragma unroll
        for (int k = 0; k < 9; ++k) Am.a[k] = mat.mass * C.a[k] - sv0 * PFt.a[k];
        if (mat.use_viscosity) {
            const float sj = sv0 * J, tr = C.a[0] + C.a[4] + C.a[8];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    Am.a[c * 3 + r] -= sj * (mat.visc_dynamic * (C.a[c * 3 + r] + C.a[r * 3 + c]) + (r == c ? mat.visc_bulk * tr : 0.f));
        }
        float4 *o = rec + 4 * i;
        o[0] = make_float4(__fdiv_rn(pos.x, A.L.dx), __fdiv_rn(pos.y, A.L.dx), __fdiv_rn(pos.z, A.L.dx), mat.mass);
        o[1] = make_float4(mat.mass * v[0], mat.mass * v[1], mat.mass * v[2], Am.a[0]);
        o[2] = make_float4(Am.a[1], Am.a[2], Am.a[3], Am.a[4]);
        o[3] = make_float4(Am.a[5], Am.a[6], Am.a[7], Am.a[8]);
    }
}

// kernels.rs:17-26 with every operation rounded on its own (no contraction)
__device__ __forceinline__ float det_kernel(float r) {
    r = fabsf(r);
    if (r < 0.5f) return __fsub_rn(0.75f, __fmul_rn(r, r));
    if (r < 1.5f) {
        const float t = __fsub_rn(1.5f, r);
        return __fmul_rn(__fmul_rn(0.5f, t), t);
    }
    return 0.f;
}

// One thread per node of the claimed blocks: the fixed-order gather.
__global__ void __launch_bounds__(ELEM_THREADS)
    k_det_gather(const float4 *rec, const uint32_t *active, const int32_t *map, const int32_t *slot_seg,
                 const uint32_t *cstart, float4 *grid, GridLayout L, const uint32_t *counters, int which,
                 uint64_t capacity) {
    if (stopped(counters)) return;
    uint64_t slots = counters[C_NSLOT0 + which];
    if (slots > capacity) slots = capacity;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < slots * 64; t += (uint64_t)gridDim.x * blockDim.x) {
        int bx, by, bz;
        block_coords(active[t >> 6], L, bx, by, bz);
        const int l = (int)(t & 63);
        const int node[3] = {L.origin[0] + 4 * bx + (l >> 4), L.origin[1] + 4 * by + ((l >> 2) & 3), L.origin[2] + 4 * bz + (l & 3)};
        float mass = 0.f, px = 0.f, py = 0.f, pz = 0.f;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    // base cell node - (i, j, k): its block's segment and cell range
                    int local;
                    const int32_t slot = node_slot(map, node[0] - i, node[1] - j, node[2] - k, L, local);
                    if (slot < 0) continue;
                    const int32_t seg = slot_seg[slot];
                    if (seg < 0) continue;
                    const uint32_t lo = cstart[(uint64_t)seg * 65 + local], hi = cstart[(uint64_t)seg * 65 + local + 1];
                    const float nf[3] = {(float)node[0], (float)node[1], (float)node[2]};
                    for (uint32_t q = lo; q < hi; ++q) {
                        const float4 r0 = rec[4 * q], r1 = rec[4 * q + 1], r2 = rec[4 * q + 2], r3 = rec[4 * q + 3];
                        const float tn[3] = {__fsub_rn(nf[0], r0.x), __fsub_rn(nf[1], r0.y), __fsub_rn(nf[2], r0.z)};
                        const float w = __fmul_rn(__fmul_rn(det_kernel(tn[0]), det_kernel(tn[1])), det_kernel(tn[2]));
                        mass = __fadd_rn(mass, __fmul_rn(w, r0.w));
                        // momentum: w (m v + A (x_i - x_p)), x_i - x_p = tn dx
                        const float d0 = tn[0] * L.dx, d1 = tn[1] * L.dx, d2 = tn[2] * L.dx;
                        const float A[9] = {r1.w, r2.x, r2.y, r2.z, r2.w, r3.x, r3.y, r3.z, r3.w};
                        px += w * (r1.x + A[0] * d0 + A[3] * d1 + A[6] * d2);
                        py += w * (r1.y + A[1] * d0 + A[4] * d1 + A[7] * d2);
                        pz += w * (r1.z + A[2] * d0 + A[5] * d1 + A[8] * d2);
                    }
                }
        grid[t] = make_float4(px, py, pz, mass);
    }
}

unsigned elem_blocks(uint64_t work) {
    uint64_t b = (work + ELEM_THREADS - 1) / ELEM_THREADS;
    uint64_t cap = (uint64_t)sm_count() * 8;
    if (b > cap) b = cap;
    return (unsigned)(b ? b : 1);
}

struct Scoped {
    sv_handle *h;
    const char *name;
    cudaEvent_t start = nullptr;
    Scoped(sv_handle *h_, const char *n) : h(h_), name(n) { timer_begin(h, name, &start); }
    ~Scoped() { timer_end(h, name, start); }
};

StepArgs make_args(sv_handle *h, float dt, float3 g) {
    StepArgs A;
    A.in = h->side[h->cur];
    A.out = h->side[h->cur ^ 1];
    A.mats = h->materials;
    A.scenes = h->scenes;
    A.counters = h->counters;
    A.perm = h->need_perm ? h->perm : nullptr;  // the state is not yet in the last binning's order
    A.seg_start = h->seg_start;
    A.seg_block = h->seg_block;
    A.map_cur = h->blockmap[h->map_cur];
    A.map_next = h->blockmap[h->map_next];
    A.grid_cur = h->grid[h->gcur];
    A.grid_next = h->grid[h->gcur ^ 1];
    A.self_latch = false;
    A.adt_pass = 0;
    A.keys_out = h->keys;
    A.defer_list = h->defer_list;
    A.pass_timer = nullptr;
    A.closure_img = nullptr;
    A.closure_hull = nullptr;
    A.adt = nullptr;
    A.fa = col::FrameArgs{};
    A.vcur = col::VariantTable{};
    A.vnext = col::VariantTable{};
    if (h->fin_active) {
        col::FrameArgs &f = A.fa;
        f.gravity = h->fin_scalars;
        f.factor = h->fin_scalars + 3;
        f.goal_both = h->fin_goal_both;
        f.goal_a = h->fin_goal_a, f.goal_b = h->fin_goal_b;
        f.nt = h->fin_nt;
        f.tri = h->fin_tri, f.tri_col = h->fin_tri_col, f.opp = h->fin_opp;
        f.vpos = h->fin_vpos, f.vnorm = h->fin_vnorm, f.tnorm = h->fin_tnorm, f.vvel = h->fin_vvel;
        f.fric = h->fin_fric, f.damp = h->fin_damp;
        f.leaf_start = h->fin_leaf_start, f.leaf_list = h->fin_leaf_list;
        for (int a = 0; a < 3; ++a) f.leaf_lo[a] = h->fin_leaf_lo[a], f.leaf_dim[a] = h->fin_leaf_dim[a];
        f.leaf_size = h->fin_leaf_size;
        f.forget = h->layout.dx * 2.2f;
        f.accept = h->layout.dx * 2.f;
        auto table = [&](int s) {
            col::VariantTable t;
            t.key = h->var_key[s], t.bits = h->var_bits[s], t.acc = h->var_acc[s], t.vel = h->var_vel[s];
            t.cap = h->var_cap;
            return t;
        };
        A.vcur = table(h->gcur);
        A.vnext = table(h->gcur ^ 1);
    }
    A.n = h->n;
    A.L = h->layout;
    A.dt = dt;
    A.gravity = g;
    return A;
}

unsigned particle_blocks(const sv_handle *h) { return (unsigned)sm_count() * (h->cta_per_sm ? h->cta_per_sm : 8); }

// Launches the particle kernel of MODE in the handle's position form, with
// the frame-input variant when one is loaded.
template <int MODE, uint32_t KSET = KSET_ALL> void launch_particles(sv_handle *h, const StepArgs &A, unsigned grid = 0) {
    const unsigned blocks = grid ? grid : particle_blocks(h);
    h->stop_latched = A.self_latch;
    if (MODE != MODE_ADVANCE && MODE != MODE_P2G && MODE != MODE_G2P_ONLY) h->force_limits_valid = false;
    if constexpr (MODE != MODE_G2P2G_LEARNED && MODE != MODE_G2P2G_ADAPTIVE) {
        if (h->fin_active) {
            if (h->layout.position_form) k_particles<true, MODE, true><<<blocks, PT, 0, h->stream>>>(A);
            else k_particles<false, MODE, true><<<blocks, PT, 0, h->stream>>>(A);
            return;
        }
    }
    if constexpr (MODE == MODE_G2P2G_LEARNED) {
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(k_particles<true, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, LEARNED_SMEM_BYTES);
            cudaFuncSetAttribute(k_particles<false, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, LEARNED_SMEM_BYTES);
            attr = true;
        }
        if (h->layout.position_form) k_particles<true, MODE><<<blocks, PT, LEARNED_SMEM_BYTES, h->stream>>>(A);
        else k_particles<false, MODE><<<blocks, PT, LEARNED_SMEM_BYTES, h->stream>>>(A);
        return;
    }
    if (h->layout.position_form) k_particles<true, MODE, false, false, KSET><<<blocks, PT, 0, h->stream>>>(A);
    else k_particles<false, MODE, false, false, KSET><<<blocks, PT, 0, h->stream>>>(A);
}

}  // namespace

int sm_count() {
    static int count = 0;
    if (!count) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
        if (count <= 0) count = 1;
    }
    return count;
}

cudaError_t launch_keys(sv_handle *h) {
    StepArgs A = make_args(h, 0.f, make_float3(0, 0, 0));
    Scoped s(h, "keys");
    if (h->layout.position_form) k_keys<true><<<elem_blocks(h->n), ELEM_THREADS, 0, h->stream>>>(A);
    else k_keys<false><<<elem_blocks(h->n), ELEM_THREADS, 0, h->stream>>>(A);
    h->keys_valid = true;
    h->stop_latched = false;  // may set ST_OUT_OF_GRID
    h->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_sort_and_segments(sv_handle *h) {
    cudaError_t err;
    if (h->n == 0) {
        err = cudaMemsetAsync(h->counters + C_NSEG, 0, sizeof(uint32_t), h->stream);
        if (err != cudaSuccess) return err;
        return cudaMemsetAsync(h->counters + C_NLIVE, 0, sizeof(uint32_t), h->stream);
    }
    {
        Scoped s(h, "radix_sort");
        err = radix_sort_pairs(h->keys, nullptr, h->sorted_keys, h->perm, h->n, h->layout.key_bits, h->sort_temp,
                               h->stream);
        if (err != cudaSuccess) return err;
        h->launches += radix_sort_launches(h->n, h->layout.key_bits);
        h->sorts += 1;
        h->need_perm = true;  // until a pass writes the state in the new order
    }
    Scoped s(h, "segments");
    uint32_t tiles = (uint32_t)((h->n + SEG_TILE - 1) / SEG_TILE);
    k_seg_count<<<tiles, ELEM_THREADS, 0, h->stream>>>(h->sorted_keys, h->n, h->tile_counts, h->counters);
    err = exclusive_scan_u32(h->tile_counts, h->tile_counts, tiles, h->scan_temp, h->stream);
    if (err != cudaSuccess) return err;
    k_seg_write<<<tiles, ELEM_THREADS, 0, h->stream>>>(h->sorted_keys, h->n, h->tile_counts, tiles, h->seg_start,
                                                       h->seg_block, h->counters);
    h->launches += 2 + scan_launches(tiles);
    return cudaGetLastError();
}

cudaError_t launch_activate(sv_handle *h, int which) {
    Scoped s(h, "activate");
    k_map_reset<<<elem_blocks(h->capacity), ELEM_THREADS, 0, h->stream>>>(h->blockmap[which], h->active[which], h->counters,
                                                                            which, h->capacity);
    k_latch<<<1, 1, 0, h->stream>>>(h->counters, which, -1, h->capacity);
    k_activate<<<elem_blocks(27 * h->n / 64 + 64), ELEM_THREADS, 0, h->stream>>>(
        h->seg_block, h->blockmap[which], h->active[which], h->capacity, h->layout, h->counters, which);
    k_latch<<<1, 1, 0, h->stream>>>(h->counters, -1, which, h->capacity);
    h->launches += 4;
    h->stop_latched = true;
    return cudaGetLastError();
}

cudaError_t launch_latch(sv_handle *h) {
    k_latch<<<1, 1, 0, h->stream>>>(h->counters, -1, -1, h->capacity);
    h->launches += 1;
    h->stop_latched = true;
    return cudaGetLastError();
}

cudaError_t launch_clear(sv_handle *h, int grid_side, int which) {
    Scoped s(h, "clear");
    k_clear_grid<<<elem_blocks(h->capacity * 64), ELEM_THREADS, 0, h->stream>>>(h->grid[grid_side], h->capacity, h->counters, which,
                                                                                  h->grid_sums + 4 * grid_side);
    h->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_limits_force(sv_handle *h, bool reduce) {
    Scoped s(h, "limits_force");
    auto *st = reinterpret_cast<adaptive::State *>(h->adt);
    if (reduce) {
        k_limits_force<<<elem_blocks(h->n), ELEM_THREADS, 0, h->stream>>>(h->side[h->cur], h->materials, h->n,
                                                                           h->layout.dx, st, h->counters);
        h->launches += 1;
    }
    k_dt_force<<<1, 1, 0, h->stream>>>(st, h->counters);
    h->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_g2p_only(sv_handle *h) {
    StepArgs A = make_args(h, 0.f, make_float3(0.f, 0.f, 0.f));
    A.adt = reinterpret_cast<adaptive::State *>(h->adt);
    A.keys_out = nullptr;
    Scoped s(h, "g2p");
    launch_particles<MODE_G2P_ONLY>(h, A);
    k_dt_integrate<<<1, 1, 0, h->stream>>>(A.adt, h->counters, h->layout.dx);
    h->launches += 2;
    h->vel_side = h->gcur;
    h->vel_map = h->map_cur;
    return cudaGetLastError();
}

// The next substep's steps as its k_dt_force will take them, from this
// substep's advance and the force limits its pass reduced (the push on a
// copy): when they differ from the ones its scatter assumed, that scatter is
// redone (p2g_redo).
__global__ void k_dt_next(adaptive::State *st, uint32_t *counters) {
    if (counters[C_STOP]) return;
    adaptive::State nx = *st;
    nx.sound = __uint_as_float(st->red_sound);
    nx.iso = __uint_as_float(st->red_iso);
    adaptive::push(nx);
    st->dt_b_next = adaptive::allowed(nx);
    st->p2g_redo = st->redo || st->dt_b_next != st->dt_spec_b;
    if (st->p2g_redo) counters[C_ADT_MISS] += 1;
}

cudaError_t launch_g2p2g_adaptive(sv_handle *h, float3 g, bool write_keys, bool use_perm) {
    auto *st = reinterpret_cast<adaptive::State *>(h->adt);
    StepArgs A = make_args(h, 0.f, g);
    A.adt = st;
    if (!write_keys) A.keys_out = nullptr;
    if (!use_perm) A.perm = nullptr;
    {
        Scoped s(h, "g2p2g_adaptive");
        A.adt_pass = 3;
        launch_particles<MODE_G2P2G_ADAPTIVE>(h, A);
        k_dt_integrate<<<1, 1, 0, h->stream>>>(st, h->counters, h->layout.dx);
    }
    {
        // the advance again at dt_c when the G2P's limits bound; then the
        // next substep's scatter again when any of its assumed steps was off
        Scoped s(h, "adaptive_redo");
        StepArgs R = A;
        R.adt_pass = 2;
        launch_particles<MODE_G2P_ADVANCE>(h, R, (unsigned)sm_count() * 5);
        k_dt_next<<<1, 1, 0, h->stream>>>(st, h->counters);
        k_clear_grid<<<elem_blocks(h->capacity * 64), ELEM_THREADS, 0, h->stream>>>(
            h->grid[h->gcur ^ 1], h->capacity, h->counters, h->map_next, h->grid_sums + 4 * (h->gcur ^ 1), &st->p2g_redo);
        StepArgs P = make_args(h, 0.f, g);
        P.adt = st;
        P.adt_pass = 4;
        P.in = h->side[h->cur ^ 1];  // the advanced state, in the binning's order
        P.perm = nullptr;
        P.keys_out = nullptr;
        P.map_next = h->blockmap[h->map_next];
        P.grid_next = h->grid[h->gcur ^ 1];
        launch_particles<MODE_P2G>(h, P, (unsigned)sm_count() * 5);
        k_adaptive_finish<<<1, 1, 0, h->stream>>>(st, h->counters, true);
    }
    h->launches += 7;
    h->vel_side = h->gcur;
    h->vel_map = h->map_cur;
    h->cur ^= 1;
    h->gcur ^= 1;
    h->map_cur = h->map_next;
    h->keys_valid = write_keys;
    h->need_perm = false;
    return cudaGetLastError();
}

cudaError_t launch_advance(sv_handle *h) {
    StepArgs A = make_args(h, 0.f, make_float3(0.f, 0.f, 0.f));
    A.adt = reinterpret_cast<adaptive::State *>(h->adt);
    Scoped s(h, "advance");
    launch_particles<MODE_ADVANCE>(h, A);
    k_adaptive_finish<<<1, 1, 0, h->stream>>>(A.adt, h->counters);
    h->launches += 2;
    h->cur ^= 1;
    h->keys_valid = true;
    h->need_perm = false;  // written in the binning's order
    return cudaGetLastError();
}

// Start of an adaptive substep: latches the stop bits of the substeps before
// it, then (unless stopped) keeps the adaptive state as it is now, to return
// to if this substep is redone after a particle left its claimed blocks -- so
// that the redo does not push its limits into the history twice.
__global__ void k_adaptive_begin(adaptive::State *st, adaptive::State *backup, uint32_t *counters) {
    const uint32_t stop = counters[C_STATUS] & STOP_MASK;
    counters[C_STOP] = stop;
    st->redo = 0, st->p2g_redo = 0;
    if (stop) return;
    *backup = *st;
    // k_limits_force reduces this substep's force limits unless the last
    // advance did
    if (!st->force_ready) st->red_sound = st->red_iso = __float_as_uint(adaptive::NONE);
}

cudaError_t launch_adaptive_begin(sv_handle *h) {
    k_adaptive_begin<<<1, 1, 0, h->stream>>>(reinterpret_cast<adaptive::State *>(h->adt),
                                             reinterpret_cast<adaptive::State *>(h->adt_backup), h->counters);
    h->launches += 1;
    h->stop_latched = true;
    return cudaGetLastError();
}

cudaError_t launch_p2g(sv_handle *h, float dt, float3 g) {
    StepArgs A = make_args(h, dt, g);
    A.map_next = h->blockmap[h->map_cur];
    A.grid_next = h->grid[h->gcur];
    A.keys_out = nullptr;
    A.vnext = A.vcur;  // the standalone scatter fills the current grid and variants
    if (h->adaptive_active) A.adt = reinterpret_cast<adaptive::State *>(h->adt);
    Scoped s(h, "p2g");
    launch_particles<MODE_P2G>(h, A);
    h->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_det_binning(sv_handle *h) {
    cudaError_t err;
    if (h->n == 0) return launch_sort_and_segments(h);
    {
        Scoped s(h, "radix_sort");
        k_det_order<<<elem_blocks(h->n), ELEM_THREADS, 0, h->stream>>>(h->side[h->cur].orig, h->keys, h->n, h->det_kbo,
                                                                       h->inv);
        err = radix_sort_pairs(h->det_kbo, nullptr, h->sorted_keys, h->det_orig, h->n, h->layout.key_bits, h->sort_temp,
                               h->stream);
        if (err != cudaSuccess) return err;
        k_det_perm<<<elem_blocks(h->n), ELEM_THREADS, 0, h->stream>>>(h->det_orig, h->inv, h->n, h->perm);
        h->launches += 2 + radix_sort_launches(h->n, h->layout.key_bits);
        h->sorts += 1;
        h->need_perm = true;
    }
    Scoped s(h, "segments");
    uint32_t tiles = (uint32_t)((h->n + SEG_TILE - 1) / SEG_TILE);
    k_seg_count<<<tiles, ELEM_THREADS, 0, h->stream>>>(h->sorted_keys, h->n, h->tile_counts, h->counters);
    err = exclusive_scan_u32(h->tile_counts, h->tile_counts, tiles, h->scan_temp, h->stream);
    if (err != cudaSuccess) return err;
    k_seg_write<<<tiles, ELEM_THREADS, 0, h->stream>>>(h->sorted_keys, h->n, h->tile_counts, tiles, h->seg_start,
                                                       h->seg_block, h->counters);
    h->launches += 2 + scan_launches(tiles);
    return cudaGetLastError();
}

cudaError_t launch_det_p2g(sv_handle *h, float dt, float3 g) {
    StepArgs A = make_args(h, dt, g);
    Scoped s(h, "p2g");
    const int which = h->map_cur;
    k_det_slot_reset<<<elem_blocks(h->capacity), ELEM_THREADS, 0, h->stream>>>(h->det_slot_seg, h->counters, which,
                                                                                 h->capacity);
    k_det_cells<<<elem_blocks(65 * std::min<uint64_t>(h->n, h->capacity)), ELEM_THREADS, 0, h->stream>>>(
        h->sorted_keys, h->seg_start, h->seg_block, h->blockmap[which], h->counters, h->det_cstart, h->det_slot_seg,
        h->det_seg_cap);
    if (h->layout.position_form) k_det_records<true><<<elem_blocks(h->n), ELEM_THREADS, 0, h->stream>>>(A, h->det_rec);
    else k_det_records<false><<<elem_blocks(h->n), ELEM_THREADS, 0, h->stream>>>(A, h->det_rec);
    k_det_gather<<<elem_blocks(h->capacity * 64), ELEM_THREADS, 0, h->stream>>>(
        h->det_rec, h->active[which], h->blockmap[which], h->det_slot_seg, h->det_cstart, h->grid[h->gcur], h->layout,
        h->counters, which, h->capacity);
    h->launches += 4;
    return cudaGetLastError();
}

cudaError_t launch_grid_update(sv_handle *h, bool clear_next, bool latch) {
    Scoped s(h, "grid_update");
    col::VariantTable var{};
    if (h->fin_active) {
        var.key = h->var_key[h->gcur], var.bits = h->var_bits[h->gcur];
        var.acc = h->var_acc[h->gcur], var.vel = h->var_vel[h->gcur], var.cap = h->var_cap;
        k_variant_meld<<<elem_blocks(h->var_cap), ELEM_THREADS, 0, h->stream>>>(var, h->grid[h->gcur],
                                                                                h->blockmap[h->map_cur], h->layout,
                                                                                h->counters);
        h->launches += 1;
    }
    const unsigned gu_blocks = (unsigned)std::min<uint64_t>((h->capacity * 64 + 2 * ELEM_THREADS - 1) / (2 * ELEM_THREADS),
                                                           (uint64_t)sm_count() * 4);
    k_grid_update<<<gu_blocks ? gu_blocks : 1, ELEM_THREADS, 0, h->stream>>>(
        h->grid[h->gcur], h->active[h->map_cur], clear_next ? h->grid[h->gcur ^ 1] : nullptr, h->capacity, h->layout,
        h->counters, h->map_cur, h->map_next, var, h->grid_sums + 4 * h->gcur, h->grid_sums + 4 * (h->gcur ^ 1));
    h->launches += 1;
    if (latch) {
        k_latch<<<1, 1, 0, h->stream>>>(h->counters, -1, -1, h->capacity);
        h->launches += 1;
        h->stop_latched = true;
    }
    return cudaGetLastError();
}

cudaError_t launch_clear_variants(sv_handle *h, int which) {
    if (!h->fin_active) return cudaSuccess;
    cudaError_t e;
    if ((e = cudaMemsetAsync(h->var_key[which], 0, (size_t)h->var_cap * sizeof(unsigned long long), h->stream)) ||
        (e = cudaMemsetAsync(h->var_bits[which], 0, (size_t)h->var_cap * col::VK * sizeof(uint32_t), h->stream)) ||
        (e = cudaMemsetAsync(h->var_acc[which], 0, (size_t)h->var_cap * col::VK * sizeof(float4), h->stream)))
        return e;
    return cudaSuccess;
}

cudaError_t launch_interpolate(sv_handle *h, double time) {
    if (!h->fin_active) return cudaSuccess;
    Scoped s(h, "interpolate");
    FinDev f;
    f.fps = h->fin_fps, f.frame = h->fin_frame, f.nv = h->fin_nv, f.nt = h->fin_nt;
    for (int a = 0; a < 3; ++a) f.g_a[a] = h->fin_g_a[a], f.g_b[a] = h->fin_g_b[a];
    f.va = h->fin_va, f.vb = h->fin_vb, f.fr_a = h->fin_fr_a, f.fr_b = h->fin_fr_b, f.dm_a = h->fin_dm_a, f.dm_b = h->fin_dm_b;
    f.tri = h->fin_tri, f.vt_start = h->fin_vt_start, f.vt_list = h->fin_vt_list;
    f.scalars = h->fin_scalars;
    f.vpos = h->fin_vpos, f.vnorm = h->fin_vnorm, f.tnorm = h->fin_tnorm, f.fric = h->fin_fric, f.damp = h->fin_damp;
    const adaptive::State *st = h->adaptive_active ? reinterpret_cast<const adaptive::State *>(h->adt) : nullptr;
    k_interp_factor<<<1, 1, 0, h->stream>>>(f, time, st, h->counters);
    h->launches += 1;
    if (h->fin_nt) {
        const unsigned b = elem_blocks(std::max<uint64_t>(3ull * h->fin_nv, h->fin_nt));
        k_interp_vertices<<<b, ELEM_THREADS, 0, h->stream>>>(f, h->counters);
        k_interp_triangles<<<elem_blocks(h->fin_nt), ELEM_THREADS, 0, h->stream>>>(f);
        k_interp_vertex_normals<<<elem_blocks(h->fin_nv), ELEM_THREADS, 0, h->stream>>>(f);
        h->launches += 3;
    }
    return cudaGetLastError();
}

cudaError_t launch_g2p_advance(sv_handle *h, float dt) {
    StepArgs A = make_args(h, dt, make_float3(0.f, 0.f, 0.f));
    Scoped s(h, "g2p_advance");
    launch_particles<MODE_G2P_ADVANCE>(h, A);
    k_finish<<<1, 1, 0, h->stream>>>(h->counters);
    h->launches += 2;
    h->vel_side = h->gcur;
    h->vel_map = h->map_cur;
    h->cur ^= 1;
    h->keys_valid = true;
    return cudaGetLastError();
}

cudaError_t launch_g2p2g(sv_handle *h, float dt, float3 g, bool write_keys, bool use_perm) {
    StepArgs A = make_args(h, dt, g);
    if (!write_keys) A.keys_out = nullptr;
    if (!use_perm) A.perm = nullptr;
    A.self_latch = !h->fin_active;
    Scoped s(h, "g2p2g");
    if (h->closure_mode == 1 && h->cl_trained && !h->fin_active) {
        A.closure_img = h->cl_img;
        A.closure_hull = reinterpret_cast<const closure::Hull *>(h->cl_hull);
        launch_particles<MODE_G2P2G_LEARNED>(h, A);
    } else if (!h->fin_active) {
        // the fused pass without fp64 code, as one resident wave taking
        // segments from the queue, then its fp64 pass, which latches the
        // stop bits for both (see k_particles)
        A.pass_timer = h->pass_timer;
        StepArgs M = A;
        M.self_latch = false;
        const unsigned wave = (unsigned)sm_count() * SV_PARTICLE_CTAS_PER_SM;
        if ((h->kind_set & ~KSET_SOLID_PLASTIC) == 0) launch_particles<MODE_G2P2G, KSET_SOLID_PLASTIC>(h, M, wave);
        else if ((h->kind_set & ~KSET_FLUID_NH) == 0) launch_particles<MODE_G2P2G, KSET_FLUID_NH>(h, M, wave);
        else launch_particles<MODE_G2P2G>(h, M, wave);
        if (h->layout.position_form) k_particles<true, MODE_G2P2G, false, true><<<sm_count(), PT, 0, h->stream>>>(A);
        else k_particles<false, MODE_G2P2G, false, true><<<sm_count(), PT, 0, h->stream>>>(A);
        h->stop_latched = A.self_latch;
        h->launches += 1;
    } else {
        launch_particles<MODE_G2P2G>(h, A);
    }
    h->launches += 1;
    if (!A.self_latch) {
        k_finish<<<1, 1, 0, h->stream>>>(h->counters);
        h->launches += 1;
    }
    h->vel_side = h->gcur;
    h->vel_map = h->map_cur;
    h->cur ^= 1;
    h->gcur ^= 1;
    h->map_cur = h->map_next;
    h->keys_valid = write_keys;
    return cudaGetLastError();
}

}  // namespace sv
