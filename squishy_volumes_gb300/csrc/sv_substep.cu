// sv_substep.cu -- the MPM substep on the GPU.
//
// Reference: Squishy Volumes rust/crates/cpu, one pass of the phase cycle
// (cpu/src/phase/mod.rs:27-41) with adaptive time steps off:
//   Sort -> ExternalForce -> UpdateGridNodes -> ScatterMomentum -> MeldGrid
//   -> CollectVelocity -> AdvanceParticles -> CullParticles.
// GB300 design:
//   keys      binning key per particle (written by the previous substep's G2P)
//   sort      stable radix sort of the keys -> permutation; 4^3-block segments
//   activate  claim the grid blocks each particle block touches (dense block
//             index -> slot), clear them
//   p2g       one CTA per particle block: stress + APIC momentum accumulated in
//             a shared-memory 6^3-node halo tile, flushed with float4 atomics
//             (ScatterMomentum, scatter_momentum.rs:22-93; the external force,
//             external_force.rs:17-50, is applied on the fly)
//   grid      momentum -> velocity (MeldGrid, meld_grid.rs:16-69) + optional
//             boundary plane
//   g2p       one CTA per particle block: the 6^3 velocity tile staged in shared
//             memory, v/C gather (collect_velocity.rs:19-75), x/F advance and
//             plasticity (advance_particles.rs:17-93), cull
//             (cull_particles.rs:17-41); writes the next state in sorted order
//             and the next binning keys.
#include <cstdio>

#include "sv_internal.h"
#include "sv_sort.cuh"

namespace sv {

namespace {

constexpr int P2G_THREADS = 256;
constexpr int G2P_THREADS = 256;
constexpr int ELEM_THREADS = 256;
constexpr int SEG_TILE = 2048;  // elements per tile of the segment builder
constexpr int SEG_ITEMS = SEG_TILE / ELEM_THREADS;

// Shared halo tile of 6^3 nodes.  Strides chosen so that the 27 stencil
// offsets of one cell land in 27 distinct banks (9i + 3j + k mod 32).
constexpr int TS_Z = 1, TS_Y = 35, TS_X = 233;
constexpr int TILE_PLANE = 5 * TS_X + 5 * TS_Y + 5 * TS_Z + 1;  // 1341

struct StepArgs {
    ParticleArrays in, out;
    const Material *mats;
    uint32_t *counters;
    const uint32_t *perm;
    const uint32_t *seg_start;
    const uint32_t *seg_block;
    const int32_t *blockmap;
    float4 *grid;
    uint32_t *keys_out;
    uint64_t n;
    GridLayout L;
    float dt;
    float3 gravity;
};

__device__ __forceinline__ uint32_t stopped(const uint32_t *counters) {
    return *(volatile const uint32_t *)&counters[C_STOP];
}

__device__ __forceinline__ void block_coords(uint32_t b, const GridLayout &L, int &bx, int &by, int &bz) {
    bz = (int)(b % (uint32_t)L.nb[2]);
    uint32_t r = b / (uint32_t)L.nb[2];
    by = (int)(r % (uint32_t)L.nb[1]);
    bx = (int)(r / (uint32_t)L.nb[1]);
}

// Neighbour t in {0,1}^3 (bit 2 = x, bit 1 = y, bit 0 = z) of block b.
__device__ __forceinline__ uint32_t neighbour_block(uint32_t b, int t, const GridLayout &L) {
    return b + (uint32_t)(((t >> 2) & 1) * L.nb[1] * L.nb[2] + ((t >> 1) & 1) * L.nb[2] + (t & 1));
}

// Binning key of a base cell given in global node coordinates.
__device__ __forceinline__ uint32_t cell_key(int cx, int cy, int cz, const GridLayout &L, bool &ok) {
    int lx = cx - L.origin[0], ly = cy - L.origin[1], lz = cz - L.origin[2];
    ok = lx >= 0 && ly >= 0 && lz >= 0 && (lx >> 2) < L.nb[0] - 1 && (ly >> 2) < L.nb[1] - 1 &&
         (lz >> 2) < L.nb[2] - 1;
    if (!ok) return SENTINEL_KEY;
    uint32_t block = ((uint32_t)(lx >> 2) * (uint32_t)L.nb[1] + (uint32_t)(ly >> 2)) * (uint32_t)L.nb[2] + (uint32_t)(lz >> 2);
    return block << 6 | (uint32_t)((lx & 3) << 4 | (ly & 3) << 2 | (lz & 3));
}

// Particle position in grid units: base cell (global node index of the
// lowest stencil node, floor(x/dx - 0.5) as kernels.rs:46-49) and fx = x/dx -
// base in [0.5, 1.5).
template <bool CELL>
__device__ __forceinline__ void grid_position(const ParticleArrays &a, uint32_t p, const float4 &pos, float dx,
                                              int base[3], float fx[3]) {
    if (!CELL) {
        float q[3] = {pos.x / dx, pos.y / dx, pos.z / dx};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float b = floorf(q[k] - 0.5f);
            base[k] = (int)b;
            fx[k] = q[k] - b;
        }
    } else {
        int4 c = a.cell[p];
        float o[3] = {pos.x, pos.y, pos.z};
        int ci[3] = {c.x, c.y, c.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            bool hi = o[k] >= 0.5f;
            base[k] = ci[k] - (hi ? 0 : 1);
            fx[k] = o[k] + (hi ? 0.f : 1.f);
        }
    }
}

__device__ __forceinline__ float sel3(const float v[3], int i) { return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]); }

__device__ __forceinline__ void load_mat9(const float *planes, uint64_t n, uint32_t p, m3f &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) m.a[k] = planes[(uint64_t)k * n + p];
}
__device__ __forceinline__ void store_mat9(float *planes, uint64_t n, uint64_t i, const m3f &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) planes[(uint64_t)k * n + i] = m.a[k];
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
            grid_position<CELL>(A.in, (uint32_t)i, pos, A.L.dx, base, fx);
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

// Writes segment starts in key order: thread t of the tile owns the
// SEG_ITEMS consecutive elements [base + t*SEG_ITEMS, ...).
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

// ------------------------------------------------------------------ grid blocks
__global__ void __launch_bounds__(ELEM_THREADS)
    k_reset_blockmap(int32_t *blockmap, const uint32_t *active, uint32_t *counters) {
    uint32_t prev = counters[C_NSLOT_PREV];
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < prev; s += gridDim.x * blockDim.x)
        blockmap[active[s]] = -1;
}

__global__ void k_latch(uint32_t *counters, int reset_slots) {
    if (reset_slots) counters[C_NSLOT] = 0;
    counters[C_STOP] = counters[C_STATUS] & STOP_MASK;
}

__global__ void __launch_bounds__(ELEM_THREADS)
    k_activate(const uint32_t *seg_block, int32_t *blockmap, uint32_t *active, uint64_t capacity, GridLayout L,
               uint32_t *counters) {
    if (stopped(counters)) return;
    uint32_t nseg = counters[C_NSEG];
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (uint64_t)nseg * 8;
         t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = neighbour_block(seg_block[t >> 3], (int)(t & 7), L);
        if (atomicCAS(&blockmap[b], -1, -2) == -1) {
            uint32_t slot = atomicAdd(&counters[C_NSLOT], 1u);
            if (slot < capacity) {
                active[slot] = b;
                blockmap[b] = (int32_t)slot;
            } else {
                blockmap[b] = -1;
                atomicOr(&counters[C_STATUS], ST_CAPACITY);
            }
        }
    }
}

__global__ void __launch_bounds__(ELEM_THREADS) k_clear_grid(float4 *grid, uint64_t capacity, uint32_t *counters) {
    uint64_t slots = counters[C_NSLOT];
    if (slots > capacity) slots = capacity;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < slots * 64; i += (uint64_t)gridDim.x * blockDim.x)
        grid[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ------------------------------------------------------------------ P2G
template <bool CELL> __global__ void __launch_bounds__(P2G_THREADS) k_p2g(StepArgs A) {
    __shared__ float tile[4][TILE_PLANE];
    __shared__ int32_t nslot[8];
    if (stopped(A.counters)) return;
    const uint32_t nseg = A.counters[C_NSEG];
    const float dx = A.L.dx;
    const float scaling = A.dt * 4.f / (dx * dx);  // scatter_momentum.rs:24-25
    const int lane = threadIdx.x & 31;
    for (uint32_t seg = blockIdx.x; seg < nseg; seg += gridDim.x) {
        const uint32_t b = A.seg_block[seg];
        const uint32_t start = A.seg_start[seg], end = A.seg_start[seg + 1];
        int bx, by, bz;
        block_coords(b, A.L, bx, by, bz);
        const int ox = A.L.origin[0] + 4 * bx, oy = A.L.origin[1] + 4 * by, oz = A.L.origin[2] + 4 * bz;
        for (int i = threadIdx.x; i < 4 * TILE_PLANE; i += P2G_THREADS) (&tile[0][0])[i] = 0.f;
        if (threadIdx.x < 8) nslot[threadIdx.x] = A.blockmap[neighbour_block(b, threadIdx.x, A.L)];
        __syncthreads();
        for (uint32_t i = start + threadIdx.x; i < end; i += P2G_THREADS) {
            const uint32_t p = A.perm[i];
            const float4 pos = A.in.pos[p];
            float4 vel = A.in.vel[p];
            const uint32_t packed = __float_as_uint(pos.w);
            const Material mat = A.mats[packed >> MATERIAL_SHIFT];
            int base[3];
            float fx[3];
            grid_position<CELL>(A.in, p, pos, dx, base, fx);
            m3f F, C;
            load_mat9(A.in.F, A.n, p, F);
            load_mat9(A.in.C, A.n, p, C);
            // external_force.rs:17-50: v += dt g (before P2G)
            vel.x += A.dt * A.gravity.x, vel.y += A.dt * A.gravity.y, vel.z += A.dt * A.gravity.z;
            const float J = det3(F);
            m3f R;
            float hard = 1.f;
            if (mat.kind == KIND_FIXED_COROTATED || mat.kind == KIND_SNOW) {
                m3f U, V;
                float S[3];
                svd3<float>(F, U, S, V, 6);
                R = mat_mul_bt(U, V);
                if (mat.kind == KIND_SNOW) hard = expf(mat.xi * (1.f - vel.w));
            }
            const m3f P = piola(mat, F, R, J, hard);
            // A = m C - s V0 P F^T [- s J V0 sigma_visc]
            const m3f PFt = mat_mul_bt(P, F);
            const float sv0 = scaling * mat.initial_volume;
            m3f Aff;
#pragma unroll
            for (int k = 0; k < 9; ++k) Aff.a[k] = mat.mass * C.a[k] - sv0 * PFt.a[k];
            if (mat.use_viscosity) {
                // util/src/elastic.rs:659-677: 2 mu_d sym(C) + mu_b tr(C) I
                const float sj = sv0 * J;
                const float tr = C.a[0] + C.a[4] + C.a[8];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        float s = mat.visc_dynamic * (C.a[c * 3 + r] + C.a[r * 3 + c]) + (r == c ? mat.visc_bulk * tr : 0.f);
                        Aff.a[c * 3 + r] -= sj * s;
                    }
            }
            const float mvx = mat.mass * vel.x, mvy = mat.mass * vel.y, mvz = mat.mass * vel.z;
            float wx[3], wy[3], wz[3], dX[3], dY[3], dZ[3];
            bspline_weights(fx[0], wx);
            bspline_weights(fx[1], wy);
            bspline_weights(fx[2], wz);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                dX[k] = ((float)k - fx[0]) * dx;
                dY[k] = ((float)k - fx[1]) * dx;
                dZ[k] = ((float)k - fx[2]) * dx;
            }
            const int tb = (base[0] - ox) * TS_X + (base[1] - oy) * TS_Y + (base[2] - oz) * TS_Z;
            // Lane-rotated stencil order: lanes of one cell hit 27 different nodes.
            int o = lane % 27;
#pragma unroll 3
            for (int q = 0; q < 27; ++q) {
                const int ii = o / 9, jj = (o / 3) % 3, kk = o % 3;
                const float w = sel3(wx, ii) * sel3(wy, jj) * sel3(wz, kk);
                const float ddx = sel3(dX, ii), ddy = sel3(dY, jj), ddz = sel3(dZ, kk);
                const float px = w * (mvx + Aff.a[0] * ddx + Aff.a[3] * ddy + Aff.a[6] * ddz);
                const float py = w * (mvy + Aff.a[1] * ddx + Aff.a[4] * ddy + Aff.a[7] * ddz);
                const float pz = w * (mvz + Aff.a[2] * ddx + Aff.a[5] * ddy + Aff.a[8] * ddz);
                const int t = tb + ii * TS_X + jj * TS_Y + kk * TS_Z;
                atomicAdd(&tile[0][t], w * mat.mass);
                atomicAdd(&tile[1][t], px);
                atomicAdd(&tile[2][t], py);
                atomicAdd(&tile[3][t], pz);
                o = o == 26 ? 0 : o + 1;
            }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < 216; t += P2G_THREADS) {
            const int tx = t / 36, ty = (t / 6) % 6, tz = t % 6;
            const int s = tx * TS_X + ty * TS_Y + tz * TS_Z;
            const float m = tile[0][s];
            if (m != 0.f || tile[1][s] != 0.f || tile[2][s] != 0.f || tile[3][s] != 0.f) {
                const int nb = (tx >> 2) * 4 + (ty >> 2) * 2 + (tz >> 2);
                const int32_t slot = nslot[nb];
                if (slot >= 0) {
                    float4 *g = &A.grid[(uint64_t)slot * 64 + ((tx & 3) * 16 + (ty & 3) * 4 + (tz & 3))];
                    atomicAdd(g, make_float4(tile[1][s], tile[2][s], tile[3][s], m));
                } else {
                    atomicOr(&A.counters[C_STATUS], ST_CAPACITY);
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ grid update
__global__ void __launch_bounds__(ELEM_THREADS)
    k_grid_update(float4 *grid, const uint32_t *active, uint64_t capacity, GridLayout L, uint32_t *counters) {
    if (stopped(counters)) return;
    uint64_t slots = counters[C_NSLOT];
    if (slots > capacity) slots = capacity;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < slots * 64; i += (uint64_t)gridDim.x * blockDim.x) {
        float4 g = grid[i];
        // meld_grid.rs:61-66: v = p / m, or 0 when m <= 0
        float m = g.w;
        float vx = 0.f, vy = 0.f, vz = 0.f;
        if (m > 0.f) vx = g.x / m, vy = g.y / m, vz = g.z / m;
        if (L.ground_mode != 0) {
            // Addition (not in the reference): boundary plane at node height.
            int bx, by, bz;
            block_coords(active[i >> 6], L, bx, by, bz);
            int l = (int)(i & 63);
            int node[3] = {L.origin[0] + 4 * bx + (l >> 4), L.origin[1] + 4 * by + ((l >> 2) & 3), L.origin[2] + 4 * bz + (l & 3)};
            if ((float)node[L.ground_axis] * L.dx <= L.ground_height) {
                float *vc[3] = {&vx, &vy, &vz};
                if (L.ground_mode == 1) vx = vy = vz = 0.f;
                else if (*vc[L.ground_axis] < 0.f) *vc[L.ground_axis] = 0.f;
            }
        }
        grid[i] = make_float4(vx, vy, vz, m);
    }
}

// ------------------------------------------------------------------ G2P
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
}

template <bool CELL> __global__ void __launch_bounds__(G2P_THREADS) k_g2p(StepArgs A) {
    __shared__ float4 gv[216];
    __shared__ int32_t nslot[8];
    if (stopped(A.counters)) {
        // Keep the state as it is (identity copy) so the buffer swap is a no-op.
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += (uint64_t)gridDim.x * blockDim.x)
            copy_particle(A.in, A.out, A.n, i, i, CELL);
        return;
    }
    const uint32_t nseg = A.counters[C_NSEG];
    const uint32_t nlive = A.counters[C_NLIVE];
    // Tombstoned particles (sorted last) are carried over unchanged.
    for (uint64_t i = nlive + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += (uint64_t)gridDim.x * blockDim.x) {
        copy_particle(A.in, A.out, A.n, A.perm[i], i, CELL);
        A.keys_out[i] = SENTINEL_KEY;
    }
    const float dx = A.L.dx;
    uint32_t fp64_count = 0;
    for (uint32_t seg = blockIdx.x; seg < nseg; seg += gridDim.x) {
        const uint32_t b = A.seg_block[seg];
        const uint32_t start = A.seg_start[seg], end = A.seg_start[seg + 1];
        int bx, by, bz;
        block_coords(b, A.L, bx, by, bz);
        const int ox = A.L.origin[0] + 4 * bx, oy = A.L.origin[1] + 4 * by, oz = A.L.origin[2] + 4 * bz;
        if (threadIdx.x < 8) nslot[threadIdx.x] = A.blockmap[neighbour_block(b, threadIdx.x, A.L)];
        __syncthreads();
        for (int t = threadIdx.x; t < 216; t += G2P_THREADS) {
            const int tx = t / 36, ty = (t / 6) % 6, tz = t % 6;
            const int32_t slot = nslot[(tx >> 2) * 4 + (ty >> 2) * 2 + (tz >> 2)];
            gv[t] = slot >= 0 ? A.grid[(uint64_t)slot * 64 + ((tx & 3) * 16 + (ty & 3) * 4 + (tz & 3))]
                              : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        for (uint32_t i = start + threadIdx.x; i < end; i += G2P_THREADS) {
            const uint32_t p = A.perm[i];
            float4 pos = A.in.pos[p];
            uint32_t packed = __float_as_uint(pos.w);
            const Material mat = A.mats[packed >> MATERIAL_SHIFT];
            int base[3];
            float fx[3];
            grid_position<CELL>(A.in, p, pos, dx, base, fx);
            float wx[3], wy[3], wz[3];
            bspline_weights(fx[0], wx);
            bspline_weights(fx[1], wy);
            bspline_weights(fx[2], wz);
            const int t0 = (base[0] - ox) * 36 + (base[1] - oy) * 6 + (base[2] - oz);
            // collect_velocity.rs:50-72
            float v[3] = {0.f, 0.f, 0.f};
            m3f C;
#pragma unroll
            for (int k = 0; k < 9; ++k) C.a[k] = 0.f;
#pragma unroll
            for (int ii = 0; ii < 3; ++ii) {
                const float ddx = ((float)ii - fx[0]) * dx;
#pragma unroll
                for (int jj = 0; jj < 3; ++jj) {
                    const float ddy = ((float)jj - fx[1]) * dx;
                    const float wxy = wx[ii] * wy[jj];
#pragma unroll
                    for (int kk = 0; kk < 3; ++kk) {
                        const float ddz = ((float)kk - fx[2]) * dx;
                        const float w = wxy * wz[kk];
                        const float4 g = gv[t0 + ii * 36 + jj * 6 + kk];
                        const float gx = g.x * w, gy = g.y * w, gz = g.z * w;
                        v[0] += gx, v[1] += gy, v[2] += gz;
                        C.a[0] += gx * ddx, C.a[1] += gy * ddx, C.a[2] += gz * ddx;
                        C.a[3] += gx * ddy, C.a[4] += gy * ddy, C.a[5] += gz * ddy;
                        C.a[6] += gx * ddz, C.a[7] += gy * ddz, C.a[8] += gz * ddz;
                    }
                }
            }
            const float cscale = 4.f / dx / dx;
#pragma unroll
            for (int k = 0; k < 9; ++k) C.a[k] *= cscale;
            // advance_particles.rs:39-41: x += v dt, F += C F dt
            m3f F;
            load_mat9(A.in.F, A.n, p, F);
            {
                m3f CF = mat_mul(C, F);
#pragma unroll
                for (int k = 0; k < 9; ++k) F.a[k] += CF.a[k] * A.dt;
            }
            int4 cell = make_int4(0, 0, 0, 0);
            if (!CELL) {
                pos.x += v[0] * A.dt, pos.y += v[1] * A.dt, pos.z += v[2] * A.dt;
            } else {
                cell = A.in.cell[p];
                float o[3] = {pos.x + v[0] * A.dt / dx, pos.y + v[1] * A.dt / dx, pos.z + v[2] * A.dt / dx};
                int ci[3] = {cell.x, cell.y, cell.z};
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float fl = floorf(o[k]);
                    ci[k] += (int)fl;
                    o[k] -= fl;
                    if (o[k] >= 1.f) o[k] = 0.f, ci[k] += 1;  // rounding guard
                }
                pos.x = o[0], pos.y = o[1], pos.z = o[2];
                cell = make_int4(ci[0], ci[1], ci[2], 0);
            }
            // plasticity (advance_particles.rs:42-86) and energy
            float plastic_j = 1.f;
            if (mat.kind == KIND_SNOW) plastic_j = A.in.vel[p].w;
            float energy = 0.f;
            const uint32_t kind = mat.kind;
            if (kind != KIND_NEO_HOOKEAN) {
                m3f U, V;
                float S[3];
                svd3<float>(F, U, S, V, 6);
                float det = det3(F);
                bool redo = false;
                if (A.L.svd_policy >= 1 && det < 0.05f) redo = true;
                if (A.L.svd_policy >= 2) {
                    float g = fminf(fabsf(S[0] - S[1]), fminf(fabsf(S[1] - S[2]), fabsf(S[0] - S[2])));
                    if (g < 1e-4f) redo = true;
                }
                if (redo) {
                    m3d Fd, Ud, Vd;
                    double Sd[3];
#pragma unroll
                    for (int k = 0; k < 9; ++k) Fd.a[k] = (double)F.a[k];
                    svd3<double>(Fd, Ud, Sd, Vd, 12);
#pragma unroll
                    for (int k = 0; k < 9; ++k) U.a[k] = (float)Ud.a[k], V.a[k] = (float)Vd.a[k];
#pragma unroll
                    for (int k = 0; k < 3; ++k) S[k] = (float)Sd[k];
                    ++fp64_count;
                }
                if (kind == KIND_SAND) {
                    // advance_particles.rs:48-71 (Drucker-Prager in Hencky strain)
                    if (mat.mu > 0.f) {
                        float e[3] = {logf(S[0]), logf(S[1]), logf(S[2])};
                        float e_tr = e[0] + e[1] + e[2];
                        float eh[3] = {e[0] - e_tr / 3.f, e[1] - e_tr / 3.f, e[2] - e_tr / 3.f};
                        float ehn = sqrtf(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]);
                        if (e_tr < 0.f && ehn > 0.f) {
                            float dg = ehn + (3.f * mat.lambda + 2.f * mat.mu) / 2.f / mat.mu * e_tr * mat.alpha;
                            if (dg > 0.f) {
                                float s[3];
#pragma unroll
                                for (int k = 0; k < 3; ++k) s[k] = expf(e[k] - dg / ehn * eh[k]);
                                F = recompose(U, s, V);
                            }
                        } else {
                            F = mat_mul_bt(U, V);
                        }
                    }
                } else if (kind == KIND_FLUID) {
                    // advance_particles.rs:77-85
                    float g = powf(S[0] * S[1] * S[2], 1.f / 3.f);
                    float s[3] = {g, g, g};
                    F = recompose(U, s, V);
                } else if (kind == KIND_SNOW) {
                    float s[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) s[k] = fminf(fmaxf(S[k], 1.f - mat.theta_c), 1.f + mat.theta_s);
                    plastic_j = plastic_j * (S[0] * S[1] * S[2]) / (s[0] * s[1] * s[2]);
                    F = recompose(U, s, V);
                }
                if (kind == KIND_FIXED_COROTATED || kind == KIND_SNOW) {
                    // psi = mu |F - R|^2 + lambda/2 (J - 1)^2 with hardening for snow
                    const float h = kind == KIND_SNOW ? expf(mat.xi * (1.f - plastic_j)) : 1.f;
                    const m3f Rm = mat_mul_bt(U, V);
                    float d2 = 0.f;
#pragma unroll
                    for (int k = 0; k < 9; ++k) d2 += (F.a[k] - Rm.a[k]) * (F.a[k] - Rm.a[k]);
                    const float Jn = det3(F);
                    energy = mat.mu * h * d2 + mat.lambda * h / 2.f * (Jn - 1.f) * (Jn - 1.f);
                }
            }
            const float Jn = det3(F);
            if (kind == KIND_FLUID) {
                // util/src/elastic.rs:546-553 inviscid energy
                float K = mat.bulk_modulus, gm = (float)mat.exponent;
                float at_rest = K * (1.f - 1.f / (1.f - gm));
                energy = K * (Jn - powi_f(Jn, 1 - mat.exponent) / (1.f - gm)) - at_rest;
            } else {
                if (!(Jn > 0.f)) {
                    // try_elastic_energy_neo_hookean: J <= 0 -> FAILED (advance_particles.rs:73-74)
                    packed |= SV_FAILED;
                    atomicOr(&A.counters[C_STATUS], ST_INVERTED);
                } else if (kind == KIND_NEO_HOOKEAN || kind == KIND_SAND) {
                    // util/src/elastic.rs:233-241
                    float I2 = 0.f;
#pragma unroll
                    for (int k = 0; k < 9; ++k) I2 += F.a[k] * F.a[k];
                    float lj = logf(Jn);
                    energy = mat.mu / 2.f * (I2 - 3.f) - mat.mu * lj + mat.lambda / 2.f * lj * lj;
                }
            }
            // cull_particles.rs:17-41: strict domain bounds
            bool inside;
            if (!CELL) {
                inside = pos.x > A.L.domain_min[0] && pos.x < A.L.domain_max[0] && pos.y > A.L.domain_min[1] &&
                         pos.y < A.L.domain_max[1] && pos.z > A.L.domain_min[2] && pos.z < A.L.domain_max[2];
            } else {
                double q[3] = {(double)cell.x + pos.x, (double)cell.y + pos.y, (double)cell.z + pos.z};
                inside = true;
#pragma unroll
                for (int k = 0; k < 3; ++k) inside = inside && q[k] > A.L.dmin_cells[k] && q[k] < A.L.dmax_cells[k];
            }
            if (!inside) packed |= SV_TOMBSTONED;
            uint32_t key = SENTINEL_KEY;
            if (!(packed & SV_TOMBSTONED)) {
                int nbase[3];
                float nfx[3];
                if (!CELL) {
                    float4 np = pos;
                    grid_position<false>(A.in, p, np, dx, nbase, nfx);
                } else {
                    float o[3] = {pos.x, pos.y, pos.z};
                    int ci[3] = {cell.x, cell.y, cell.z};
#pragma unroll
                    for (int k = 0; k < 3; ++k) nbase[k] = ci[k] - (o[k] >= 0.5f ? 0 : 1);
                }
                bool ok;
                key = cell_key(nbase[0], nbase[1], nbase[2], A.L, ok);
                if (!ok) atomicOr(&A.counters[C_STATUS], ST_OUT_OF_GRID);
            }
            pos.w = __uint_as_float(packed);
            A.out.pos[i] = pos;
            if (CELL) A.out.cell[i] = cell;
            A.out.vel[i] = make_float4(v[0], v[1], v[2], plastic_j);
            store_mat9(A.out.C, A.n, i, C);
            store_mat9(A.out.F, A.n, i, F);
            A.out.energy[i] = energy;
            A.out.orig[i] = A.in.orig[p];
            A.keys_out[i] = key;
        }
        __syncthreads();
    }
    // count fp64 SVDs (one atomic per warp)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fp64_count += __shfl_xor_sync(0xffffffffu, fp64_count, o);
    if ((threadIdx.x & 31) == 0 && fp64_count) atomicAdd(&A.counters[C_FP64], fp64_count);
}

__global__ void k_finish(uint32_t *counters, uint64_t capacity) {
    uint32_t slots = counters[C_NSLOT];
    counters[C_NSLOT_PREV] = slots < capacity ? slots : (uint32_t)capacity;
    if (!counters[C_STOP]) counters[C_SUBSTEPS] += 1;
}

StepArgs make_args(sv_handle *h, float dt, float3 g) {
    StepArgs A;
    A.in = h->side[h->cur];
    A.out = h->side[h->cur ^ 1];
    A.mats = h->materials;
    A.counters = h->counters;
    A.perm = h->perm;
    A.seg_start = h->seg_start;
    A.seg_block = h->seg_block;
    A.blockmap = h->blockmap;
    A.grid = h->grid;
    A.keys_out = h->keys;
    A.n = h->n;
    A.L = h->layout;
    A.dt = dt;
    A.gravity = g;
    return A;
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

cudaError_t launch_grid_activate(sv_handle *h) {
    Scoped s(h, "activate");
    k_reset_blockmap<<<elem_blocks(h->capacity), ELEM_THREADS, 0, h->stream>>>(h->blockmap, h->active_blocks, h->counters);
    k_latch<<<1, 1, 0, h->stream>>>(h->counters, 1);
    k_activate<<<elem_blocks(8 * h->n / 64 + 64), ELEM_THREADS, 0, h->stream>>>(
        h->seg_block, h->blockmap, h->active_blocks, h->capacity, h->layout, h->counters);
    k_clear_grid<<<elem_blocks(h->capacity * 64), ELEM_THREADS, 0, h->stream>>>(h->grid, h->capacity, h->counters);
    k_latch<<<1, 1, 0, h->stream>>>(h->counters, 0);
    h->launches += 5;
    return cudaGetLastError();
}

cudaError_t launch_p2g(sv_handle *h, float dt, float3 g) {
    StepArgs A = make_args(h, dt, g);
    Scoped s(h, "p2g");
    unsigned blocks = (unsigned)sm_count() * 6;
    if (h->layout.position_form) k_p2g<true><<<blocks, P2G_THREADS, 0, h->stream>>>(A);
    else k_p2g<false><<<blocks, P2G_THREADS, 0, h->stream>>>(A);
    h->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_grid_update(sv_handle *h) {
    Scoped s(h, "grid_update");
    k_grid_update<<<elem_blocks(h->capacity * 64), ELEM_THREADS, 0, h->stream>>>(h->grid, h->active_blocks, h->capacity,
                                                                                 h->layout, h->counters);
    k_latch<<<1, 1, 0, h->stream>>>(h->counters, 0);
    h->launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_g2p(sv_handle *h, float dt) {
    StepArgs A = make_args(h, dt, make_float3(0, 0, 0));
    Scoped s(h, "g2p");
    unsigned blocks = (unsigned)sm_count() * 6;
    if (h->layout.position_form) k_g2p<true><<<blocks, G2P_THREADS, 0, h->stream>>>(A);
    else k_g2p<false><<<blocks, G2P_THREADS, 0, h->stream>>>(A);
    h->launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_finish_substep(sv_handle *h) {
    k_finish<<<1, 1, 0, h->stream>>>(h->counters, h->capacity);
    h->cur ^= 1;
    h->launches += 1;
    return cudaGetLastError();
}

}  // namespace sv
