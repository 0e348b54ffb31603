// sv_collide.cuh -- frame input, colliders and the collider-variant grid.
//
// Frame input (rust/crates/xpu/src/frame_input.rs:33-65): gravity, particle
// goals and triangle-mesh colliders of frames a and b, interpolated linearly
// every substep (rust/crates/cpu/src/phase/interpolate_input.rs:18-106).
//
// Colliders (rust/crates/cpu/src/phase/collide.rs:21-206): each live particle
// finds, per collider, the closest triangle within the forget distance among
// the triangles whose padded leaf box holds its leaf cell, keeps one side bit
// and one "near" bit per collider (rust/crates/util/src/collider_bits.rs), and
// is pushed back (with friction and damping) when it crossed to the other
// side.  Here the leaf boxes are rasterised into a dense CSR grid of leaf
// cells on the host once per frame input -- the exact candidate set the
// reference's bounding-volume hierarchy returns a superset of.
//
// The grid keeps one momentum variant per (node, collider bits)
// (rust/crates/cpu/src/phase/update_grid_nodes.rs:94-118) and melds the
// compatible variants of a node (rust/crates/cpu/src/phase/meld_grid.rs:16-69).
// Particles with bits 0 use the dense block grid; the others a node-keyed
// hash table with up to VK variant slots per node.
#pragma once
#include <stdint.h>

#include "sv_math.cuh"

namespace sv {
namespace col {

constexpr int VK = 4;                 // variant slots per node in the table
constexpr uint32_t NO_TRI = 0xFFFFFFFFu;
constexpr float EPS = 1e-5f;          // util/src/consts.rs:11 NORMALIZATION_EPS

// Device view of the frame input.
struct FrameArgs {
    // interpolated, written by the interpolation kernels each substep
    const float *gravity;         // [3]
    const float *factor;          // [1] factor of frame b
    // goals (original particle order): bit 0 = HAS_GOAL in both frames
    const uint32_t *goal_both;    // nullptr: no goals
    const float *goal_a, *goal_b; // [n][3]
    // colliders
    uint32_t nt;
    const uint32_t *tri, *tri_col, *opp;   // [nt][3], [nt], [nt][3]
    const float *vpos, *vnorm, *tnorm;     // interpolated [nv][3], [nv][3], [nt][3]
    const float *vvel;                     // [nv][3] (b - a) fps
    const float *fric, *damp;              // interpolated [nt]
    const uint32_t *leaf_start, *leaf_list;  // CSR over the dense leaf box
    int32_t leaf_lo[3], leaf_dim[3];
    float leaf_size;
    float forget, accept;                  // 2.2 dx, 2 dx (file_input/src/header.rs:60-66)
};

// One table of collider variants (ping-pong like the grids).
struct VariantTable {
    unsigned long long *key;  // [cap] packed node + 1, 0 = empty
    uint32_t *bits;           // [cap * VK], 0 = empty slot
    float4 *acc;              // [cap * VK] momentum, mass (scatter)
    float4 *vel;              // [cap * VK] melded velocity, mass (gather)
    uint32_t cap;             // power of two
};

__host__ __device__ inline unsigned long long node_key(int x, int y, int z) {
    return ((unsigned long long)((uint32_t)(x + (1 << 20)) & 0x1FFFFFu) << 42 |
            (unsigned long long)((uint32_t)(y + (1 << 20)) & 0x1FFFFFu) << 21 |
            (unsigned long long)((uint32_t)(z + (1 << 20)) & 0x1FFFFFu)) + 1ull;
}
__device__ inline uint32_t key_hash(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    return (uint32_t)k;
}

// util/src/collider_bits.rs:34-38
__host__ __device__ inline bool compatible(uint32_t a, uint32_t b) { return (((a & b) >> 16) & (a ^ b)) == 0u; }

// Slot of variant `bits` at node (x, y, z), claimed when `claim`; -1 when
// absent (lookup) or when the table or the node's slots are full (claim).
__device__ inline int64_t variant_slot(const VariantTable &t, int x, int y, int z, uint32_t bits, bool claim) {
    const unsigned long long k = node_key(x, y, z);
    uint32_t h = key_hash(k) & (t.cap - 1);
    for (uint32_t probe = 0; probe < t.cap; ++probe, h = (h + 1) & (t.cap - 1)) {
        unsigned long long cur = t.key[h];
        if (cur == 0ull) {
            if (!claim) return -1;
            cur = atomicCAS(&t.key[h], 0ull, k);
            if (cur == 0ull) cur = k;
        }
        if (cur != k) continue;
        for (int j = 0; j < VK; ++j) {
            uint32_t b = t.bits[(uint64_t)h * VK + j];
            if (b == 0u) {
                if (!claim) return -1;
                b = atomicCAS(&t.bits[(uint64_t)h * VK + j], 0u, bits);
                if (b == 0u) b = bits;
            }
            if (b == bits) return (int64_t)h * VK + j;
        }
        return -1;
    }
    return -1;
}

// Entry of node (x, y, z) (its VK slots start at the returned index * VK), or -1.
__device__ inline int64_t node_entry(const VariantTable &t, int x, int y, int z) {
    const unsigned long long k = node_key(x, y, z);
    uint32_t h = key_hash(k) & (t.cap - 1);
    for (uint32_t probe = 0; probe < t.cap; ++probe, h = (h + 1) & (t.cap - 1)) {
        const unsigned long long cur = t.key[h];
        if (cur == 0ull) return -1;
        if (cur == k) return h;
    }
    return -1;
}

// ------------------------------------------------------------------ geometry (f32, mesh_util/src/mesh.rs)
__device__ inline void cross3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1], o[1] = a[2] * b[0] - a[0] * b[2], o[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ inline float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

struct Dist {
    float distance, to_p[3], normal[3];
};

// mesh.rs:253-280
__device__ inline Dist segment_result(const float p[3], const float s[3], const float e[3], const float sn[3],
                                      const float segn[3], const float en[3]) {
    const float seg[3] = {e[0] - s[0], e[1] - s[1], e[2] - s[2]};
    const float ps[3] = {p[0] - s[0], p[1] - s[1], p[2] - s[2]};
    const float along = dot3(ps, seg) / dot3(seg, seg);
    Dist r;
    const float *nn;
    if (along < 0.f) {
        for (int a = 0; a < 3; ++a) r.to_p[a] = ps[a];
        nn = sn;
    } else if (along < 1.f) {
        for (int a = 0; a < 3; ++a) r.to_p[a] = p[a] - s[a] - seg[a] * along;
        nn = segn;
    } else {
        for (int a = 0; a < 3; ++a) r.to_p[a] = p[a] - e[a];
        nn = en;
    }
    r.distance = sqrtf(dot3(r.to_p, r.to_p));
    for (int a = 0; a < 3; ++a) r.normal[a] = nn[a];
    return r;
}

// mesh.rs:282-308
__device__ inline float triangle_distance(const float p[3], const float A[3], const float B[3], const float C[3],
                                          const float n[3]) {
    const float ab[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
    const float bc[3] = {B[0] - C[0], B[1] - C[1], B[2] - C[2]};
    const float ca[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
    const float cp[3] = {C[0] - p[0], C[1] - p[1], C[2] - p[2]};
    const float ap[3] = {A[0] - p[0], A[1] - p[1], A[2] - p[2]};
    const float bp[3] = {B[0] - p[0], B[1] - p[1], B[2] - p[2]};
    float x[3];
    cross3(bc, cp, x);
    const bool sa = dot3(n, x) > 0.f;
    cross3(ca, ap, x);
    const bool sb = dot3(n, x) > 0.f;
    cross3(ab, bp, x);
    const bool sc = dot3(n, x) > 0.f;
    if (sa && sb && sc) {
        const float pa[3] = {p[0] - A[0], p[1] - A[1], p[2] - A[2]};
        return fabsf(dot3(pa, n));
    }
    const float z[3] = {0.f, 0.f, 0.f};
    float d = 3.402823466e+38f;
    if (!sa) d = fminf(d, segment_result(p, B, C, z, z, z).distance);
    if (!sb) d = fminf(d, segment_result(p, C, A, z, z, z).distance);
    if (!sc) d = fminf(d, segment_result(p, A, B, z, z, z).distance);
    return d;
}

__device__ inline void bits_set(uint32_t &b, int c, int side) {  // collider_bits.rs:22-32; -1 = None
    b &= ~(0x00010001u << c);
    if (side == 1) b |= 0x00010001u << c;
    else if (side == 0) b |= 0x00010000u << c;
}

// collide.rs:21-206 for one live particle at P (world units) with velocity v
// and collider bits `bits` (both updated); dt is the step of the phase.
__device__ inline void collide_particle(const FrameArgs &f, const float P[3], float v[3], uint32_t &bits, float dt) {
    int32_t q[3];
    bool inside = true;
    for (int a = 0; a < 3; ++a) {
        q[a] = (int32_t)floorf(P[a] / f.leaf_size) - f.leaf_lo[a];
        inside = inside && q[a] >= 0 && q[a] < f.leaf_dim[a];
    }
    uint32_t c0 = 0, c1 = 0;
    if (inside) {
        const uint64_t cell = ((uint64_t)q[0] * f.leaf_dim[1] + q[1]) * f.leaf_dim[2] + q[2];
        c0 = f.leaf_start[cell], c1 = f.leaf_start[cell + 1];
    }
    if (c0 == c1) {  // nothing to check (collide.rs:53-56)
        bits = 0u;
        return;
    }
    uint32_t closest[16];
    float mind[16];
    for (int c = 0; c < 16; ++c) closest[c] = NO_TRI, mind[c] = 3.402823466e+38f;
    for (uint32_t k = c0; k < c1; ++k) {
        const uint32_t t = f.leaf_list[k];
        const float n[3] = {f.tnorm[3 * t], f.tnorm[3 * t + 1], f.tnorm[3 * t + 2]};
        if (n[0] == 0.f && n[1] == 0.f && n[2] == 0.f) continue;
        const float *A = f.vpos + 3 * f.tri[3 * t], *B = f.vpos + 3 * f.tri[3 * t + 1], *C = f.vpos + 3 * f.tri[3 * t + 2];
        const float d = triangle_distance(P, A, B, C, n);
        if (d >= f.forget) continue;
        const uint32_t c = f.tri_col[t];
        if (d < mind[c]) mind[c] = d, closest[c] = t;
    }
    for (int c = 0; c < 16; ++c) {
        if (closest[c] == NO_TRI) {
            bits_set(bits, c, -1);
            continue;
        }
        const uint32_t t = closest[c];
        const uint32_t ia = f.tri[3 * t], ib = f.tri[3 * t + 1], ic = f.tri[3 * t + 2];
        const float n[3] = {f.tnorm[3 * t], f.tnorm[3 * t + 1], f.tnorm[3 * t + 2]};
        const float *A = f.vpos + 3 * ia, *B = f.vpos + 3 * ib, *C = f.vpos + 3 * ic;
        float edge_n[3][3];
        for (int e = 0; e < 3; ++e) {
            const uint32_t o = f.opp[3 * t + e];
            for (int a = 0; a < 3; ++a) edge_n[e][a] = o != NO_TRI ? n[a] + f.tnorm[3 * o + a] : 0.f;
        }
        const float ab[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
        const float bc[3] = {B[0] - C[0], B[1] - C[1], B[2] - C[2]};
        const float ca[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
        float x1[3];
        cross3(ca, ab, x1);
        const float area2 = dot3(n, x1);
        const float cp[3] = {C[0] - P[0], C[1] - P[1], C[2] - P[2]};
        const float ap[3] = {A[0] - P[0], A[1] - P[1], A[2] - P[2]};
        const float bp[3] = {B[0] - P[0], B[1] - P[1], B[2] - P[2]};
        cross3(bc, cp, x1);
        const float ba = dot3(n, x1) / area2;
        cross3(ca, ap, x1);
        const float bb = dot3(n, x1) / area2;
        cross3(ab, bp, x1);
        const float bcb = dot3(n, x1) / area2;
        Dist r;
        if (ba > 0.f && bb > 0.f && bcb > 0.f) {
            const float pa[3] = {P[0] - A[0], P[1] - A[1], P[2] - A[2]};
            const float h = dot3(pa, n);
            r.distance = fabsf(h);
            for (int a = 0; a < 3; ++a) r.to_p[a] = n[a] * h, r.normal[a] = n[a];
        } else {
            const float *na = f.vnorm + 3 * ia, *nb = f.vnorm + 3 * ib, *nc = f.vnorm + 3 * ic;
            r = segment_result(P, A, B, na, edge_n[0], nb);
            const Dist r2 = segment_result(P, B, C, nb, edge_n[1], nc);
            const Dist r3 = segment_result(P, C, A, nc, edge_n[2], na);
            if (r2.distance < r.distance) r = r2;
            if (r3.distance < r.distance) r = r3;
        }
        if (r.normal[0] == 0.f && r.normal[1] == 0.f && r.normal[2] == 0.f) {
            bits_set(bits, c, -1);
            continue;
        }
        const bool new_side = 0.f <= dot3(r.to_p, r.normal);
        if (!(bits & (0x00010000u << c))) {
            if (r.distance < f.accept) bits_set(bits, c, new_side ? 1 : 0);
            continue;
        }
        if (((bits & (1u << c)) != 0u) == new_side) continue;
        if (r.distance > EPS) {
            float rel[3], cn[3];
            for (int a = 0; a < 3; ++a) {
                const float cv = f.vvel[3 * ia + a] * ba + f.vvel[3 * ib + a] * bb + f.vvel[3 * ic + a] * bcb;
                rel[a] = v[a] - cv;
                cn[a] = r.to_p[a] / r.distance;
            }
            const float rn = dot3(rel, cn);
            float nv[3], tv[3];
            for (int a = 0; a < 3; ++a) nv[a] = cn[a] * rn, tv[a] = rel[a] - nv[a];
            const float tvn = sqrtf(dot3(tv, tv));
            if (tvn > EPS) {
                const float mag = fminf(f.fric[t] * r.distance / dt, tvn);
                for (int a = 0; a < 3; ++a) v[a] -= tv[a] / tvn * mag;
            }
            const float dmp = fminf(f.damp[t], 1.f);
            for (int a = 0; a < 3; ++a) v[a] -= dmp * nv[a];
        }
        for (int a = 0; a < 3; ++a) v[a] -= r.to_p[a] / dt;
    }
}

}  // namespace col
}  // namespace sv
