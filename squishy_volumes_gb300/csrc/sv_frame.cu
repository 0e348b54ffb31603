// sv_frame.cu -- loading a frame input (sv_set_frame_input): gravity and goals
// of frames a and b, the collider meshes' topology (mesh_util/src/mesh.rs:
// 29-147), their vertex velocities (xpu/src/frame_input.rs:329-343), the
// leaf-cell candidate lists that stand in for the reference's bounding-volume
// hierarchy (frame_input.rs:345-390), the collider bits and the variant
// tables of the grid.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "sv_collide.cuh"
#include "sv_internal.h"

namespace sv {

namespace {

int fail(const std::string &m) {
    set_last_error(m);
    return -1;
}

#define FR_CUDA(expr)                                                                                      \
    do {                                                                                                   \
        cudaError_t e_ = (expr);                                                                           \
        if (e_ != cudaSuccess) return fail(std::string("sv_set_frame_input: ") + #expr + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T> cudaError_t upload(T **dst, const T *src, size_t count) {
    cudaFree(*dst);
    *dst = nullptr;
    cudaError_t e = cudaMalloc((void **)dst, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    if (count && src) e = cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}
template <class T> cudaError_t alloc(T **dst, size_t count) {
    cudaFree(*dst);
    *dst = nullptr;
    return cudaMalloc((void **)dst, std::max<size_t>(count, 1) * sizeof(T));
}

void free_geometry(sv_handle *h) {
    void *ptrs[] = {h->fin_scalars, h->fin_goal_both, h->fin_goal_a, h->fin_goal_b, h->fin_tri, h->fin_tri_col,
                    h->fin_opp, h->fin_va, h->fin_vb, h->fin_vvel, h->fin_fr_a, h->fin_fr_b, h->fin_dm_a,
                    h->fin_dm_b, h->fin_vt_start, h->fin_vt_list, h->fin_leaf_start, h->fin_leaf_list, h->fin_vpos,
                    h->fin_vnorm, h->fin_tnorm, h->fin_fric, h->fin_damp};
    for (void *p : ptrs) cudaFree(p);
    h->fin_scalars = nullptr, h->fin_goal_both = nullptr, h->fin_goal_a = h->fin_goal_b = nullptr;
    h->fin_tri = h->fin_tri_col = h->fin_opp = nullptr;
    h->fin_va = h->fin_vb = h->fin_vvel = nullptr;
    h->fin_fr_a = h->fin_fr_b = h->fin_dm_a = h->fin_dm_b = nullptr;
    h->fin_vt_start = h->fin_vt_list = h->fin_leaf_start = h->fin_leaf_list = nullptr;
    h->fin_vpos = h->fin_vnorm = h->fin_tnorm = h->fin_fric = h->fin_damp = nullptr;
}

void free_bits_and_variants(sv_handle *h) {
    for (int s = 0; s < 2; ++s) {
        cudaFree(h->side[s].cbits), cudaFree(h->side[s].cbits_done);
        h->side[s].cbits = h->side[s].cbits_done = nullptr;
        cudaFree(h->var_key[s]), cudaFree(h->var_bits[s]), cudaFree(h->var_acc[s]), cudaFree(h->var_vel[s]);
        h->var_key[s] = nullptr, h->var_bits[s] = nullptr, h->var_acc[s] = h->var_vel[s] = nullptr;
    }
    h->var_cap = 0;
}

}  // namespace

void free_frame(sv_handle *h) {
    free_geometry(h);
    free_bits_and_variants(h);
}

}  // namespace sv

using namespace sv;

extern "C" int sv_set_time(sv_handle *h, double time) {
    if (!h) return fail("sv_set_time: NULL handle");
    h->time = time;
    h->pending_valid = false;
    return 0;
}

extern "C" int sv_get_time(sv_handle *h, double *time) {
    if (!h || !time) return fail("sv_get_time: NULL argument");
    *time = h->time;
    return 0;
}

extern "C" int sv_set_frame_input(sv_handle *h, const sv_frame_input *in) {
    if (!h) return fail("sv_set_frame_input: NULL handle");
    if (in && h->deterministic) return fail("sv_set_frame_input: the deterministic P2G mode takes no frame input");
    FR_CUDA(cudaStreamSynchronize(h->stream));
    drop_graphs(h);
    h->pending_valid = false;
    if (!in) {
        h->fin_active = false;
        free_frame(h);
        return 0;
    }
    if (h->batched) return fail("sv_set_frame_input: not available for batched handles");
    if (in->frames_per_second == 0) return fail("sv_set_frame_input: frames_per_second must be positive");
    const uint64_t n = h->n;
    const uint32_t nv = in->n_vertices, nt = in->n_triangles;
    const bool has_b = in->has_b != 0;
    if (nt) {
        if (!in->triangles || !in->triangle_collider || !in->vertex_positions_a || !in->friction_a || !in->damping_a ||
            (has_b && (!in->vertex_positions_b || !in->friction_b || !in->damping_b)))
            return fail("sv_set_frame_input: collider arrays missing");
        if (!(in->leaf_size > 0.f)) return fail("sv_set_frame_input: leaf_size must be positive");
        for (uint32_t t = 0; t < nt; ++t) {
            if (in->triangle_collider[t] >= 16) return fail("sv_set_frame_input: at most 16 colliders");
            for (int k = 0; k < 3; ++k)
                if (in->triangles[3 * t + k] >= nv)
                    return fail("sv_set_frame_input: vertex index out of range in triangle " + std::to_string(t));
        }
    }
    // ---- topology (mesh.rs:49-135): opposites and the vertex -> triangle lists,
    // emptied at vertices whose neighbours are not each shared by two triangles
    std::vector<uint32_t> opp(3 * (size_t)nt, col::NO_TRI), vt_start(nv + 1, 0), vt_list;
    if (nt) {
        std::map<std::pair<uint32_t, uint32_t>, std::vector<uint32_t>> edges;
        auto edge = [](uint32_t a, uint32_t b) { return a < b ? std::make_pair(a, b) : std::make_pair(b, a); };
        for (uint32_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k) edges[edge(in->triangles[3 * t + k], in->triangles[3 * t + (k + 1) % 3])].push_back(t);
        for (auto &e : edges)
            if (e.second.size() > 2) return fail("sv_set_frame_input: non-manifold edge");
        for (uint32_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k)
                for (uint32_t o : edges[edge(in->triangles[3 * t + k], in->triangles[3 * t + (k + 1) % 3])])
                    if (o != t) opp[3 * t + k] = o;
        std::vector<std::vector<uint32_t>> vt(nv);
        for (uint32_t t = 0; t < nt; ++t)
            for (int k = 0; k < 3; ++k) vt[in->triangles[3 * t + k]].push_back(t);
        for (uint32_t v = 0; v < nv; ++v) {
            std::map<uint32_t, int> count;
            for (uint32_t t : vt[v])
                for (int k = 0; k < 3; ++k)
                    if (in->triangles[3 * t + k] != v) ++count[in->triangles[3 * t + k]];
            for (auto &c : count)
                if (c.second != 2) {
                    vt[v].clear();
                    break;
                }
            vt_start[v + 1] = vt_start[v] + (uint32_t)vt[v].size();
            vt_list.insert(vt_list.end(), vt[v].begin(), vt[v].end());
        }
    }
    // ---- vertex velocities (frame_input.rs:329-343) and the padded leaf boxes
    // of the triangles over both frames (frame_input.rs:345-390)
    const float *vb = has_b ? in->vertex_positions_b : in->vertex_positions_a;
    std::vector<float> vvel(3 * (size_t)nv, 0.f);
    if (has_b)
        for (size_t k = 0; k < 3 * (size_t)nv; ++k) vvel[k] = (vb[k] - in->vertex_positions_a[k]) * (float)in->frames_per_second;
    int32_t lo[3] = {0, 0, 0}, dim[3] = {0, 0, 0};
    std::vector<uint32_t> leaf_start(1, 0), leaf_list;
    if (nt) {
        const float margin = h->layout.dx * 2.2f, leaf = in->leaf_size;
        std::vector<int32_t> bmin(3 * (size_t)nt), bmax(3 * (size_t)nt);
        int32_t glo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, ghi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
        for (uint32_t t = 0; t < nt; ++t)
            for (int a = 0; a < 3; ++a) {
                float mn = 3.402823466e+38f, mx = -mn;
                for (int k = 0; k < 3; ++k) {
                    const uint32_t v = in->triangles[3 * t + k];
                    mn = std::min(mn, std::min(in->vertex_positions_a[3 * v + a], vb[3 * v + a]));
                    mx = std::max(mx, std::max(in->vertex_positions_a[3 * v + a], vb[3 * v + a]));
                }
                bmin[3 * t + a] = (int32_t)std::floor((mn - margin) / leaf);
                bmax[3 * t + a] = (int32_t)std::ceil((mx + margin) / leaf);
                glo[a] = std::min(glo[a], bmin[3 * t + a]), ghi[a] = std::max(ghi[a], bmax[3 * t + a]);
            }
        uint64_t cells = 1;
        for (int a = 0; a < 3; ++a) lo[a] = glo[a], dim[a] = ghi[a] - glo[a] + 1, cells *= (uint64_t)dim[a];
        if (cells > (1ull << 26)) return fail("sv_set_frame_input: collider leaf box too large (raise leaf_size)");
        std::vector<uint32_t> count(cells + 1, 0);
        uint64_t entries = 0;
        auto cell_of = [&](int x, int y, int z) { return ((uint64_t)(x - lo[0]) * dim[1] + (y - lo[1])) * dim[2] + (z - lo[2]); };
        for (uint32_t t = 0; t < nt; ++t) {
            for (int x = bmin[3 * t]; x <= bmax[3 * t]; ++x)
                for (int y = bmin[3 * t + 1]; y <= bmax[3 * t + 1]; ++y)
                    for (int z = bmin[3 * t + 2]; z <= bmax[3 * t + 2]; ++z) ++count[cell_of(x, y, z) + 1], ++entries;
            if (entries > (1ull << 28)) return fail("sv_set_frame_input: too many leaf-cell entries (raise leaf_size)");
        }
        leaf_start.assign(cells + 1, 0);
        for (uint64_t c = 0; c < cells; ++c) leaf_start[c + 1] = leaf_start[c] + count[c + 1];
        leaf_list.assign(entries, 0);
        std::vector<uint32_t> fill(leaf_start.begin(), leaf_start.end() - 1);
        for (uint32_t t = 0; t < nt; ++t)  // ascending triangle order within each cell
            for (int x = bmin[3 * t]; x <= bmax[3 * t]; ++x)
                for (int y = bmin[3 * t + 1]; y <= bmax[3 * t + 1]; ++y)
                    for (int z = bmin[3 * t + 2]; z <= bmax[3 * t + 2]; ++z) leaf_list[fill[cell_of(x, y, z)]++] = t;
    }
    // ---- goals: bit 0 = HAS_GOAL in both frames (external_force.rs:38-44)
    const bool goals = in->goal_flags_a && in->goal_positions_a;
    std::vector<uint32_t> both;
    if (goals) {
        const uint32_t *fb = has_b && in->goal_flags_b ? in->goal_flags_b : in->goal_flags_a;
        both.resize(n);
        for (uint64_t i = 0; i < n; ++i) both[i] = ((in->goal_flags_a[i] & SV_HAS_GOAL) && (fb[i] & SV_HAS_GOAL)) ? 1u : 0u;
    }
    // ---- upload
    free_geometry(h);
    FR_CUDA(alloc(&h->fin_scalars, 4));
    if (goals) {
        FR_CUDA(upload(&h->fin_goal_both, both.data(), n));
        FR_CUDA(upload(&h->fin_goal_a, in->goal_positions_a, 3 * n));
        FR_CUDA(upload(&h->fin_goal_b, has_b && in->goal_positions_b ? in->goal_positions_b : in->goal_positions_a, 3 * n));
    }
    if (nt) {
        FR_CUDA(upload(&h->fin_tri, in->triangles, 3 * (size_t)nt));
        FR_CUDA(upload(&h->fin_tri_col, in->triangle_collider, nt));
        FR_CUDA(upload(&h->fin_opp, opp.data(), 3 * (size_t)nt));
        FR_CUDA(upload(&h->fin_va, in->vertex_positions_a, 3 * (size_t)nv));
        FR_CUDA(upload(&h->fin_vb, vb, 3 * (size_t)nv));
        FR_CUDA(upload(&h->fin_vvel, vvel.data(), 3 * (size_t)nv));
        FR_CUDA(upload(&h->fin_fr_a, in->friction_a, nt));
        FR_CUDA(upload(&h->fin_fr_b, has_b ? in->friction_b : in->friction_a, nt));
        FR_CUDA(upload(&h->fin_dm_a, in->damping_a, nt));
        FR_CUDA(upload(&h->fin_dm_b, has_b ? in->damping_b : in->damping_a, nt));
        FR_CUDA(upload(&h->fin_vt_start, vt_start.data(), vt_start.size()));
        FR_CUDA(upload(&h->fin_vt_list, vt_list.data(), vt_list.size()));
        FR_CUDA(upload(&h->fin_leaf_start, leaf_start.data(), leaf_start.size()));
        FR_CUDA(upload(&h->fin_leaf_list, leaf_list.data(), leaf_list.size()));
        FR_CUDA(alloc(&h->fin_vpos, 3 * (size_t)nv));
        FR_CUDA(alloc(&h->fin_vnorm, 3 * (size_t)nv));
        FR_CUDA(alloc(&h->fin_tnorm, 3 * (size_t)nt));
        FR_CUDA(alloc(&h->fin_fric, nt));
        FR_CUDA(alloc(&h->fin_damp, nt));
    }
    h->fin_fps = in->frames_per_second, h->fin_frame = in->frame, h->fin_has_b = has_b;
    for (int a = 0; a < 3; ++a) h->fin_g_a[a] = in->gravity_a[a], h->fin_g_b[a] = has_b ? in->gravity_b[a] : in->gravity_a[a];
    h->fin_nv = nt ? nv : 0, h->fin_nt = nt;
    for (int a = 0; a < 3; ++a) h->fin_leaf_lo[a] = lo[a], h->fin_leaf_dim[a] = dim[a];
    h->fin_leaf_size = in->leaf_size > 0.f ? in->leaf_size : 1.f;
    // ---- collider bits: the input's until a substep ran without a frame
    // input (whose Collide would have cleared them), and the variant tables
    if (!h->side[0].cbits) {
        std::vector<uint32_t> bits(n, 0u);
        if (h->substeps_total == 0 && !h->collider_bits.empty()) {
            std::vector<uint32_t> orig(n);
            FR_CUDA(cudaMemcpy(orig.data(), h->side[h->cur].orig, n * 4, cudaMemcpyDeviceToHost));
            for (uint64_t s = 0; s < n; ++s) bits[s] = h->collider_bits[orig[s]];
        }
        for (int s = 0; s < 2; ++s) {
            FR_CUDA(upload(&h->side[s].cbits, bits.data(), n));
            FR_CUDA(upload(&h->side[s].cbits_done, bits.data(), n));
        }
    }
    if (!h->var_key[0]) {
        uint32_t cap = 1u << 16;
        while (cap < 4 * n && cap < (1u << 22)) cap <<= 1;
        for (int s = 0; s < 2; ++s) {
            FR_CUDA(alloc(&h->var_key[s], cap));
            FR_CUDA(alloc(&h->var_bits[s], (size_t)cap * col::VK));
            FR_CUDA(alloc(&h->var_acc[s], (size_t)cap * col::VK));
            FR_CUDA(alloc(&h->var_vel[s], (size_t)cap * col::VK));
            FR_CUDA(cudaMemset(h->var_key[s], 0, (size_t)cap * sizeof(unsigned long long)));
            FR_CUDA(cudaMemset(h->var_bits[s], 0, (size_t)cap * col::VK * sizeof(uint32_t)));
            FR_CUDA(cudaMemset(h->var_acc[s], 0, (size_t)cap * col::VK * sizeof(float4)));
        }
        h->var_cap = cap;
    }
    // the uploads and fills above ran on the legacy default stream, with
    // which the handle's non-blocking stream does not synchronise
    FR_CUDA(cudaDeviceSynchronize());
    h->fin_active = true;
    return 0;
}
