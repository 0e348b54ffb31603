// sv_api.cu -- the C ABI (include/squishy_volumes_cuda.h): handle lifecycle,
// upload/download in the reference's particle layout, and the substep loop of
// CpuState::produce_next_state (rust/crates/cpu/src/cpu_state.rs:146-197).
#include <algorithm>
#include <array>
#include <chrono>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "sv_adaptive.cuh"
#include "sv_internal.h"
#include "sv_sort.cuh"

using namespace sv;

namespace {

thread_local std::string g_last_error;

int fail(const std::string &msg) {
    g_last_error = msg;
    return -1;
}

#define SV_CUDA(expr)                                                                                \
    do {                                                                                             \
        cudaError_t e_ = (expr);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return fail(std::string("CUDA error in ") + #expr + ": " + cudaGetErrorString(e_));     \
    } while (0)

template <class T> cudaError_t dalloc(sv_handle *h, T **p, uint64_t count) {
    size_t bytes = (size_t)count * sizeof(T);
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e == cudaSuccess) h->device_bytes += bytes;
    return e;
}

// The buffers whose size is fixed at creation (both particle sides, the
// binning and sort work arrays, the block maps, the counters) are carved out
// of one allocation: one cudaMalloc and one cudaFree per handle instead of
// thirty, about 1.6 ms less per create/destroy pair.
struct Arena {
    std::vector<std::pair<void **, size_t>> parts;
    size_t total = 0;
    template <class T> void add(T **p, uint64_t count) {
        size_t bytes = (size_t)count * sizeof(T);
        if (bytes == 0) bytes = 16;
        parts.push_back({reinterpret_cast<void **>(p), total});
        total += (bytes + 255) & ~size_t(255);
    }
    cudaError_t commit(sv_handle *h) {
        char *base = nullptr;
        cudaError_t e = cudaMalloc((void **)&base, total ? total : 256);
        if (e != cudaSuccess) return e;
        h->arena = base;
        h->device_bytes += total;
        for (auto &pt : parts) *pt.first = base + pt.second;
        return cudaSuccess;
    }
};

void free_handle(sv_handle *h) {
    if (!h) return;
    cudaFree(h->arena);
    for (int s = 0; s < 2; ++s) cudaFree(h->active[s]), cudaFree(h->grid[s]);
    if (h->host_counters) cudaFreeHost(h->host_counters);
    for (auto &p : h->timer.pending) cudaEventDestroy(p.second.first), cudaEventDestroy(p.second.second);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto &kv : h->graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    free_closure(h);
    free_frame(h);
    cudaFree(h->adt), cudaFree(h->adt_backup);
    cudaFree(h->det_kbo), cudaFree(h->det_orig), cudaFree(h->det_cstart), cudaFree(h->det_slot_seg), cudaFree(h->det_rec);
    if (h->wait_event) cudaEventDestroy(h->wait_event);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
}

struct MaterialKey {
    Material m;
    bool operator==(const MaterialKey &o) const { return std::memcmp(&m, &o.m, sizeof(Material)) == 0; }
};
struct MaterialHash {
    size_t operator()(const MaterialKey &k) const {
        const uint32_t *w = reinterpret_cast<const uint32_t *>(&k.m);
        uint64_t h = 1469598103934665603ull;
        for (size_t i = 0; i < sizeof(Material) / 4; ++i) h = (h ^ w[i]) * 1099511628211ull;
        return (size_t)h;
    }
};

int build_material(const sv_particles *p, uint64_t i, Material &m, std::string &err);


// The host pass of sv_create over host threads: per particle its material
// (deduplicated ParticleParameters, numbered in order of first appearance
// like a sequential pass) and the bounds of the live particles of each
// scene.  Errors are those a sequential pass meets first: the lowest
// particle with an invalid parameter set, else a non-finite position.
struct Prepass {
    std::vector<Material> mats;
    std::vector<uint32_t> mat_index;
    std::vector<std::array<double, 3>> lo, hi;  // per scene, of live particles
    bool any_bits = false;                      // some particle has collider bits
    std::string err;
};

void prepass(const sv_particles *ps, uint32_t n_scenes, const std::vector<uint64_t> &first, Prepass &out) {
    const uint64_t n = first[n_scenes];
    out.mat_index.assign(n, 0);
    const uint64_t per = 1u << 16;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned T = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(std::min(hw, 64u), (n + per - 1) / per));
    struct Part {
        std::vector<Material> mats;
        std::vector<uint32_t> remap;
        std::vector<std::array<double, 3>> lo, hi;
        uint64_t err_at = UINT64_MAX;
        std::string err;
        bool nonfinite = false, any_bits = false;
    };
    std::vector<Part> parts(T);
    auto range = [&](unsigned t, uint64_t &g0, uint64_t &g1) { g0 = n * t / T, g1 = n * (t + 1) / T; };
    auto pass1 = [&](unsigned t) {
        Part &pt = parts[t];
        pt.lo.assign(n_scenes, {INFINITY, INFINITY, INFINITY});
        pt.hi.assign(n_scenes, {-INFINITY, -INFINITY, -INFINITY});
        std::unordered_map<MaterialKey, uint32_t, MaterialHash> index;
        Material prev{};
        uint32_t prev_idx = UINT32_MAX;
        uint64_t g0, g1;
        range(t, g0, g1);
        uint32_t s = (uint32_t)(std::upper_bound(first.begin(), first.end(), g0) - first.begin()) - 1;
        uint32_t *mat_index = out.mat_index.data();
        // one scene's run of this part at a time, its arrays and bounds in locals
        for (uint64_t a = g0; a < g1; ++s) {
            while (a >= first[s + 1]) ++s;
            const sv_particles *p = &ps[s];
            const uint64_t b = std::min<uint64_t>(g1, first[s + 1]), base = first[s];
            const uint32_t *flags = p->flags, *bits = p->collider_bits;
            const float *pos = p->positions;
            // the parameter words same_as_previous compares, non-NULL ones only
            const uint32_t *words[13];
            int nw = 0;
            for (const void *q : {(const void *)p->mass, (const void *)p->initial_volume, (const void *)p->model,
                                  (const void *)p->mu, (const void *)p->lambda, (const void *)p->sand_alpha,
                                  (const void *)p->exponent, (const void *)p->bulk_modulus,
                                  (const void *)p->viscosity_dynamic, (const void *)p->viscosity_bulk,
                                  (const void *)p->hardening, (const void *)p->crit_compression,
                                  (const void *)p->crit_stretch})
                if (q) words[nw++] = static_cast<const uint32_t *>(q);
            double lo[3] = {pt.lo[s][0], pt.lo[s][1], pt.lo[s][2]}, hi[3] = {pt.hi[s][0], pt.hi[s][1], pt.hi[s][2]};
            bool nonfinite = false, any_bits = false;
            for (uint64_t g = a; g < b; ++g) {
                const uint64_t i = g - base;
                if (bits && bits[i]) any_bits = true;
                const uint32_t f = flags[i];
                if (!(f & SV_TOMBSTONED)) {
                    for (int c = 0; c < 3; ++c) {
                        const double x = pos[3 * i + c];
                        nonfinite |= !std::isfinite(x);
                        lo[c] = std::min(lo[c], x), hi[c] = std::max(hi[c], x);
                    }
                }
                // the previous particle (same scene, this part) had the material prev_idx
                if (prev_idx != UINT32_MAX && g > a && f == flags[i - 1]) {
                    bool same = true;
                    for (int k = 0; k < nw && same; ++k) same = words[k][i] == words[k][i - 1];
                    if (same) {
                        mat_index[g] = prev_idx;
                        continue;
                    }
                }
                Material m;
                std::string err;
                if (build_material(p, i, m, err)) {
                    pt.err_at = g, pt.err = err;
                    return;
                }
                m.scene = s;
                if (prev_idx != UINT32_MAX && std::memcmp(&m, &prev, sizeof(m)) == 0) {
                    mat_index[g] = prev_idx;
                    continue;
                }
                auto it = index.find(MaterialKey{m});
                uint32_t idx;
                if (it == index.end()) {
                    idx = (uint32_t)pt.mats.size();
                    index.emplace(MaterialKey{m}, idx);
                    pt.mats.push_back(m);
                } else {
                    idx = it->second;
                }
                mat_index[g] = idx;  // local to the part until the merge
                prev = m, prev_idx = idx;
            }
            for (int c = 0; c < 3; ++c) pt.lo[s][c] = lo[c], pt.hi[s][c] = hi[c];
            pt.nonfinite |= nonfinite, pt.any_bits |= any_bits;
            a = b;
        }
    };
    auto run = [&](auto &&fn) {
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < T; ++t) pool.emplace_back(fn, t);
        fn(0u);
        for (auto &th : pool) th.join();
    };
    run(pass1);
    for (const Part &pt : parts)
        if (pt.err_at != UINT64_MAX) {  // parts in index order: the first one found is the lowest
            out.err = pt.err;
            return;
        }
    // merge the parts' materials in part order, which keeps first-appearance order
    std::unordered_map<MaterialKey, uint32_t, MaterialHash> index;
    for (Part &pt : parts) {
        pt.remap.resize(pt.mats.size());
        for (size_t k = 0; k < pt.mats.size(); ++k) {
            auto it = index.find(MaterialKey{pt.mats[k]});
            if (it == index.end()) {
                if (out.mats.size() >= MAX_MATERIALS) {
                    out.err = "more than 2^24 distinct particle parameter sets";
                    return;
                }
                it = index.emplace(MaterialKey{pt.mats[k]}, (uint32_t)out.mats.size()).first;
                out.mats.push_back(pt.mats[k]);
            }
            pt.remap[k] = it->second;
        }
    }
    bool identity = true;  // every part found its materials in the global order
    for (const Part &pt : parts)
        for (size_t k = 0; k < pt.remap.size(); ++k) identity &= pt.remap[k] == k;
    if (!identity)
        run([&](unsigned t) {
            uint64_t g0, g1;
            range(t, g0, g1);
            const std::vector<uint32_t> &r = parts[t].remap;
            bool same = true;
            for (size_t k = 0; k < r.size(); ++k) same &= r[k] == k;
            if (same) return;
            for (uint64_t g = g0; g < g1; ++g) out.mat_index[g] = r[out.mat_index[g]];
        });
    if (out.mats.empty()) out.mats.push_back(Material{});
    out.lo.assign(n_scenes, {INFINITY, INFINITY, INFINITY});
    out.hi.assign(n_scenes, {-INFINITY, -INFINITY, -INFINITY});
    bool nonfinite = false;
    for (const Part &pt : parts) {
        nonfinite |= pt.nonfinite;
        out.any_bits |= pt.any_bits;
        for (uint32_t s = 0; s < n_scenes; ++s)
            for (int a = 0; a < 3; ++a)
                out.lo[s][a] = std::min(out.lo[s][a], pt.lo[s][a]), out.hi[s][a] = std::max(out.hi[s][a], pt.hi[s][a]);
    }
    if (nonfinite) out.err = "non-finite particle position";
}

int build_material(const sv_particles *p, uint64_t i, Material &m, std::string &err) {
    std::memset(&m, 0, sizeof(m));
    uint32_t f = p->flags[i];
    bool solid = f & SV_IS_SOLID, fluid = f & SV_IS_FLUID;
    if (solid == fluid) {
        err = "particle " + std::to_string(i) + ": exactly one of IS_SOLID and IS_FLUID must be set";
        return -1;
    }
    if (f & ~0x7Fu) {
        err = "particle " + std::to_string(i) + ": unknown flag bits set";
        return -1;
    }
    m.mass = p->mass[i];
    m.initial_volume = p->initial_volume[i];
    uint32_t model = p->model ? p->model[i] : SV_MODEL_REFERENCE;
    if (f & SV_USE_VISCOSITY) {
        if (!p->viscosity_dynamic || !p->viscosity_bulk) {
            err = "USE_VISCOSITY set but viscosity arrays are NULL";
            return -1;
        }
        m.use_viscosity = 1;
        m.visc_dynamic = p->viscosity_dynamic[i];
        m.visc_bulk = p->viscosity_bulk[i];
    }
    if (fluid) {
        if (model != SV_MODEL_REFERENCE) {
            err = "particle " + std::to_string(i) + ": fluids only have the reference model";
            return -1;
        }
        m.kind = KIND_FLUID;
        m.exponent = p->exponent ? p->exponent[i] : 0;
        m.bulk_modulus = p->bulk_modulus ? p->bulk_modulus[i] : 0.f;
        // util/src/elastic.rs:527-543
        if (m.exponent <= 1) {
            err = "particle " + std::to_string(i) + ": exponent must be greater than 1";
            return -1;
        }
        if (m.bulk_modulus < 0.f) {
            err = "particle " + std::to_string(i) + ": bulk modulus is negative";
            return -1;
        }
        return 0;
    }
    m.mu = p->mu ? p->mu[i] : 0.f;
    m.lambda = p->lambda ? p->lambda[i] : 0.f;
    if (model == SV_MODEL_FIXED_COROTATED) {
        m.kind = KIND_FIXED_COROTATED;
    } else if (model == SV_MODEL_SNOW) {
        m.kind = KIND_SNOW;
        m.xi = p->hardening ? p->hardening[i] : 0.f;
        m.theta_c = p->crit_compression ? p->crit_compression[i] : 0.f;
        m.theta_s = p->crit_stretch ? p->crit_stretch[i] : 0.f;
    } else if (model == SV_MODEL_REFERENCE) {
        if (f & SV_USE_SAND_ALPHA) {
            if (!p->sand_alpha) {
                err = "USE_SAND_ALPHA set but sand_alpha is NULL";
                return -1;
            }
            m.kind = KIND_SAND;
            m.alpha = p->sand_alpha[i];
        } else {
            m.kind = KIND_NEO_HOOKEAN;
        }
    } else {
        err = "particle " + std::to_string(i) + ": unknown model";
        return -1;
    }
    return 0;
}

// (Re)allocates both grids and both slot lists with `capacity` blocks.  The
// slot lists are copied so the block maps can still be reset from them.
cudaError_t alloc_grid(sv_handle *h, uint64_t capacity) {
    cudaError_t e;
    uint32_t *active[2] = {nullptr, nullptr};
    float4 *grid[2] = {nullptr, nullptr};
    for (int s = 0; s < 2; ++s) {
        if ((e = dalloc(h, &active[s], capacity)) != cudaSuccess || (e = dalloc(h, &grid[s], capacity * 64)) != cudaSuccess) {
            for (int t = 0; t < 2; ++t) cudaFree(active[t]), cudaFree(grid[t]);
            return e;
        }
    }
    // the old slot lists are copied on the handle's stream; nothing is freed
    // or swapped in until that copy has completed without error
    for (int s = 0; s < 2 && h->active[s]; ++s)
        if ((e = cudaMemcpyAsync(active[s], h->active[s], std::min(capacity, h->capacity) * 4, cudaMemcpyDeviceToDevice,
                                 h->stream)) != cudaSuccess)
            break;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        for (int t = 0; t < 2; ++t) cudaFree(active[t]), cudaFree(grid[t]);
        h->device_bytes -= 2 * (capacity * 4 + capacity * 64 * sizeof(float4));
        return e;
    }
    for (int s = 0; s < 2; ++s) {
        if (h->active[s]) {
            cudaFree(h->active[s]);
            cudaFree(h->grid[s]);
            h->device_bytes -= h->capacity * 4 + h->capacity * 64 * sizeof(float4);
        }
        h->active[s] = active[s];
        h->grid[s] = grid[s];
    }
    h->capacity = capacity;
    return cudaSuccess;
}

// Scatter of the current state into grid[gcur] after a fresh binning: the
// start of a run, or the recovery after a particle left its claimed blocks.
// The deterministic mode's work buffers, sized for the grid block capacity.
cudaError_t ensure_det_buffers(sv_handle *h) {
    if (h->det_kbo && h->det_seg_cap >= h->capacity) return cudaSuccess;
    cudaError_t e;
    if (!h->det_kbo) {
        if ((e = dalloc(h, &h->det_kbo, h->n)) || (e = dalloc(h, &h->det_orig, h->n)) ||
            (e = dalloc(h, &h->det_rec, 4 * h->n)))
            return e;
    }
    cudaFree(h->det_cstart), cudaFree(h->det_slot_seg);
    h->det_cstart = nullptr, h->det_slot_seg = nullptr;
    if ((e = dalloc(h, &h->det_cstart, 65 * h->capacity)) || (e = dalloc(h, &h->det_slot_seg, h->capacity))) return e;
    h->det_seg_cap = h->capacity;
    return cudaSuccess;
}

int standalone_p2g(sv_handle *h, float dt, float3 g) {
    if (!h->keys_valid) SV_CUDA(launch_keys(h));
    if (h->deterministic) {
        SV_CUDA(ensure_det_buffers(h));
        SV_CUDA(launch_det_binning(h));
    } else {
        SV_CUDA(launch_sort_and_segments(h));
    }
    const int which = h->map_cur ^ 1;
    SV_CUDA(launch_activate(h, which));
    h->map_cur = h->map_next = which;
    SV_CUDA(launch_clear(h, h->gcur, which));
    if (h->fin_active) {
        SV_CUDA(launch_interpolate(h, h->time));
        SV_CUDA(launch_clear_variants(h, h->gcur));
    }
    if (h->deterministic) SV_CUDA(launch_det_p2g(h, dt, g));
    else SV_CUDA(launch_p2g(h, dt, g));
    // a scatter that failed (e.g. a record outside the claimed blocks) stops
    // the passes that would gather from it
    SV_CUDA(launch_latch(h));
    h->pending_valid = true;
    h->pending_dt = dt;
    h->pending_g[0] = g.x, h->pending_g[1] = g.y, h->pending_g[2] = g.z;
    h->need_perm = true;
    h->since_sort = 0;
    return 0;
}

bool in_frame(const sv_handle *h, double t) {
    return (long long)std::floor(t * (double)h->fin_fps) == (long long)h->fin_frame;
}

// One substep: (every sort_interval substeps) binning sort and block claims
// for the next grid, grid update, fused gather/advance/scatter.  With a
// frame input the scatter belongs to the substep starting at t_next: the
// input is interpolated there first, and when t_next lies outside the loaded
// frame the substep only gathers and advances (the next call scatters once
// the next frame is loaded).
int fused_substep(sv_handle *h, float dt, float3 g, double t_next = 0.0) {
    if (h->deterministic) {
        // gather and advance, then the next substep's scatter binned afresh
        // and gathered per node in the fixed order, into the other grid (the
        // one gathered from keeps the substep's velocities)
        SV_CUDA(launch_grid_update(h, false));
        SV_CUDA(launch_g2p_advance(h, dt));
        h->need_perm = false;
        h->gcur ^= 1;
        return standalone_p2g(h, dt, g);
    }
    if (h->fin_active && !in_frame(h, t_next)) {
        SV_CUDA(launch_grid_update(h, false));
        SV_CUDA(launch_g2p_advance(h, dt));
        h->need_perm = false;
        h->since_sort = h->sort_interval;
        h->pending_valid = false;
        return 0;
    }
    if (h->since_sort >= h->sort_interval) {
        if (!h->keys_valid) SV_CUDA(launch_keys(h));
        SV_CUDA(launch_sort_and_segments(h));
        const int which = h->map_cur ^ 1;
        SV_CUDA(launch_activate(h, which));
        h->map_next = which;
        h->need_perm = true;
        h->since_sort = 0;
    } else {
        h->map_next = h->map_cur;
    }
    if (h->fin_active) {
        SV_CUDA(launch_interpolate(h, t_next));
        SV_CUDA(launch_clear_variants(h, h->gcur ^ 1));
    }
    // the plain pass latches its own stop bits, so after it (or after the
    // binning's block claims) the grid update needs no latch of its own
    SV_CUDA(launch_grid_update(h, true, !h->stop_latched));
    const bool write_keys = h->since_sort + 1 >= h->sort_interval;
    SV_CUDA(launch_g2p2g(h, dt, g, write_keys, h->need_perm));
    h->need_perm = false;
    h->since_sort += 1;
    return 0;
}

// One adaptive substep in the split form: the limits need reductions over
// all particles between the gather and the advance, so binning, limits
// before force, P2G, grid update, G2P, limits before integrate and advance
// each take their own pass.  Used with a frame input loaded, and where the
// fused form's speculative steps keep failing.
int adaptive_substep(sv_handle *h, float3 g) {
    SV_CUDA(launch_adaptive_begin(h));
    // The binning is redone every sort_interval substeps, as in the fused
    // path: particles that left their segment's tile scatter and gather
    // through global memory, and one that left the claimed blocks stops the
    // substep (ST_MOVED_FAR), which sv_step_adaptive then redoes.
    if (h->since_sort >= h->sort_interval) {
        if (!h->keys_valid) SV_CUDA(launch_keys(h));
        SV_CUDA(launch_sort_and_segments(h));
        const int which = h->map_cur ^ 1;
        SV_CUDA(launch_activate(h, which));
        h->map_cur = h->map_next = which;
        h->since_sort = 0;
    }
    if (h->fin_active) {
        SV_CUDA(launch_interpolate(h, 0.0));  // at the device time of the substep
        SV_CUDA(launch_clear_variants(h, h->gcur));
    }
    // Later substeps of a call take the force limits that the advance before
    // them reduced (a stopped substep stops all that follow it).
    SV_CUDA(launch_limits_force(h, h->limits_pass_pending));
    h->limits_pass_pending = false;
    SV_CUDA(launch_clear(h, h->gcur, h->map_cur));
    SV_CUDA(launch_p2g(h, 0.f, g));
    SV_CUDA(launch_grid_update(h, false));
    SV_CUDA(launch_g2p_only(h));
    SV_CUDA(launch_advance(h));
    h->since_sort += 1;
    return 0;
}

// One adaptive substep in the fused form (no frame input loaded), shaped
// like fused_substep: the pass that advances this substep also scatters the
// next one, at the steps the adaptive state will allow unless one of the
// limits still to come binds (launch_g2p2g_adaptive checks and redoes).  The
// first substep of a call, and the one after a recovery, scatter their own
// momentum first, binned afresh.
int adaptive_substep_fused(sv_handle *h, float3 g) {
    SV_CUDA(launch_adaptive_begin(h));
    if (!h->pending_valid) {
        SV_CUDA(launch_limits_force(h, h->limits_pass_pending));
        h->limits_pass_pending = false;
        if (!h->keys_valid) SV_CUDA(launch_keys(h));
        SV_CUDA(launch_sort_and_segments(h));
        const int which = h->map_cur ^ 1;
        SV_CUDA(launch_activate(h, which));
        h->map_cur = h->map_next = which;
        SV_CUDA(launch_clear(h, h->gcur, which));
        SV_CUDA(launch_p2g(h, 0.f, g));
        SV_CUDA(launch_latch(h));  // a failed scatter stops the substep before its gather
        h->pending_valid = true;
        h->need_perm = true;
        h->since_sort = 0;
    } else {
        SV_CUDA(launch_limits_force(h, false));  // the force step's push
        if (h->since_sort >= h->sort_interval) {
            if (!h->keys_valid) SV_CUDA(launch_keys(h));
            SV_CUDA(launch_sort_and_segments(h));
            const int which = h->map_cur ^ 1;
            SV_CUDA(launch_activate(h, which));
            h->map_next = which;
            h->need_perm = true;
            h->since_sort = 0;
        } else {
            h->map_next = h->map_cur;
        }
    }
    SV_CUDA(launch_grid_update(h, true, !h->stop_latched));
    const bool write_keys = h->since_sort + 1 >= h->sort_interval;
    SV_CUDA(launch_g2p2g_adaptive(h, g, write_keys, h->need_perm));
    h->since_sort += 1;
    return 0;
}

void clear_graphs(sv_handle *h) {
    for (auto &kv : h->graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    h->graphs.clear();
}

// One binning period (the binning substep and the substeps up to the next
// binning) as a CUDA graph: captured the first time a given launch
// configuration occurs, replayed afterwards.  Every launch of a period reads
// its counts from device memory, so the captured launches stay valid; only
// the pointers and the host-side bookkeeping differ between configurations,
// and those are in the key and the saved state.  `adaptive`: substeps of the
// fused adaptive form, whose steps all come from the device (key dt -1).
// Runs `count` substeps (whole binning periods by default) as one CUDA graph,
// captured on first use for the host state they start from.
int run_period_graph(sv_handle *h, float dt, float3 g, bool adaptive = false, uint32_t count = 0) {
    auto substep = [&]() { return adaptive ? adaptive_substep_fused(h, g) : fused_substep(h, dt, g); };
    sv_handle::GraphKey key{h->cur,
                            h->gcur,
                            h->map_cur,
                            h->map_next,
                            h->sort_interval,
                            std::min(h->since_sort, h->sort_interval),
                            count ? count : h->sort_interval,
                            h->keys_valid,
                            h->need_perm,
                            h->stop_latched,
                            adaptive ? -1.f : dt,
                            {g.x, g.y, g.z}};
    auto it = h->graphs.find(key);
    if (it == h->graphs.end() && key.count != key.period && h->partial_seen.insert(key).second) {
        // A part of a period is captured only when it recurs (a caller's
        // fixed substep count): a one-off part would pay its capture and
        // instantiation for nothing.
        for (uint32_t s = 0; s < key.count; ++s)
            if (substep()) return -1;
        return 0;
    }
    if (it == h->graphs.end()) {
        // host bookkeeping before the period, put back if the capture fails
        const int cur0 = h->cur, gcur0 = h->gcur, map_cur0 = h->map_cur, map_next0 = h->map_next;
        const int vel_side0 = h->vel_side, vel_map0 = h->vel_map;
        const bool keys_valid0 = h->keys_valid, need_perm0 = h->need_perm, stop_latched0 = h->stop_latched;
        const uint32_t since0 = h->since_sort;
        const uint64_t l0 = h->launches, sorts0 = h->sorts;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            int rc = 0;
            for (uint32_t s = 0; s < key.count && rc == 0; ++s) rc = substep();
            e = cudaStreamEndCapture(h->stream, &graph);
            if (rc && e == cudaSuccess) e = cudaErrorStreamCaptureInvalidated;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
        }
        if (e != cudaSuccess) {
            // The stream cannot be captured (e.g. the legacy default stream):
            // run the period launch by launch from now on.
            (void)cudaGetLastError();
            g_last_error.clear();
            h->cur = cur0, h->gcur = gcur0, h->map_cur = map_cur0, h->map_next = map_next0;
            h->vel_side = vel_side0, h->vel_map = vel_map0;
            h->keys_valid = keys_valid0, h->need_perm = need_perm0, h->since_sort = since0;
            h->stop_latched = stop_latched0;
            h->launches = l0, h->sorts = sorts0;
            h->use_graphs = false;
            for (uint32_t s = 0; s < key.count; ++s)
                if (substep()) return -1;
            return 0;
        }
        sv_handle::GraphState st;
        st.exec = exec;
        st.cur = h->cur, st.gcur = h->gcur, st.map_cur = h->map_cur, st.map_next = h->map_next;
        st.vel_side = h->vel_side, st.vel_map = h->vel_map;
        st.keys_valid = h->keys_valid, st.need_perm = h->need_perm, st.since_sort = h->since_sort;
        st.stop_latched = h->stop_latched;
        st.launches = h->launches - l0;
        st.sorts = h->sorts - sorts0;
        it = h->graphs.emplace(key, st).first;
        h->launches = l0;
        h->sorts = sorts0;  // counted again below, like a replay
    }
    const sv_handle::GraphState &st = it->second;
    SV_CUDA(cudaGraphLaunch(st.exec, h->stream));
    h->cur = st.cur, h->gcur = st.gcur, h->map_cur = st.map_cur, h->map_next = st.map_next;
    h->vel_side = st.vel_side, h->vel_map = st.vel_map;
    h->keys_valid = st.keys_valid, h->need_perm = st.need_perm, h->since_sort = st.since_sort;
    h->stop_latched = st.stop_latched;
    h->launches += st.launches;
    h->sorts += st.sorts;
    h->graph_launches += 1;
    return 0;
}

int read_counters(sv_handle *h) {
    SV_CUDA(cudaMemcpyAsync(h->host_counters, h->counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    SV_CUDA(cudaStreamSynchronize(h->stream));
    return 0;
}

// The same read for the substep loops, waiting like the reference's GPU
// backend (gpu_state.rs:509-522 polls its device every 100 ms and checks the
// harness in between): the queued work cannot be recalled, so the wait
// polls the copy's event and notes a cancel request seen meanwhile in
// *canceled; the caller stops queueing once the chunk in flight has
// completed.
int read_counters_polled(sv_handle *h, const volatile int32_t *cancel, bool *canceled) {
    SV_CUDA(cudaMemcpyAsync(h->host_counters, h->counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    if (!h->wait_event) SV_CUDA(cudaEventCreateWithFlags(&h->wait_event, cudaEventDisableTiming));
    SV_CUDA(cudaEventRecord(h->wait_event, h->stream));
    // The GPU idles from the end of the queued work until the caller queues
    // more, so the wait polls without sleeping (a 50 us sleep cost up to
    // 2 % of a 20-substep call); yielding leaves the core to other threads.
    while (true) {
        const cudaError_t q = cudaEventQuery(h->wait_event);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) SV_CUDA(q);
        if (cancel && *cancel && canceled) *canceled = true;
        std::this_thread::yield();
    }
    if (cancel && *cancel && canceled) *canceled = true;
    return 0;
}

}  // namespace

namespace sv {

void timer_begin(sv_handle *h, const char *, cudaEvent_t *start) {
    if (!h->profiling) return;
    cudaEventCreate(start);
    cudaEventRecord(*start, h->stream);
}

void timer_end(sv_handle *h, const char *name, cudaEvent_t start) {
    if (!h->profiling || !start) return;
    cudaEvent_t stop;
    cudaEventCreate(&stop);
    cudaEventRecord(stop, h->stream);
    h->timer.pending.push_back({name, {start, stop}});
}

void set_last_error(const std::string &msg) { g_last_error = msg; }

void drop_graphs(sv_handle *h) { clear_graphs(h); }

int refresh_counters(sv_handle *h) { return read_counters(h); }

}  // namespace sv

extern "C" {

const char *sv_last_error_string(void) { return g_last_error.c_str(); }

namespace {

// Shared by sv_create (one scene) and sv_create_batched (many).  Batched
// scenes are laid side by side in x and y in one block index, each
// translated by a whole number of cells (so translation is exact in the
// int32-cell position form, which batched handles always use) and separated
// by at least 16 cells, more than any particle can travel before its own
// scene's domain culls it.
int create_impl(const sv_consts *cs, const sv_particles *ps, uint32_t n_scenes, bool batched, sv_handle **out) {
    g_last_error.clear();
    if (!cs || !ps || !out || n_scenes == 0) return fail("sv_create: NULL argument");
    *out = nullptr;
    const sv_consts &c = cs[0];
    uint64_t n = 0;
    std::vector<uint64_t> first(n_scenes + 1, 0);
    for (uint32_t s = 0; s < n_scenes; ++s) {
        const sv_particles *p = &ps[s];
        const sv_consts &cc = cs[s];
        if (p->n > 0 && (!p->flags || !p->positions || !p->position_gradients || !p->velocities ||
                         !p->velocity_gradients || !p->mass || !p->initial_volume))
            return fail("sv_create: required particle array is NULL");
        if (!(cc.grid_node_size > 0.f)) return fail("sv_create: grid_node_size must be positive");
        if (cc.position_form > 1) return fail("sv_create: unknown position_form");
        if (cc.ground_mode < 0 || cc.ground_mode > 2 || cc.ground_axis < 0 || cc.ground_axis > 2)
            return fail("sv_create: invalid ground plane settings");
        if (batched && (cc.grid_node_size != c.grid_node_size || cc.ground_mode != c.ground_mode ||
                        cc.ground_axis != c.ground_axis || cc.ground_height != c.ground_height ||
                        cc.svd_fp64_policy != c.svd_fp64_policy))
            return fail("sv_create_batched: scenes must share grid_node_size, ground plane and SVD policy");
        if (batched && cc.ground_mode != 0 && cc.ground_axis != 2)
            return fail("sv_create_batched: the ground plane must be on axis 2 (scenes are laid out in x and y)");
        if (batched)
            for (uint64_t i = 0; i < p->n; ++i)
                if (p->collider_bits && p->collider_bits[i] != 0)
                    return fail("sv_create_batched: batched scenes have no colliders; collider bits must be 0");
        first[s + 1] = first[s] + p->n;
    }
    n = first[n_scenes];
    if (n >= (1ull << 31)) return fail("sv_create: too many particles (limit 2^31 - 1)");

    // materials (deduplicated ParticleParameters, one set per scene) and the
    // bounds of the live particles
    Prepass pre;
    prepass(ps, n_scenes, first, pre);
    if (!pre.err.empty()) return fail("sv_create: " + pre.err);
    std::vector<Material> &mats = pre.mats;
    const std::vector<uint32_t> &mat_index = pre.mat_index;

    if (c.deterministic_p2g > 1) return fail("sv_create: deterministic_p2g must be 0 or 1");
    if (c.deterministic_p2g && (batched || c.position_form != 0))
        return fail("sv_create: deterministic_p2g needs fp32 positions (position_form 0) and a single scene");
    sv_handle *h = new sv_handle();
    h->n = n;
    h->batched = batched;
    h->scene_first = first;
    if (c.sort_interval == 0) {
        h->adaptive_interval = true;
        h->sort_interval = h->max_interval = 8;
    } else {
        h->adaptive_interval = false;
        h->sort_interval = h->max_interval = c.sort_interval;
    }
    GridLayout &L = h->layout;
    L.dx = c.grid_node_size;
    L.ground_mode = c.ground_mode, L.ground_axis = c.ground_axis, L.ground_height = c.ground_height;
    L.position_form = batched ? 1u : c.position_form;
    L.svd_policy = c.svd_fp64_policy;
    h->deterministic = c.deterministic_p2g == 1;
    for (int a = 0; a < 3; ++a) {
        L.domain_min[a] = c.domain_min[a], L.domain_max[a] = c.domain_max[a];
        L.dmin_cells[a] = (double)c.domain_min[a] / (double)L.dx;
        L.dmax_cells[a] = (double)c.domain_max[a] / (double)L.dx;
    }
    // Per scene: cell extent of its domain and initial live particles (which
    // may start outside the domain; they are culled after their first substep).
    std::vector<SceneInfo> scenes(n_scenes);
    std::vector<std::array<int64_t, 3>> clo(n_scenes), chi(n_scenes);
    for (uint32_t s = 0; s < n_scenes; ++s) {
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min<double>(cs[s].domain_min[a], pre.lo[s][a]);
            hi[a] = std::max<double>(cs[s].domain_max[a], pre.hi[s][a]);
        }
        for (int a = 0; a < 3; ++a) {
            const double cmin = std::floor(lo[a] / L.dx - 0.5), cmax = std::floor(hi[a] / L.dx - 0.5);
            if (!(cmax - cmin < 4.0e8) || !(std::fabs(cmin) < 1.0e9) || !(std::fabs(cmax) < 1.0e9)) {
                free_handle(h);
                return fail("sv_create: domain too large for the dense block index");
            }
            clo[s][a] = (int64_t)cmin, chi[s][a] = (int64_t)cmax;
            scenes[s].dmin[a] = (double)cs[s].domain_min[a] / (double)L.dx;
            scenes[s].dmax[a] = (double)cs[s].domain_max[a] / (double)L.dx;
            scenes[s].off[a] = 0;
        }
    }
    if (batched) {
        // slots of the largest scene extent plus 16 cells, in a near-square x-y grid
        int64_t slot[2] = {0, 0};
        for (uint32_t s = 0; s < n_scenes; ++s)
            for (int a = 0; a < 2; ++a) slot[a] = std::max<int64_t>(slot[a], chi[s][a] - clo[s][a] + 1 + 16);
        for (int a = 0; a < 2; ++a) slot[a] = (slot[a] + 3) / 4 * 4;
        const uint32_t cols = (uint32_t)std::ceil(std::sqrt((double)n_scenes));
        for (uint32_t s = 0; s < n_scenes; ++s) {
            const int64_t ix = s % cols, iy = s / cols;
            scenes[s].off[0] = (int32_t)(ix * slot[0] + 8 - clo[s][0]);
            scenes[s].off[1] = (int32_t)(iy * slot[1] + 8 - clo[s][1]);
            scenes[s].off[2] = 0;
        }
    }
    uint64_t total = 1;
    for (int a = 0; a < 3; ++a) {
        int64_t cmin = INT64_MAX, cmax = INT64_MIN;
        for (uint32_t s = 0; s < n_scenes; ++s) {
            cmin = std::min<int64_t>(cmin, clo[s][a] + scenes[s].off[a]);
            cmax = std::max<int64_t>(cmax, chi[s][a] + scenes[s].off[a]);
        }
        if (cmax - cmin >= (int64_t)4e8 || cmin < -(int64_t)1e9 || cmax > (int64_t)1e9) {
            free_handle(h);
            return fail("sv_create: domain too large for the dense block index");
        }
        L.origin[a] = (int32_t)(cmin - 8);
        L.nb[a] = (int32_t)((cmax - L.origin[a]) >> 2) + 4;
        total *= (uint64_t)L.nb[a];
        if (total >= (1ull << 26)) {
            free_handle(h);
            return fail("sv_create: the dense block index would reach 2^26 blocks of 4^3 nodes "
                        "(domain / grid_node_size too large)");
        }
    }
    L.total_blocks = total;
    L.key_bits = 0;
    while ((1ull << L.key_bits) <= total * 64) ++L.key_bits;

    auto cuda_fail = [&](cudaError_t e, const char *what) {
        free_handle(h);
        return fail(std::string("sv_create: ") + what + ": " + cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e, "stream");
    h->stream = h->own_stream;
    const bool cell = L.position_form == 1;
    Arena arena;
    for (int s = 0; s < 2; ++s) {
        ParticleArrays &a = h->side[s];
        arena.add(&a.pos, n), arena.add(&a.vel, n), arena.add(&a.C, 9 * n), arena.add(&a.F, 9 * n);
        arena.add(&a.energy, n), arena.add(&a.orig, n);
        if (cell) arena.add(&a.cell, n);
    }
    h->sort_temp_bytes = radix_sort_temp_bytes(n);
    uint64_t tiles = (n + 2047) / 2048 + 1;
    arena.add(&h->materials, mats.size()), arena.add(&h->scenes, n_scenes);
    arena.add(&h->keys, n), arena.add(&h->sorted_keys, n), arena.add(&h->perm, n), arena.add(&h->inv, n);
    arena.add(&h->defer_list, n);
    arena.add(&h->grid_sums, 8);
    arena.add(&h->pass_timer, 3);
    arena.add(&h->seg_start, n + 1), arena.add(&h->seg_block, n), arena.add(&h->counters, C_COUNT);
    arena.add((char **)&h->sort_temp, h->sort_temp_bytes), arena.add(&h->tile_counts, tiles);
    arena.add((char **)&h->scan_temp, scan_temp_bytes(tiles));
    arena.add(&h->blockmap[0], total), arena.add(&h->blockmap[1], total);
    if ((e = arena.commit(h))) return cuda_fail(e, "particle and work buffers");
    h->n_materials = (uint32_t)mats.size();
    // the isolated-particle limit of a solid depends on its parameters and
    // dx only (limit_time_step.rs:137-151): once per material, not per particle
    for (Material &m : mats)
        m.iso_limit = m.kind == KIND_FLUID ? adaptive::NONE
                                           : adaptive::isolated_limit<float>(false, m.mu, m.lambda, 0.f, 0, m.mass,
                                                                             m.initial_volume, 1.f, L.dx);
    h->host_materials = mats;
    h->host_scenes = scenes;
    h->kind_set = 0;
    for (const Material &m : mats) h->kind_set |= 1u << m.kind;
    // blocks claimed are about n / 200 for bodies of 8 particles per cell;
    // n / 16 leaves room for sparse ones, and sv_step doubles it on overflow
    uint64_t cap = c.block_capacity ? c.block_capacity : std::min<uint64_t>(total, std::max<uint64_t>(65536, n / 16));
    if ((e = alloc_grid(h, cap))) return cuda_fail(e, "grid");
    if ((e = cudaMallocHost((void **)&h->host_counters, C_COUNT * sizeof(uint32_t)))) return cuda_fail(e, "pinned");

    if ((e = cudaMemcpy(h->materials, mats.data(), mats.size() * sizeof(Material), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(h->scenes, scenes.data(), n_scenes * sizeof(SceneInfo), cudaMemcpyHostToDevice)) ||
        (e = cudaMemset(h->blockmap[0], 0xFF, total * 4)) || (e = cudaMemset(h->blockmap[1], 0xFF, total * 4)) ||
        (e = cudaMemset(h->counters, 0, C_COUNT * 4)) || (e = cudaMemset(h->grid_sums, 0, 8 * sizeof(double))) ||
        (e = cudaMemset(h->pass_timer, 0, 3 * sizeof(uint64_t))))
        return cuda_fail(e, "upload");
    h->direct_host = c.host_transfer == 0 && pageable_access();
    if (h->direct_host) {
        // one kernel reads the caller's arrays (sv_transfer.cu)
        if ((e = upload_direct(h, ps, n_scenes, first.data(), mat_index.data()))) return cuda_fail(e, "upload");
    } else {
        // Host staging in the device layout, then one copy per array.
        std::vector<float4> pos(n), vel(n);
        std::vector<int4> cellv(cell ? n : 0);
        std::vector<float> C(9 * n), F(9 * n), en(n);
        std::vector<uint32_t> orig(n);
        for (uint32_t sc = 0; sc < n_scenes; ++sc) {
            const sv_particles *p = &ps[sc];
            for (uint64_t li = 0; li < p->n; ++li) {
                const uint64_t i = first[sc] + li;
                uint32_t packed = (p->flags[li] & FLAG_MASK) | (mat_index[i] << MATERIAL_SHIFT);
                float x = p->positions[3 * li], y = p->positions[3 * li + 1], z = p->positions[3 * li + 2];
                if (!cell) {
                    pos[i] = make_float4(x, y, z, 0.f);
                } else {
                    double q[3] = {(double)x / L.dx, (double)y / L.dx, (double)z / L.dx};
                    int ci[3];
                    float o[3];
                    for (int a = 0; a < 3; ++a) {
                        double f = std::floor(q[a]);
                        ci[a] = (int)f + scenes[sc].off[a];
                        o[a] = (float)(q[a] - f);
                        if (o[a] >= 1.f) o[a] = 0.f, ci[a] += 1;
                    }
                    pos[i] = make_float4(o[0], o[1], o[2], 0.f);
                    cellv[i] = make_int4(ci[0], ci[1], ci[2], 0);
                }
                std::memcpy(&pos[i].w, &packed, 4);
                vel[i] = make_float4(p->velocities[3 * li], p->velocities[3 * li + 1], p->velocities[3 * li + 2],
                                     p->plastic_j ? p->plastic_j[li] : 1.f);
                for (int k = 0; k < 9; ++k) {
                    C[(uint64_t)k * n + i] = p->velocity_gradients[9 * li + k];
                    F[(uint64_t)k * n + i] = p->position_gradients[9 * li + k];
                }
                en[i] = p->elastic_energies ? p->elastic_energies[li] : 0.f;
                orig[i] = (uint32_t)i;
            }
        }
        ParticleArrays &a = h->side[0];
        if ((e = cudaMemcpy(a.pos, pos.data(), n * 16, cudaMemcpyHostToDevice)) ||
            (cell && (e = cudaMemcpy(a.cell, cellv.data(), n * 16, cudaMemcpyHostToDevice))) ||
            (e = cudaMemcpy(a.vel, vel.data(), n * 16, cudaMemcpyHostToDevice)) ||
            (e = cudaMemcpy(a.C, C.data(), 9 * n * 4, cudaMemcpyHostToDevice)) ||
            (e = cudaMemcpy(a.F, F.data(), 9 * n * 4, cudaMemcpyHostToDevice)) ||
            (e = cudaMemcpy(a.energy, en.data(), n * 4, cudaMemcpyHostToDevice)) ||
            (e = cudaMemcpy(a.orig, orig.data(), n * 4, cudaMemcpyHostToDevice)))
            return cuda_fail(e, "upload");
    }
    // kept only when some particle starts with collider bits (empty: all 0)
    h->collider_bits.clear();
    if (!batched && ps[0].collider_bits && pre.any_bits)
        h->collider_bits.assign(ps[0].collider_bits, ps[0].collider_bits + n);
    h->keys_valid = false;
    // the uploads and fills above ran on the legacy default stream, with
    // which the handle's non-blocking stream does not synchronise
    if ((e = cudaDeviceSynchronize())) return cuda_fail(e, "upload");
    *out = h;
    return 0;
}

}  // namespace

int sv_create(const sv_consts *c, const sv_particles *p, sv_handle **out) { return create_impl(c, p, 1, false, out); }

int sv_create_batched(const sv_consts *consts, const sv_particles *particles, uint32_t n_scenes, sv_handle **out) {
    return create_impl(consts, particles, n_scenes, true, out);
}

uint32_t sv_scene_count(sv_handle *h) { return h ? (uint32_t)h->host_scenes.size() : 0u; }

void sv_destroy(sv_handle *h) { free_handle(h); }

int sv_step(sv_handle *h, uint32_t n_substeps, float dt, const float gravity[3], const volatile int32_t *cancel,
            uint32_t *status_out, uint32_t *substeps_done) {
    g_last_error.clear();
    if (!h) return fail("sv_step: NULL handle");
    if (status_out) *status_out = 0;
    if (substeps_done) *substeps_done = 0;
    if (!(dt > 0.f)) return fail("sv_step: dt must be positive");  // cpu_state.rs:170-172 ZeroTimeStep
    float3 g = gravity ? make_float3(gravity[0], gravity[1], gravity[2]) : make_float3(0.f, 0.f, 0.f);
    if (read_counters(h)) return -1;
    h->force_limits_valid = false;  // fixed substeps (graph replays included) move the particles
    // A previous energy error does not carry over: the reference checks each
    // substep afresh (cpu_state.rs:178-183).
    if (h->host_counters[C_STATUS] & (ST_INVERTED | ST_SAND_MU)) {
        h->host_counters[C_STATUS] &= ~(ST_INVERTED | ST_SAND_MU);
        SV_CUDA(cudaMemcpyAsync(h->counters + C_STATUS, h->host_counters + C_STATUS, 4, cudaMemcpyHostToDevice, h->stream));
        h->pending_valid = false;
    }
    // with a frame input, gravity comes from the input and the pending
    // scatter was made for the substep starting at h->time
    const bool same_inputs = h->pending_valid && h->pending_dt == dt &&
                             (h->fin_active || (h->pending_g[0] == g.x && h->pending_g[1] == g.y && h->pending_g[2] == g.z));
    if (!same_inputs) h->pending_valid = false;
    const uint32_t base = h->host_counters[C_SUBSTEPS];
    // the fp64 conservation sums of sv_get_stats: only the call's last
    // substep takes them (reset to every substep when the call returns)
    struct SumsAt {
        sv_handle *h;
        ~SumsAt() { cudaMemsetAsync(h->counters + C_SUMS_AT, 0, 4, h->stream); }
    } sums_at{h};
    h->host_counters[C_SUMS_AT] = n_substeps ? base + n_substeps - 1 : 0;
    SV_CUDA(cudaMemcpyAsync(h->counters + C_SUMS_AT, h->host_counters + C_SUMS_AT, 4, cudaMemcpyHostToDevice, h->stream));
    const uint32_t fp64_before = h->host_counters[C_FP64];
    uint32_t fallback_before = h->host_counters[C_FALLBACK];
    uint32_t status = 0;
    uint32_t done = 0, timed = 0;
    // Substeps are queued in chunks and the counters read after each.  With
    // a cancel flag the chunks are shorter, so that a cancel request takes
    // effect within 16 substeps of the one running.
    const uint32_t chunk = cancel ? 16 : 64;
    bool canceled = false;
    while (done < n_substeps) {
        if (canceled || (cancel && *cancel)) {
            status |= SV_STATUS_CANCELED;
            break;
        }
        const uint32_t todo = std::min(chunk, n_substeps - done);
        if (!h->pending_valid) {
            if (h->fin_active && !in_frame(h, h->time))
                return fail("sv_step: the substep's time lies outside the loaded frame input (wrong frame loaded)");
            if (standalone_p2g(h, dt, g)) return -1;
        }
        double t_q = h->time;  // start time of the substep after the one launched
        for (uint32_t s = 0; s < todo;) {
            // CUDA graphs: whole binning periods once the binning keys come
            // from the previous substep (steady state), and the start or the
            // rest of a period where the call's substep count cuts one (a
            // 20-substep call with binning every 8 replays 8 + 8 + 4, then
            // 4 + 8 + 8 in the next call)
            if (h->use_graphs && !h->fin_active && !h->deterministic && !h->profiling &&
                (h->since_sort < h->sort_interval || h->keys_valid)) {
                const uint32_t left = todo - s;
                const uint32_t count = h->since_sort >= h->sort_interval
                                           ? std::min(h->sort_interval, left)
                                           : std::min(h->sort_interval - h->since_sort, left);
                if (run_period_graph(h, dt, g, false, count)) return -1;
                s += count;
            } else {
                t_q += (double)dt;
                if (fused_substep(h, dt, g, t_q)) return -1;
                s += 1;
                if (!h->pending_valid) break;  // the frame's last substep: nothing pending
            }
        }
        if (read_counters_polled(h, cancel, &canceled)) return -1;
        const uint32_t st = h->host_counters[C_STATUS];
        done = h->host_counters[C_SUBSTEPS] - base;
        for (; timed < done; ++timed) h->time += (double)dt;  // cpu_state.rs:186-189
        // passes that ran stopped left the state as it was but wrote no
        // binning keys: the next binning computes them afresh
        if (st & STOP_MASK) h->keys_valid = false;
        if (st & ST_OUT_OF_GRID) return fail("sv_step: a live particle left the grid block index");
        if (h->host_counters[C_CLOSURE_ERR]) return fail("sv_step: a tensor-core wait of the learned closure timed out");
        if (st & ST_VARIANT_FULL) return fail("sv_step: the collider variant table is full");
        if (st & ST_SAND_MU) {
            // the reference asserts mu > 0 here (advance_particles.rs:57)
            h->substeps_total += done;
            if (status_out) *status_out = status | SV_STATUS_SAND_INVALID_MU;
            if (substeps_done) *substeps_done = done;
            return fail("sv_step: a sand particle with mu <= 0 was compressed (the reference asserts mu > 0)");
        }
        if (st & (ST_CAPACITY | ST_MOVED_FAR)) {
            if (st & ST_CAPACITY) {
                // Grow and redo what was skipped (gpu_state.rs:562-599 redoes a
                // frame with doubled capacity).
                const uint64_t cap = std::min<uint64_t>(h->layout.total_blocks, h->capacity * 2);
                if (cap <= h->capacity) return fail("sv_step: grid block capacity exhausted");
                SV_CUDA(alloc_grid(h, cap));
                clear_graphs(h);  // they bake the old grid pointers
            }
            // A particle left the blocks claimed at the last binning: its
            // scatter is incomplete, so bin again and redo the scatter.
            if (st & ST_MOVED_FAR) h->sort_interval = std::max<uint32_t>(1, h->sort_interval / 2);
            h->host_counters[C_STATUS] &= ~(ST_CAPACITY | ST_MOVED_FAR);
            SV_CUDA(cudaMemcpyAsync(h->counters + C_STATUS, h->host_counters + C_STATUS, 4, cudaMemcpyHostToDevice,
                                    h->stream));
            SV_CUDA(cudaStreamSynchronize(h->stream));
            h->pending_valid = false;
            // an inversion in the same substeps is still reported below
            if (!(st & ST_INVERTED)) continue;
        }
        if (canceled && done < n_substeps) status |= SV_STATUS_CANCELED;
        if (h->adaptive_interval && todo > 0) {
            // Bin more often when many gathers miss their shared tile, less
            // often when almost none do.
            const double miss = (double)(h->host_counters[C_FALLBACK] - fallback_before) / ((double)h->n * todo + 1.0);
            if (miss > 0.02 && h->sort_interval > 1) h->sort_interval /= 2;
            else if (miss < 0.002 && h->sort_interval < h->max_interval) h->sort_interval *= 2;
        }
        fallback_before = h->host_counters[C_FALLBACK];
        if (st & ST_INVERTED) {
            status |= SV_STATUS_PARTICLE_INVERTED;
            h->pending_valid = false;
            // the failed substep does not advance the time (cpu_state.rs:178-183)
            if (done > 0) h->time -= (double)dt;
            break;
        }
    }
    h->substeps_total += done;
    h->fp64_total += (uint32_t)(h->host_counters[C_FP64] - fp64_before);
    if (status_out) *status_out = status;
    if (substeps_done) *substeps_done = done;
    return 0;
}

// ------------------------------------------------------------------ adaptive time steps
// CpuState::produce_next_state with adaptive_time_steps = true
// (cpu_state.rs:146-197): substeps run while time < target_time, each with
// the phase order of phase/mod.rs:27-41.  The time steps live on the device;
// a substep that starts at or after the target time is a no-op (stop latch).
// A substep runs in the fused form (adaptive_substep_fused) or the split
// one (adaptive_substep), see there.

int sv_step_adaptive(sv_handle *h, double *time_inout, double target_time, float max_time_step,
                     const float gravity[3], const volatile int32_t *cancel, uint32_t *status_out,
                     uint32_t *substeps_done) {
    g_last_error.clear();
    if (!h || !time_inout) return fail("sv_step_adaptive: NULL argument");
    if (status_out) *status_out = 0;
    if (substeps_done) *substeps_done = 0;
    if (!(max_time_step > 0.f)) return fail("sv_step_adaptive: max_time_step must be positive");
    float3 g = gravity ? make_float3(gravity[0], gravity[1], gravity[2]) : make_float3(0.f, 0.f, 0.f);
    adaptive::State st;
    if (!h->adt) {
        SV_CUDA(cudaMalloc(&h->adt, sizeof(adaptive::State)));
        SV_CUDA(cudaMalloc(&h->adt_backup, sizeof(adaptive::State)));
        std::memset(&st, 0, sizeof(st));
        st.vel = st.def = st.sound = st.iso = adaptive::NONE;
        st.hist_len = 0;
    } else {
        SV_CUDA(cudaMemcpyAsync(&st, h->adt, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
        SV_CUDA(cudaStreamSynchronize(h->stream));
    }
    st.max_dt = max_time_step;  // cpu_state.rs:162
    st.time = *time_inout;
    st.target = target_time;
    if (!h->force_limits_valid) {
        // the particles changed since the last advance reduced the force
        // limits: the first substep's k_limits_force reduces them
        st.force_ready = 0;
        st.red_sound = st.red_iso = 0x7f7fffffu;  // FLT_MAX bits
    }
    h->limits_pass_pending = true;
    SV_CUDA(cudaMemcpyAsync(h->adt, &st, sizeof(st), cudaMemcpyHostToDevice, h->stream));
    if (read_counters(h)) return -1;
    h->host_counters[C_STATUS] &= ~(ST_INVERTED | ST_TIME_REACHED | ST_ZERO_DT | ST_SAND_MU);
    SV_CUDA(cudaMemcpyAsync(h->counters + C_STATUS, h->host_counters + C_STATUS, 4, cudaMemcpyHostToDevice, h->stream));
    // the fused path's pending scatter and binning do not survive this call
    h->pending_valid = false;
    h->keys_valid = false;
    h->since_sort = h->sort_interval;
    if (!(st.time < target_time)) return 0;
    const uint32_t base = h->host_counters[C_SUBSTEPS];
    uint32_t fallback_before = h->host_counters[C_FALLBACK], substeps_before = base;
    uint32_t status = 0;
    h->adaptive_active = true;
    const bool fused = !h->fin_active;  // with a frame input the substep runs split
    double t_now = st.time;        // device time after the last batch
    float dt_last = max_time_step; // its last advance step
    int rc = 0;
    bool canceled = false;
    while (true) {
        if (canceled || (cancel && *cancel)) {
            status |= SV_STATUS_CANCELED;
            break;
        }
        // The fused form pays for a speculation that failed with a second
        // pass (and a second scatter): where limits keep binding (a run
        // governed by its velocity limit) the split form is cheaper.  Batches
        // whose speculations failed in more than a fifth of their substeps
        // switch to it for the next eight batches, then the fused form is
        // tried again.
        const bool use_fused = fused && h->adt_split_batches == 0;
        if (!use_fused && h->adt_split_batches > 0) h->adt_split_batches -= 1;
        if (!use_fused) h->pending_valid = false;  // the split form scatters each substep itself
        const uint32_t miss0 = h->host_counters[C_ADT_MISS], done0 = h->host_counters[C_SUBSTEPS];
        // Substeps queued past the target run stopped, yet each still copies
        // the particle state through its passes: queue what the remaining
        // time needs at the last step taken (at most 16; more batches follow
        // when the steps shrink).
        uint32_t want = 16;
        if (dt_last > 0.f) {
            const double need = std::ceil((target_time - t_now) / (double)dt_last - 1e-9);
            want = (uint32_t)std::min(16.0, std::max(1.0, need));
        }
        for (uint32_t s = 0; s < want && rc == 0;) {
            // whole binning periods of the fused form replay CUDA graphs, as
            // in sv_step
            if (use_fused && h->use_graphs && !h->profiling && h->pending_valid && h->keys_valid &&
                h->since_sort >= h->sort_interval && want - s >= h->sort_interval) {
                rc = run_period_graph(h, 0.f, g, true);
                s += h->sort_interval;
            } else {
                rc = use_fused ? adaptive_substep_fused(h, g) : adaptive_substep(h, g);
                if (!use_fused) h->adt_split_substeps += 1;
                s += 1;
            }
        }
        if (rc == 0) {
            adaptive::State now;
            if (cudaMemcpyAsync(&now, h->adt, sizeof(now), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) rc = -1;
            if (rc == 0 && read_counters_polled(h, cancel, &canceled)) rc = -1;  // waits for the copy too
            if (rc == 0) t_now = now.time, dt_last = now.dt_c;
        }
        if (rc) {
            rc = -1;
            break;
        }
        const uint32_t stw = h->host_counters[C_STATUS];
        if (use_fused && 5 * (h->host_counters[C_ADT_MISS] - miss0) > h->host_counters[C_SUBSTEPS] - done0 + 1)
            h->adt_split_batches = 8;
        if (stw & ST_OUT_OF_GRID) {
            rc = fail("sv_step_adaptive: a live particle left the grid block index");
            break;
        }
        if (stw & ST_ZERO_DT) {
            rc = fail("sv_step_adaptive: zero time step");  // Error::ZeroTimeStep
            break;
        }
        if (stw & ST_WRONG_FRAME) {
            rc = fail("sv_step_adaptive: the substep's time lies outside the loaded frame input (wrong frame loaded)");
            break;
        }
        if (stw & ST_VARIANT_FULL) {
            rc = fail("sv_step_adaptive: the collider variant table is full");
            break;
        }
        if (stw & ST_SAND_MU) {
            // the reference asserts mu > 0 here (advance_particles.rs:57)
            status |= SV_STATUS_SAND_INVALID_MU;
            rc = fail("sv_step_adaptive: a sand particle with mu <= 0 was compressed (the reference asserts mu > 0)");
            break;
        }
        if (stw & (STOP_MASK & ~ST_TIME_REACHED)) h->keys_valid = false;  // stopped advances copied in place
        if (stw & (ST_CAPACITY | ST_MOVED_FAR)) {
            if (stw & ST_CAPACITY) {
                const uint64_t cap = std::min<uint64_t>(h->layout.total_blocks, h->capacity * 2);
                if (cap <= h->capacity) {
                    rc = fail("sv_step_adaptive: grid block capacity exhausted");
                    break;
                }
                if (alloc_grid(h, cap) != cudaSuccess) {
                    rc = fail("sv_step_adaptive: grid allocation failed");
                    break;
                }
                clear_graphs(h);
            }
            if (stw & ST_MOVED_FAR) h->sort_interval = std::max<uint32_t>(1, h->sort_interval / 2);
            // Redo the stopped substep from its start, binned afresh, with the
            // adaptive state it began with (its limits not yet in the history)
            // -- unless it completed and only its scatter of the next substep
            // failed (the fused form), which the next substep redoes.
            bool completed = false;
            if (fused) {
                adaptive::State now, back;
                SV_CUDA(cudaMemcpyAsync(&now, h->adt, sizeof(now), cudaMemcpyDeviceToHost, h->stream));
                SV_CUDA(cudaMemcpyAsync(&back, h->adt_backup, sizeof(back), cudaMemcpyDeviceToHost, h->stream));
                SV_CUDA(cudaStreamSynchronize(h->stream));
                completed = now.substeps != back.substeps;
            }
            if (!completed)
                SV_CUDA(cudaMemcpyAsync(h->adt, h->adt_backup, sizeof(adaptive::State), cudaMemcpyDeviceToDevice,
                                        h->stream));
            h->pending_valid = false;
            h->limits_pass_pending = true;
            h->since_sort = h->sort_interval;
            h->host_counters[C_STATUS] &= ~(ST_CAPACITY | ST_MOVED_FAR);
            SV_CUDA(cudaMemcpyAsync(h->counters + C_STATUS, h->host_counters + C_STATUS, 4, cudaMemcpyHostToDevice,
                                    h->stream));
            if (!(stw & ST_INVERTED)) continue;
        }
        if (h->adaptive_interval) {
            // as in sv_step: bin more often when many gathers miss their tile
            const double miss = (double)(h->host_counters[C_FALLBACK] - fallback_before) /
                                ((double)h->n * (h->host_counters[C_SUBSTEPS] - substeps_before) + 1.0);
            if (miss > 0.02 && h->sort_interval > 1) h->sort_interval /= 2;
            else if (miss < 0.002 && h->sort_interval < h->max_interval) h->sort_interval *= 2;
        }
        fallback_before = h->host_counters[C_FALLBACK];
        substeps_before = h->host_counters[C_SUBSTEPS];
        if (stw & ST_INVERTED) {
            status |= SV_STATUS_PARTICLE_INVERTED;
            break;
        }
        if (stw & ST_TIME_REACHED) break;
    }
    h->adaptive_active = false;
    h->keys_valid = false;
    h->pending_valid = false;  // a scatter made at adaptive steps
    h->force_limits_valid = rc == 0;
    if (rc) {
        if (status_out) *status_out = status;
        if (substeps_done) *substeps_done = h->host_counters[C_SUBSTEPS] - base;
        return -1;
    }
    SV_CUDA(cudaMemcpyAsync(&st, h->adt, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    SV_CUDA(cudaStreamSynchronize(h->stream));
    h->host_counters[C_STATUS] &= ~ST_TIME_REACHED;
    SV_CUDA(cudaMemcpy(h->counters + C_STATUS, h->host_counters + C_STATUS, 4, cudaMemcpyHostToDevice));
    const uint32_t done = h->host_counters[C_SUBSTEPS] - base;
    h->substeps_total += done;
    *time_inout = st.time;
    h->time = st.time;
    if (status_out) *status_out = status;
    if (substeps_done) *substeps_done = done;
    return 0;
}

int sv_time_step_limits(sv_handle *h, float out[8]) {
    g_last_error.clear();
    if (!h || !out) return fail("sv_time_step_limits: NULL argument");
    for (int k = 0; k < 8; ++k) out[k] = adaptive::NONE;
    if (!h->adt) return 0;
    adaptive::State st;
    SV_CUDA(cudaMemcpyAsync(&st, h->adt, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    SV_CUDA(cudaStreamSynchronize(h->stream));
    out[0] = st.dt_a, out[1] = st.dt_b, out[2] = st.dt_c;
    out[3] = st.vel, out[4] = st.def, out[5] = st.sound, out[6] = st.iso;
    out[7] = adaptive::allowed(st);
    return 0;
}

int sv_p2g_only(sv_handle *h, float dt, const float gravity[3]) {
    g_last_error.clear();
    if (!h) return fail("sv_p2g_only: NULL handle");
    float3 g = gravity ? make_float3(gravity[0], gravity[1], gravity[2]) : make_float3(0.f, 0.f, 0.f);
    if (standalone_p2g(h, dt, g)) return -1;
    SV_CUDA(launch_grid_update(h, false));
    h->vel_side = h->gcur;
    h->vel_map = h->map_cur;
    // the grid now holds velocities: the next substep scatters again
    h->pending_valid = false;
    if (read_counters(h)) return -1;
    if (h->host_counters[C_STATUS] & ST_CAPACITY) return fail("sv_p2g_only: grid block capacity exceeded");
    return 0;
}

int sv_download(sv_handle *h, sv_particles *o) {
    g_last_error.clear();
    if (!h || !o) return fail("sv_download: NULL argument");
    if (o->n != h->n) return fail("sv_download: particle count mismatch");
    if (h->direct_host) return download_direct(h, o, 0, h->n);  // kernels write the caller's arrays (sv_transfer.cu)
    const uint64_t n = h->n;
    const ParticleArrays &a = h->side[h->cur];
    std::vector<float4> pos(n), vel(n);
    std::vector<int4> cellv(h->layout.position_form == 1 ? n : 0);
    std::vector<float> C(9 * n), F(9 * n), en(n);
    std::vector<uint32_t> orig(n), cbits(a.cbits_done ? n : 0);
    HostParticles hp;
    hp.n = n;
    hp.pos = pos.data(), hp.vel = vel.data(), hp.cell = cellv.empty() ? nullptr : cellv.data();
    hp.C = C.data(), hp.F = F.data(), hp.energy = en.data();
    hp.orig = orig.data(), hp.cbits = cbits.empty() ? nullptr : cbits.data();
    SV_CUDA(copy_particles_async(h, hp));
    SV_CUDA(cudaStreamSynchronize(h->stream));
    if (!unpack_particles(hp, unpack_info(h, false), o)) return fail("sv_download: corrupt original index");
    return 0;
}

int sv_download_scene(sv_handle *h, uint32_t scene, sv_particles *o) {
    g_last_error.clear();
    if (!h || !o) return fail("sv_download_scene: NULL argument");
    if (scene >= h->host_scenes.size()) return fail("sv_download_scene: no such scene");
    const uint64_t b = h->scene_first[scene], m = h->scene_first[scene + 1] - b;
    if (o->n != m) return fail("sv_download_scene: particle count mismatch");
    if (h->direct_host) {
        // the scene's range only, straight into the caller's arrays
        return download_direct(h, o, b, m);
    }
    const uint64_t n = h->n;
    std::vector<uint32_t> flags(n), bits(n);
    std::vector<float> x(3 * n), F(9 * n), v(3 * n), C(9 * n), en(n), pj(n);
    sv_particles all{};
    all.n = n;
    all.flags = flags.data(), all.positions = x.data(), all.position_gradients = F.data();
    all.velocities = v.data(), all.velocity_gradients = C.data(), all.elastic_energies = en.data();
    all.collider_bits = bits.data(), all.plastic_j = pj.data();
    if (sv_download(h, &all) < 0) return -1;
    if (o->flags) std::memcpy(o->flags, flags.data() + b, m * 4);
    if (o->positions) std::memcpy(o->positions, x.data() + 3 * b, m * 12);
    if (o->position_gradients) std::memcpy(o->position_gradients, F.data() + 9 * b, m * 36);
    if (o->velocities) std::memcpy(o->velocities, v.data() + 3 * b, m * 12);
    if (o->velocity_gradients) std::memcpy(o->velocity_gradients, C.data() + 9 * b, m * 36);
    if (o->elastic_energies) std::memcpy(o->elastic_energies, en.data() + b, m * 4);
    if (o->collider_bits) std::memcpy(o->collider_bits, bits.data() + b, m * 4);
    if (o->plastic_j) std::memcpy(o->plastic_j, pj.data() + b, m * 4);
    return 0;
}

int sv_download_grid(sv_handle *h, int32_t *node_ids, float *masses, float *velocities, uint64_t capacity,
                     uint64_t *count) {
    g_last_error.clear();
    if (!h) return fail("sv_download_grid: NULL handle");
    if (read_counters(h)) return -1;
    uint64_t slots = 0, var_cap = 0;
    grid_sizes(h, slots, var_cap);
    std::vector<uint32_t> active(slots);
    std::vector<float4> g(slots * 64);
    HostGrid hg;
    hg.slots = slots, hg.active = active.data(), hg.grid = g.data();  // the bits-0 nodes only
    SV_CUDA(copy_grid_async(h, hg));
    SV_CUDA(cudaStreamSynchronize(h->stream));
    const std::vector<GridNode> nodes = grid_nodes(hg, h->layout);
    if (count) *count = nodes.size();
    for (uint64_t i = 0; i < nodes.size() && i < capacity; ++i) {
        if (node_ids) std::memcpy(&node_ids[3 * i], nodes[i].id, 12);
        if (masses) masses[i] = nodes[i].v.w;
        if (velocities) velocities[3 * i] = nodes[i].v.x, velocities[3 * i + 1] = nodes[i].v.y, velocities[3 * i + 2] = nodes[i].v.z;
    }
    return 0;
}

int sv_binning(sv_handle *h, uint32_t *keys, uint32_t *perm, uint32_t *original_index) {
    g_last_error.clear();
    if (!h) return fail("sv_binning: NULL handle");
    if (!h->keys_valid) SV_CUDA(launch_keys(h));
    SV_CUDA(launch_sort_and_segments(h));
    // the segments changed: the next substep bins and scatters afresh
    h->pending_valid = false;
    SV_CUDA(cudaStreamSynchronize(h->stream));
    const uint64_t n = h->n;
    if (keys) SV_CUDA(cudaMemcpy(keys, h->keys, n * 4, cudaMemcpyDeviceToHost));
    if (perm) SV_CUDA(cudaMemcpy(perm, h->perm, n * 4, cudaMemcpyDeviceToHost));
    if (original_index) SV_CUDA(cudaMemcpy(original_index, h->side[h->cur].orig, n * 4, cudaMemcpyDeviceToHost));
    return 0;
}

int sv_grid_layout(sv_handle *h, int32_t origin[3], int32_t nblocks[3]) {
    if (!h) return fail("sv_grid_layout: NULL handle");
    for (int a = 0; a < 3; ++a) {
        if (origin) origin[a] = h->layout.origin[a];
        if (nblocks) nblocks[a] = h->layout.nb[a];
    }
    return 0;
}

int sv_sort_pairs(const uint32_t *keys, uint32_t *perm, uint64_t n) {
    g_last_error.clear();
    if (n == 0) return 0;
    if (!keys || !perm) return fail("sv_sort_pairs: NULL argument");
    if (n >= (1ull << 32)) return fail("sv_sort_pairs: n must be below 2^32");
    uint32_t *dk = nullptr, *dko = nullptr, *dv = nullptr;
    void *temp = nullptr;
    size_t tb = radix_sort_temp_bytes(n);
    // sort on the significant bits only: the passes follow the largest key
    uint32_t any = 0;
    for (uint64_t i = 0; i < n; ++i) any |= keys[i];
    int key_bits = 1;  // all-zero keys still take one pass, which writes the identity
    while (key_bits < 32 && (any >> key_bits) != 0) ++key_bits;
    cudaError_t e;
    if ((e = cudaMalloc(&dk, n * 4)) || (e = cudaMalloc(&dko, n * 4)) || (e = cudaMalloc(&dv, n * 4)) ||
        (e = cudaMalloc(&temp, tb)) || (e = cudaMemcpy(dk, keys, n * 4, cudaMemcpyHostToDevice)) ||
        (e = radix_sort_pairs(dk, nullptr, dko, dv, n, key_bits, temp, 0)) ||
        (e = cudaMemcpy(perm, dv, n * 4, cudaMemcpyDeviceToHost))) {
        cudaFree(dk), cudaFree(dko), cudaFree(dv), cudaFree(temp);
        return fail(std::string("sv_sort_pairs: ") + cudaGetErrorString(e));
    }
    cudaFree(dk), cudaFree(dko), cudaFree(dv), cudaFree(temp);
    return 0;
}

int sv_get_stats(sv_handle *h, sv_stats *out) {
    if (!h || !out) return fail("sv_get_stats: NULL argument");
    if (read_counters(h)) return -1;
    out->particles = h->n;
    out->live_particles = h->host_counters[C_NLIVE];
    out->particle_blocks = h->host_counters[C_NSEG];
    out->grid_blocks = h->host_counters[C_NSLOT0 + h->map_cur];
    out->fp64_svd = h->fp64_total;
    out->substeps = h->substeps_total;
    out->device_bytes = h->device_bytes;
    out->kernel_launches = h->launches;
    out->sorts = h->sorts;
    out->sort_interval = h->sort_interval;
    out->tile_misses = h->host_counters[C_FALLBACK];
    out->graph_replays = h->graph_launches;
    out->cta_per_sm = h->cta_per_sm;
    out->closure_learned = h->host_counters[C_CLOSURE];
    out->closure_fallbacks = h->host_counters[C_CLOSURE_FB];
    out->closure_mode = (uint64_t)h->closure_mode;
    out->adaptive_misses = h->host_counters[C_ADT_MISS];
    out->adaptive_split = h->adt_split_substeps;
    // the grid the last substep gathered from (its sums were taken by the
    // grid update that turned it into velocities)
    double sums[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    SV_CUDA(cudaMemcpy(sums, h->grid_sums, sizeof(sums), cudaMemcpyDeviceToHost));
    const int gs = h->vel_side >= 0 ? h->vel_side : h->gcur;
    out->grid_mass = sums[4 * gs];
    for (int a = 0; a < 3; ++a) out->grid_momentum[a] = sums[4 * gs + 1 + a];
    uint64_t timer[3] = {0, 0, 0};
    SV_CUDA(cudaMemcpy(timer, h->pass_timer, sizeof(timer), cudaMemcpyDeviceToHost));
    out->pass_ns = timer[1];
    out->pass_count = timer[2];
    return 0;
}

int sv_autotune(sv_handle *h, float dt, const float gravity[3], uint32_t substeps_per_trial, uint32_t *sort_interval_out,
                uint32_t *cta_per_sm_out) {
    g_last_error.clear();
    if (!h) return fail("sv_autotune: NULL handle");
    if (!(dt > 0.f)) return fail("sv_autotune: dt must be positive");
    if (substeps_per_trial == 0) substeps_per_trial = 16;
    // snapshot of the current particle side (trials advance it)
    ParticleArrays &a = h->side[h->cur];
    const uint64_t n = h->n;
    const bool cell = h->layout.position_form == 1;
    struct Span {
        void *dev;
        size_t bytes;
        void *copy;
    };
    std::vector<Span> spans = {{a.pos, n * 16, nullptr}, {a.vel, n * 16, nullptr}, {a.C, n * 36, nullptr},
                               {a.F, n * 36, nullptr},   {a.energy, n * 4, nullptr}, {a.orig, n * 4, nullptr}};
    if (cell) spans.push_back({a.cell, n * 16, nullptr});
    auto release = [&]() {
        for (auto &s : spans) cudaFree(s.copy);
    };
    SV_CUDA(cudaStreamSynchronize(h->stream));
    for (auto &s : spans) {
        cudaError_t e = cudaMalloc(&s.copy, s.bytes ? s.bytes : 16);
        if (e != cudaSuccess) {
            release();
            return fail(std::string("sv_autotune: ") + cudaGetErrorString(e));
        }
        cudaMemcpyAsync(s.copy, s.dev, s.bytes, cudaMemcpyDeviceToDevice, h->stream);
    }
    const int cur0 = h->cur;
    const uint64_t substeps0 = h->substeps_total, fp64_0 = h->fp64_total;
    auto restore = [&]() {
        cudaStreamSynchronize(h->stream);
        h->cur = cur0;
        ParticleArrays &b = h->side[h->cur];
        void *dst[] = {b.pos, b.vel, b.C, b.F, b.energy, b.orig, b.cell};
        // on the handle's stream: the kernels that follow read the restored state
        for (size_t i = 0; i < spans.size(); ++i)
            cudaMemcpyAsync(dst[i], spans[i].copy, spans[i].bytes, cudaMemcpyDeviceToDevice, h->stream);
        h->pending_valid = false;
        h->keys_valid = false;
        h->since_sort = 0;
        cudaMemsetAsync(h->counters + C_STATUS, 0, 4, h->stream);
    };
    // Every candidate starts from the snapshot, warms up over two of its
    // binning periods (its first scatter, the CUDA graph capture, the
    // binning pattern of its steady state), then times three repeats of at
    // least 48 substeps; the median repeat ranks it.  The configuration the
    // handle had is a candidate too, and it is kept unless another one is
    // faster by more than 2 %.
    const uint32_t si0 = h->sort_interval, cta0 = h->cta_per_sm;
    const bool adaptive0 = h->adaptive_interval;
    struct Cand {
        uint32_t si, cta;
    };
    // Two stages: the binning interval at the handle's CTAs per SM, then the
    // CTAs per SM at the best interval (the plain fused pass runs as one
    // resident wave whatever that setting is; the other passes use it).
    std::vector<Cand> cands = {{si0, cta0}};
    for (uint32_t si : {2u, 4u, 6u, 8u, 12u, 16u})
        if (si != si0) cands.push_back({si, cta0});
    const size_t stage1 = cands.size();
    const uint32_t trial = std::max<uint32_t>(substeps_per_trial, 48);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0), cudaEventCreate(&e1);
    h->adaptive_interval = false;
    double ms_default = 0.0, best_ms = 1e300;
    uint32_t best_si = si0, best_cta = cta0;
    for (size_t ci = 0;; ++ci) {
        if (ci == stage1)
            for (uint32_t cta : {8u, 16u, 32u, 64u})
                if (cta != cta0) cands.push_back({best_si, cta});
        if (ci >= cands.size()) break;
        const Cand c = cands[ci];
        restore();
        clear_graphs(h);
        h->sort_interval = h->max_interval = c.si;
        h->cta_per_sm = c.cta;
        uint32_t st = 0, done = 0;
        if (sv_step(h, 2 * c.si + 2, dt, gravity, nullptr, &st, &done) < 0 || st) continue;
        double rep[3];
        bool ok = true;
        for (int r = 0; r < 3 && ok; ++r) {
            const uint32_t k = ((trial + c.si - 1) / c.si) * c.si;  // whole binning periods
            cudaEventRecord(e0, h->stream);
            ok = sv_step(h, k, dt, gravity, nullptr, &st, &done) == 0 && st == 0;
            cudaEventRecord(e1, h->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            rep[r] = (double)ms / k;
        }
        if (!ok) continue;
        std::sort(rep, rep + 3);
        const double med = rep[1];
        if (ci == 0) ms_default = med;
        if (med < best_ms) best_ms = med, best_si = c.si, best_cta = c.cta;
    }
    if (ms_default > 0.0 && best_ms > ms_default * 0.98) best_si = si0, best_cta = cta0;
    const bool keep_default = best_si == si0 && best_cta == cta0;
    cudaEventDestroy(e0), cudaEventDestroy(e1);
    restore();
    release();
    clear_graphs(h);
    // a kept default keeps its adaptive interval; a tuned interval is fixed
    h->adaptive_interval = keep_default && adaptive0;
    h->sort_interval = best_si;
    h->max_interval = keep_default && adaptive0 ? 8 : best_si;
    h->cta_per_sm = best_cta;
    h->substeps_total = substeps0, h->fp64_total = fp64_0;
    if (sort_interval_out) *sort_interval_out = best_si;
    if (cta_per_sm_out) *cta_per_sm_out = best_cta;
    g_last_error.clear();
    return 0;
}

int sv_set_graphs(sv_handle *h, int enable) {
    if (!h) return fail("sv_set_graphs: NULL handle");
    h->use_graphs = enable != 0;
    return 0;
}

int sv_set_host_transfer(sv_handle *h, uint32_t mode, uint32_t *direct) {
    if (!h) return fail("sv_set_host_transfer: NULL handle");
    if (mode > 1) return fail("sv_set_host_transfer: mode must be 0 or 1");
    h->direct_host = mode == 0 && pageable_access();
    if (direct) *direct = h->direct_host ? 1u : 0u;
    return 0;
}

int sv_set_stream(sv_handle *h, void *stream) {
    if (!h) return fail("sv_set_stream: NULL handle");
    SV_CUDA(cudaStreamSynchronize(h->stream));
    h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    clear_graphs(h);
    return 0;
}

int sv_set_profiling(sv_handle *h, int enable) {
    if (!h) return fail("sv_set_profiling: NULL handle");
    h->profiling = enable != 0;
    return 0;
}

int sv_profile_report(sv_handle *h, char *buffer, uint64_t capacity) {
    if (!h) return fail("sv_profile_report: NULL handle");
    SV_CUDA(cudaStreamSynchronize(h->stream));
    for (auto &p : h->timer.pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        auto &t = h->timer.totals[p.first];
        t.first += 1, t.second += ms;
        cudaEventDestroy(p.second.first), cudaEventDestroy(p.second.second);
    }
    h->timer.pending.clear();
    std::string s = "{";
    bool first = true;
    for (auto &kv : h->timer.totals) {
        char buf[256];
        snprintf(buf, sizeof buf, "%s\"%s\": {\"launches\": %llu, \"ms\": %.6f}", first ? "" : ", ", kv.first.c_str(),
                 (unsigned long long)kv.second.first, kv.second.second);
        s += buf;
        first = false;
    }
    s += "}";
    if (buffer && capacity) {
        size_t m = std::min<size_t>(s.size(), capacity - 1);
        std::memcpy(buffer, s.data(), m);
        buffer[m] = 0;
    }
    h->timer.totals.clear();
    return (int)s.size();
}

}  // extern "C"
