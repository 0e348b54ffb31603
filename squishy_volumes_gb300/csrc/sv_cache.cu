// sv_cache.cu -- the state back on the host, the reference's frame files and
// an asynchronous frame cache.
//
//  - copy_particles_async / unpack_particles: one particle side to the host
//    and back into the original particle order (the reference's
//    reverse_sort_map restore in CpuState::to_io_state, cpu/src/cpu_state.rs:71-104);
//    sv_download and the cache share them.
//  - copy_grid_async / grid_nodes: the grid gathered by the last substep as
//    (node, collider bits) entries sorted like the reference's GridKey
//    (cpu_state.rs:106-128; cpu/src/grid_nodes.rs:15-33).
//  - sv_frame_write / sv_frame_read: IoState::write / read
//    (file_frame/src/io_state.rs:31-75): magic and version bytes
//    (file_util/src/lib.rs:27-99), then bincode 1.3.3 with its default
//    options over IoState (io_state.rs:11-18), Particles (particles.rs:92-109),
//    ParticleParameters (:55-90) and GridNodes (grid_nodes.rs:10-15).
//  - sv_cache_*: the store thread (cache/src/store_thread.rs:27-110) with
//    frame_path (cache/src/util.rs:9-11).  A store queues the device-to-host
//    copies on the handle's stream and returns; the writer thread waits for
//    them, restores the particle order, serialises and writes.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sv_collide.cuh"
#include "sv_internal.h"

static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "frame files are little endian; so is the host");

namespace sv {

// ------------------------------------------------------------------ state copies
namespace {

// The current particle side as device pointers in HostParticles' shape.
HostParticles device_view(const sv_handle *h) {
    const ParticleArrays &a = h->side[h->cur];
    HostParticles v;
    v.n = h->n;
    v.pos = a.pos, v.vel = a.vel, v.cell = h->layout.position_form == 1 ? a.cell : nullptr;
    v.C = a.C, v.F = a.F, v.energy = a.energy, v.orig = a.orig, v.cbits = a.cbits_done;
    return v;
}

// The grid the last substep gathered (and its variant table) likewise.
HostGrid device_grid_view(const sv_handle *h, uint64_t slots, uint64_t var_cap) {
    HostGrid v;
    v.slots = slots, v.var_cap = var_cap;
    if (slots) v.active = h->active[h->vel_map], v.grid = h->grid[h->vel_side];
    if (var_cap) {
        // the variant table the last substep gathered from (melded velocities)
        const int s = h->vel_side;
        v.var_key = h->var_key[s], v.var_bits = h->var_bits[s], v.var_vel = h->var_vel[s];
    }
    return v;
}

}  // namespace

// Copies between any two such views (device or host memory) on `s`; the
// arrays dst lacks (cell, cbits) are skipped.
cudaError_t copy_particles(const HostParticles &d, const HostParticles &a, cudaStream_t s) {
    const uint64_t n = a.n;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d.pos, a.pos, n * 16, cudaMemcpyDefault, s)) ||
        (e = cudaMemcpyAsync(d.vel, a.vel, n * 16, cudaMemcpyDefault, s)) ||
        (e = cudaMemcpyAsync(d.C, a.C, 9 * n * 4, cudaMemcpyDefault, s)) ||
        (e = cudaMemcpyAsync(d.F, a.F, 9 * n * 4, cudaMemcpyDefault, s)) ||
        (e = cudaMemcpyAsync(d.energy, a.energy, n * 4, cudaMemcpyDefault, s)) ||
        (e = cudaMemcpyAsync(d.orig, a.orig, n * 4, cudaMemcpyDefault, s)))
        return e;
    if (d.cell && a.cell && (e = cudaMemcpyAsync(d.cell, a.cell, n * 16, cudaMemcpyDefault, s))) return e;
    if (d.cbits && a.cbits && (e = cudaMemcpyAsync(d.cbits, a.cbits, n * 4, cudaMemcpyDefault, s))) return e;
    return cudaSuccess;
}

cudaError_t copy_grid(const HostGrid &d, const HostGrid &a, cudaStream_t s) {
    cudaError_t e;
    if (a.slots) {
        if ((e = cudaMemcpyAsync(d.active, a.active, a.slots * 4, cudaMemcpyDefault, s)) ||
            (e = cudaMemcpyAsync(d.grid, a.grid, a.slots * 64 * sizeof(float4), cudaMemcpyDefault, s)))
            return e;
    }
    if (a.var_cap) {
        const uint64_t c = a.var_cap;
        if ((e = cudaMemcpyAsync(d.var_key, a.var_key, c * sizeof(unsigned long long), cudaMemcpyDefault, s)) ||
            (e = cudaMemcpyAsync(d.var_bits, a.var_bits, c * col::VK * 4, cudaMemcpyDefault, s)) ||
            (e = cudaMemcpyAsync(d.var_vel, a.var_vel, c * col::VK * sizeof(float4), cudaMemcpyDefault, s)))
            return e;
    }
    return cudaSuccess;
}

cudaError_t copy_particles_async(sv_handle *h, const HostParticles &d) {
    return copy_particles(d, device_view(h), h->stream);
}

UnpackInfo unpack_info(const sv_handle *h, bool own_bits) {
    UnpackInfo u;
    u.cell = h->layout.position_form == 1;
    u.dx = h->layout.dx;
    u.scenes = h->host_scenes;
    u.materials = h->host_materials;
    u.stepped = h->substeps_total > 0;
    if (own_bits) u.initial_bits_copy = h->collider_bits;
    else u.initial_bits = h->collider_bits.data();
    return u;
}

bool unpack_particles(const HostParticles &src, const UnpackInfo &u, sv_particles *o) {
    const uint64_t n = src.n;
    const uint32_t *bits0 = u.initial_bits_copy.empty() ? u.initial_bits : u.initial_bits_copy.data();
    for (uint64_t s = 0; s < n; ++s) {
        const uint64_t i = src.orig[s];
        if (i >= n) return false;
        const float4 p = src.pos[s], v = src.vel[s];
        uint32_t packed;
        std::memcpy(&packed, &p.w, 4);
        if (o->flags) o->flags[i] = packed & FLAG_MASK;
        if (o->positions) {
            if (!u.cell) {
                o->positions[3 * i] = p.x, o->positions[3 * i + 1] = p.y, o->positions[3 * i + 2] = p.z;
            } else {
                // back to the scene's own coordinates
                const uint32_t mi = packed >> MATERIAL_SHIFT;
                const SceneInfo &sc = u.scenes[mi < u.materials.size() ? u.materials[mi].scene : 0];
                const int4 c = src.cell[s];
                o->positions[3 * i] = (float)(((double)(c.x - sc.off[0]) + p.x) * u.dx);
                o->positions[3 * i + 1] = (float)(((double)(c.y - sc.off[1]) + p.y) * u.dx);
                o->positions[3 * i + 2] = (float)(((double)(c.z - sc.off[2]) + p.z) * u.dx);
            }
        }
        if (o->velocities) o->velocities[3 * i] = v.x, o->velocities[3 * i + 1] = v.y, o->velocities[3 * i + 2] = v.z;
        if (o->plastic_j) o->plastic_j[i] = v.w;
        for (int k = 0; k < 9; ++k) {
            if (o->position_gradients) o->position_gradients[9 * i + k] = src.F[(uint64_t)k * n + s];
            if (o->velocity_gradients) o->velocity_gradients[9 * i + k] = src.C[(uint64_t)k * n + s];
        }
        if (o->elastic_energies) o->elastic_energies[i] = src.energy[s];
        if (o->collider_bits) {
            // without colliders every substep's Collide clears a live
            // particle's bits (collide.rs:53-56)
            if (src.cbits) o->collider_bits[i] = src.cbits[s];
            else o->collider_bits[i] = (u.stepped && !(packed & SV_TOMBSTONED)) ? 0u : (bits0 ? bits0[i] : 0u);
        }
    }
    return true;
}

void grid_sizes(const sv_handle *h, uint64_t &slots, uint64_t &var_cap) {
    slots = h->vel_side < 0 ? 0 : std::min<uint64_t>(h->host_counters[C_NSLOT0 + h->vel_map], h->capacity);
    var_cap = (h->fin_active && h->vel_side >= 0 && h->var_key[h->vel_side]) ? h->var_cap : 0;
}

cudaError_t copy_grid_async(sv_handle *h, const HostGrid &d) {
    return copy_grid(d, device_grid_view(h, d.slots, d.var_cap), h->stream);
}

std::vector<GridNode> grid_nodes(const HostGrid &g, const GridLayout &L) {
    std::vector<GridNode> nodes;
    for (uint64_t s = 0; s < g.slots; ++s) {
        const uint32_t b = g.active[s];
        const int bz = (int)(b % (uint32_t)L.nb[2]), r = (int)(b / (uint32_t)L.nb[2]);
        const int by = r % L.nb[1], bx = r / L.nb[1];
        for (int l = 0; l < 64; ++l) {
            const float4 v = g.grid[s * 64 + l];
            if (!(v.w > 0.f)) continue;
            GridNode nd;
            nd.id[0] = L.origin[0] + 4 * bx + (l >> 4);
            nd.id[1] = L.origin[1] + 4 * by + ((l >> 2) & 3);
            nd.id[2] = L.origin[2] + 4 * bz + (l & 3);
            nd.bits = 0;
            nd.v = v;
            nodes.push_back(nd);
        }
    }
    for (uint64_t e = 0; e < g.var_cap; ++e) {
        const unsigned long long k = g.var_key[e];
        if (k == 0ull) continue;
        // node key: 21 bits per axis, biased by 2^20, plus one (col::node_key)
        const unsigned long long q = k - 1ull;
        const int32_t id[3] = {(int32_t)((q >> 42) & 0x1FFFFFull) - (1 << 20), (int32_t)((q >> 21) & 0x1FFFFFull) - (1 << 20),
                               (int32_t)(q & 0x1FFFFFull) - (1 << 20)};
        for (int j = 0; j < col::VK; ++j) {
            const uint32_t bits = g.var_bits[e * col::VK + j];
            const float4 v = g.var_vel[e * col::VK + j];
            if (!bits || !(v.w > 0.f)) continue;
            GridNode nd;
            std::memcpy(nd.id, id, 12);
            nd.bits = bits;
            nd.v = v;
            nodes.push_back(nd);
        }
    }
    std::sort(nodes.begin(), nodes.end(), [](const GridNode &x, const GridNode &y) {
        if (x.id[0] != y.id[0]) return x.id[0] < y.id[0];
        if (x.id[1] != y.id[1]) return x.id[1] < y.id[1];
        if (x.id[2] != y.id[2]) return x.id[2] < y.id[2];
        return x.bits < y.bits;
    });
    return nodes;
}

}  // namespace sv

using namespace sv;

namespace {

// ------------------------------------------------------------------ frame file format
constexpr size_t MAGIC_LEN = 32, VERSION_LEN = 64;  // file_util/src/lib.rs:27-29
constexpr char MAGIC[MAGIC_LEN + 1] = "Squishy Volumes Frame File Magic";  // io_state.rs:20-29

int cfail(const std::string &msg) {
    set_last_error(msg);
    return -1;
}

std::string version_or_default(const char *v) { return v ? std::string(v) : std::string(SV_FRAME_VERSION); }

// Buffered little-endian output; remembers the first failure.
struct Sink {
    FILE *f = nullptr;
    std::vector<uint8_t> buf = std::vector<uint8_t>(1 << 22);
    size_t used = 0;
    uint64_t total = 0;
    bool ok = true;
    void flush() {
        if (used && ok && std::fwrite(buf.data(), 1, used, f) != used) ok = false;
        used = 0;
    }
    void put(const void *p, size_t bytes) {
        const uint8_t *s = static_cast<const uint8_t *>(p);
        total += bytes;
        while (bytes) {
            if (used == buf.size()) flush();
            const size_t k = std::min(bytes, buf.size() - used);
            std::memcpy(buf.data() + used, s, k);
            used += k, s += k, bytes -= k;
        }
    }
    template <class T> void scalar(T v) { put(&v, sizeof(T)); }
    void len(uint64_t n) { scalar<uint64_t>(n); }  // bincode sequence length
    // a Vec of `n` elements of `width` values each (0 where the array is absent)
    template <class T> void vec(const T *a, uint64_t n, int width) {
        len(n);
        if (a) {
            put(a, (size_t)n * width * sizeof(T));
        } else {
            const T z[9] = {};
            for (uint64_t i = 0; i < n; ++i) put(z, width * sizeof(T));
        }
    }
};

template <class T> T at(const T *a, uint64_t i) { return a ? a[i] : T(0); }

// IoState (io_state.rs:11-18) through bincode's serde data model: structs as
// their fields in order, [T; N] as N elements, Vec as u64 length + elements,
// Option as u8 0 / 1 + value, enums as u32 variant index + fields.
void serialise(Sink &w, const sv_frame &f) {
    const uint64_t n = f.n;
    w.scalar<double>(f.time);
    w.vec(f.flags, n, 1);
    w.len(n);  // parameters: Vec<ParticleParameters>
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t fl = at(f.flags, i);
        w.scalar<float>(at(f.mass, i));
        w.scalar<float>(at(f.initial_volume, i));
        if (fl & SV_USE_VISCOSITY) {
            w.scalar<uint8_t>(1);
            w.scalar<float>(at(f.viscosity_dynamic, i));
            w.scalar<float>(at(f.viscosity_bulk, i));
        } else {
            w.scalar<uint8_t>(0);
        }
        if (fl & SV_IS_FLUID) {
            w.scalar<uint32_t>(1);  // Fluid { exponent, bulk_modulus }
            w.scalar<int32_t>(at(f.exponent, i));
            w.scalar<float>(at(f.bulk_modulus, i));
        } else {
            w.scalar<uint32_t>(0);  // Solid { mu, lambda, sand_alpha }
            w.scalar<float>(at(f.mu, i));
            w.scalar<float>(at(f.lambda, i));
            if (fl & SV_USE_SAND_ALPHA) {
                w.scalar<uint8_t>(1);
                w.scalar<float>(at(f.sand_alpha, i));
            } else {
                w.scalar<uint8_t>(0);
            }
        }
    }
    w.vec(f.elastic_energies, n, 1);
    w.vec(f.collider_bits, n, 1);
    w.vec(f.positions, n, 3);
    w.vec(f.position_gradients, n, 9);
    w.vec(f.velocities, n, 3);
    w.vec(f.velocity_gradients, n, 9);
    w.vec(f.initial_positions, n, 3);
    if (f.has_grid) {
        const uint64_t m = f.n_nodes;
        w.scalar<uint8_t>(1);
        w.vec(f.node_ids, m, 3);
        w.vec(f.node_collider_bits, m, 1);
        w.vec(f.node_masses, m, 1);
        w.vec(f.node_velocities, m, 3);
    } else {
        w.scalar<uint8_t>(0);
    }
}

// Writes next to `path` first and renames, like IoState::write.
std::string write_frame_file(const char *path, const sv_frame &f, const std::string &version, uint64_t &bytes) {
    if (version.size() > VERSION_LEN) return "frame file: version string longer than 64 bytes";
    const std::string temp = std::string(path) + ".temp";
    Sink w;
    w.f = std::fopen(temp.c_str(), "wb");
    if (!w.f) return "frame file: cannot create " + temp;
    w.put(MAGIC, MAGIC_LEN);
    char vb[VERSION_LEN] = {};
    std::memcpy(vb, version.data(), version.size());
    w.put(vb, VERSION_LEN);
    serialise(w, f);
    w.flush();
    const bool closed = std::fclose(w.f) == 0;
    if (!w.ok || !closed) {
        std::remove(temp.c_str());
        return "frame file: writing " + temp + " failed";
    }
    if (std::rename(temp.c_str(), path) != 0) {
        std::remove(temp.c_str());
        return std::string("frame file: cannot move it to ") + path;
    }
    bytes = w.total;
    return "";
}

// Buffered input; remembers running out of bytes.
struct Source {
    FILE *f = nullptr;
    std::vector<uint8_t> buf = std::vector<uint8_t>(1 << 22);
    size_t pos = 0, end = 0;
    bool ok = true;
    void get(void *p, size_t bytes) {
        uint8_t *d = static_cast<uint8_t *>(p);
        while (bytes && ok) {
            if (pos == end) {
                end = std::fread(buf.data(), 1, buf.size(), f), pos = 0;
                if (end == 0) {
                    ok = false;
                    break;
                }
            }
            const size_t k = std::min(bytes, end - pos);
            std::memcpy(d, buf.data() + pos, k);
            pos += k, d += k, bytes -= k;
        }
    }
    template <class T> T scalar() {
        T v{};
        get(&v, sizeof(T));
        return v;
    }
    // a Vec of `width`-value elements into `a` (or skipped when a is NULL)
    template <class T> bool vec(T *a, uint64_t expect, int width) {
        const uint64_t n = scalar<uint64_t>();
        if (!ok || n != expect) return false;
        if (a) {
            get(a, (size_t)n * width * sizeof(T));
        } else {
            T tmp[9];
            for (uint64_t i = 0; i < n && ok; ++i) get(tmp, width * sizeof(T));
        }
        return ok;
    }
};

template <class T> void set(T *a, uint64_t i, T v) {
    if (a) a[i] = v;
}

bool has_arrays(const sv_frame &f) {
    return f.flags || f.mass || f.initial_volume || f.viscosity_dynamic || f.viscosity_bulk || f.mu || f.lambda ||
           f.sand_alpha || f.exponent || f.bulk_modulus || f.elastic_energies || f.collider_bits || f.positions ||
           f.position_gradients || f.velocities || f.velocity_gradients || f.initial_positions || f.node_ids ||
           f.node_collider_bits || f.node_masses || f.node_velocities;
}

// IoState::read: the header, then the bincode body.  With no arrays only
// the sizes are read (the particle Vecs are skipped to reach the grid's).
std::string read_frame_file(const char *path, const std::string &version, sv_frame &f) {
    Source r;
    r.f = std::fopen(path, "rb");
    if (!r.f) return std::string("frame file: cannot open ") + path;
    struct Closer {
        FILE *f;
        ~Closer() { std::fclose(f); }
    } closer{r.f};
    char magic[MAGIC_LEN], vb[VERSION_LEN];
    r.get(magic, MAGIC_LEN);
    if (!r.ok) return "frame file: failed to read the magic bytes";
    if (std::memcmp(magic, MAGIC, MAGIC_LEN) != 0) return "frame file: magic bytes mismatch";
    r.get(vb, VERSION_LEN);
    if (!r.ok) return "frame file: failed to read the version bytes";
    char want[VERSION_LEN] = {};
    if (version.size() > VERSION_LEN) return "frame file: version string longer than 64 bytes";
    std::memcpy(want, version.data(), version.size());
    if (std::memcmp(vb, want, VERSION_LEN) != 0) {
        const std::string found(vb, strnlen(vb, VERSION_LEN));
        return "frame file: version mismatch, found " + found + ", but expected " + version;
    }
    const bool fill = has_arrays(f);
    const uint64_t cap_n = f.n, cap_m = f.n_nodes;
    f.time = r.scalar<double>();
    const uint64_t n = r.scalar<uint64_t>();  // flags
    if (!r.ok) return "frame file: truncated";
    if (fill && n != cap_n) return "frame file: the particle count differs from the buffers'";
    std::vector<uint32_t> flags(n);
    r.get(flags.data(), n * 4);
    if (f.flags && r.ok) std::memcpy(f.flags, flags.data(), n * 4);
    if (r.scalar<uint64_t>() != n || !r.ok) return "frame file: particle arrays of different lengths";
    for (uint64_t i = 0; i < n && r.ok; ++i) {
        set(f.mass, i, r.scalar<float>());
        set(f.initial_volume, i, r.scalar<float>());
        float vd = 0.f, vbk = 0.f;
        const uint8_t visc = r.scalar<uint8_t>();
        if (visc == 1) vd = r.scalar<float>(), vbk = r.scalar<float>();
        else if (visc != 0) return "frame file: bad Option tag";
        set(f.viscosity_dynamic, i, vd);
        set(f.viscosity_bulk, i, vbk);
        const uint32_t variant = r.scalar<uint32_t>();
        float mu = 0.f, lambda = 0.f, alpha = 0.f, K = 0.f;
        int32_t gamma = 0;
        if (variant == 0) {
            mu = r.scalar<float>(), lambda = r.scalar<float>();
            const uint8_t sa = r.scalar<uint8_t>();
            if (sa == 1) alpha = r.scalar<float>();
            else if (sa != 0) return "frame file: bad Option tag";
        } else if (variant == 1) {
            gamma = r.scalar<int32_t>(), K = r.scalar<float>();
        } else {
            return "frame file: bad enum variant";
        }
        set(f.mu, i, mu), set(f.lambda, i, lambda), set(f.sand_alpha, i, alpha);
        set(f.exponent, i, gamma), set(f.bulk_modulus, i, K);
    }
    if (!r.vec(f.elastic_energies, n, 1) || !r.vec(f.collider_bits, n, 1) || !r.vec(f.positions, n, 3) ||
        !r.vec(f.position_gradients, n, 9) || !r.vec(f.velocities, n, 3) || !r.vec(f.velocity_gradients, n, 9) ||
        !r.vec(f.initial_positions, n, 3))
        return "frame file: truncated or particle arrays of different lengths";
    const uint8_t grid = r.scalar<uint8_t>();
    if (!r.ok || grid > 1) return "frame file: truncated or bad grid tag";
    f.n = n;
    f.has_grid = grid;
    f.n_nodes = 0;
    if (grid) {
        const uint64_t m = r.scalar<uint64_t>();
        if (!r.ok) return "frame file: truncated";
        if (fill && m != cap_m) return "frame file: the grid node count differs from the buffers'";
        f.n_nodes = m;
        if (!fill) return "";
        std::vector<int32_t> ids(3 * m);
        r.get(ids.data(), m * 12);
        if (f.node_ids && r.ok) std::memcpy(f.node_ids, ids.data(), m * 12);
        if (!r.vec(f.node_collider_bits, m, 1) || !r.vec(f.node_masses, m, 1) || !r.vec(f.node_velocities, m, 3))
            return "frame file: truncated or grid arrays of different lengths";
    }
    return "";
}

// ------------------------------------------------------------------ the cache
// Host copy of a frame's arrays (the statics, or a queued host frame).
struct FrameData {
    double time = 0.0;
    uint64_t n = 0, m = 0;
    bool has_grid = false;
    std::vector<uint32_t> flags, collider_bits, node_bits;
    std::vector<float> mass, V0, visc_d, visc_b, mu, lambda, alpha, K, energy, x, F, v, C, x0, node_m, node_v;
    std::vector<int32_t> gamma, node_ids;
};

template <class T> std::vector<T> copy_of(const T *a, uint64_t count) {
    return a ? std::vector<T>(a, a + count) : std::vector<T>();
}
template <class T> T *ptr_or_null(std::vector<T> &v) { return v.empty() ? nullptr : v.data(); }

FrameData copy_frame(const sv_frame &f) {
    FrameData d;
    d.time = f.time, d.n = f.n, d.has_grid = f.has_grid != 0, d.m = f.has_grid ? f.n_nodes : 0;
    const uint64_t n = f.n, m = d.m;
    d.flags = copy_of(f.flags, n), d.mass = copy_of(f.mass, n), d.V0 = copy_of(f.initial_volume, n);
    d.visc_d = copy_of(f.viscosity_dynamic, n), d.visc_b = copy_of(f.viscosity_bulk, n);
    d.mu = copy_of(f.mu, n), d.lambda = copy_of(f.lambda, n), d.alpha = copy_of(f.sand_alpha, n);
    d.gamma = copy_of(f.exponent, n), d.K = copy_of(f.bulk_modulus, n);
    d.energy = copy_of(f.elastic_energies, n), d.collider_bits = copy_of(f.collider_bits, n);
    d.x = copy_of(f.positions, 3 * n), d.F = copy_of(f.position_gradients, 9 * n);
    d.v = copy_of(f.velocities, 3 * n), d.C = copy_of(f.velocity_gradients, 9 * n);
    d.x0 = copy_of(f.initial_positions, 3 * n);
    d.node_ids = copy_of(f.node_ids, 3 * m), d.node_bits = copy_of(f.node_collider_bits, m);
    d.node_m = copy_of(f.node_masses, m), d.node_v = copy_of(f.node_velocities, 3 * m);
    return d;
}

sv_frame view_of(FrameData &d) {
    sv_frame f{};
    f.time = d.time, f.n = d.n;
    f.flags = ptr_or_null(d.flags), f.mass = ptr_or_null(d.mass), f.initial_volume = ptr_or_null(d.V0);
    f.viscosity_dynamic = ptr_or_null(d.visc_d), f.viscosity_bulk = ptr_or_null(d.visc_b);
    f.mu = ptr_or_null(d.mu), f.lambda = ptr_or_null(d.lambda), f.sand_alpha = ptr_or_null(d.alpha);
    f.exponent = ptr_or_null(d.gamma), f.bulk_modulus = ptr_or_null(d.K);
    f.elastic_energies = ptr_or_null(d.energy), f.collider_bits = ptr_or_null(d.collider_bits);
    f.positions = ptr_or_null(d.x), f.position_gradients = ptr_or_null(d.F);
    f.velocities = ptr_or_null(d.v), f.velocity_gradients = ptr_or_null(d.C);
    f.initial_positions = ptr_or_null(d.x0);
    f.has_grid = d.has_grid, f.n_nodes = d.m;
    f.node_ids = ptr_or_null(d.node_ids), f.node_collider_bits = ptr_or_null(d.node_bits);
    f.node_masses = ptr_or_null(d.node_m), f.node_velocities = ptr_or_null(d.node_v);
    return f;
}

// One set of state buffers of a frame in flight: pinned host or device memory.
struct Buffers {
    bool device = false;
    uint64_t n_cap = 0, slots_cap = 0, var_cap_cap = 0;
    bool has_cell = false, has_cbits = false;
    HostParticles p;
    HostGrid g;

    template <class T> cudaError_t alloc(T **ptr, uint64_t count) {
        const size_t bytes = std::max<size_t>((size_t)count * sizeof(T), 16);
        return device ? cudaMalloc((void **)ptr, bytes) : cudaHostAlloc((void **)ptr, bytes, cudaHostAllocDefault);
    }
    void drop(void *ptr) {
        if (!ptr) return;
        if (device) cudaFree(ptr);
        else cudaFreeHost(ptr);
    }
    void free_particles() {
        for (void *q : {(void *)p.pos, (void *)p.vel, (void *)p.cell, (void *)p.C, (void *)p.F, (void *)p.energy,
                        (void *)p.orig, (void *)p.cbits})
            drop(q);
        p = HostParticles{};
        n_cap = 0, has_cell = has_cbits = false;
    }
    void release() {
        free_particles();
        for (void *q : {(void *)g.active, (void *)g.grid, (void *)g.var_key, (void *)g.var_bits, (void *)g.var_vel}) drop(q);
        g = HostGrid{};
        slots_cap = var_cap_cap = 0;
    }
    cudaError_t ensure(uint64_t n, bool cell, bool cbits, uint64_t slots, uint64_t var_cap) {
        cudaError_t e = cudaSuccess;
        if (n > n_cap || (cell && !has_cell) || (cbits && !has_cbits)) {
            const uint64_t c = std::max(n, n_cap);
            const bool want_cell = cell || has_cell, want_cbits = cbits || has_cbits;
            free_particles();
            if ((e = alloc(&p.pos, c)) || (e = alloc(&p.vel, c)) || (e = alloc(&p.C, 9 * c)) || (e = alloc(&p.F, 9 * c)) ||
                (e = alloc(&p.energy, c)) || (e = alloc(&p.orig, c)) || (want_cell && (e = alloc(&p.cell, c))) ||
                (want_cbits && (e = alloc(&p.cbits, c))))
                return e;
            n_cap = c, has_cell = want_cell, has_cbits = want_cbits;
        }
        if (slots > slots_cap) {
            drop(g.active), drop(g.grid);
            g.active = nullptr, g.grid = nullptr;
            if ((e = alloc(&g.active, slots)) || (e = alloc(&g.grid, slots * 64))) return e;
            slots_cap = slots;
        }
        if (var_cap > var_cap_cap) {
            drop(g.var_key), drop(g.var_bits), drop(g.var_vel);
            g.var_key = nullptr, g.var_bits = nullptr, g.var_vel = nullptr;
            if ((e = alloc(&g.var_key, var_cap)) || (e = alloc(&g.var_bits, var_cap * col::VK)) ||
                (e = alloc(&g.var_vel, var_cap * col::VK)))
                return e;
            var_cap_cap = var_cap;
        }
        return cudaSuccess;
    }
    // views sized for one frame (cell and cbits only where the state has them)
    HostParticles particles(uint64_t n, bool cell, bool cbits) const {
        HostParticles v = p;
        v.n = n;
        if (!cell) v.cell = nullptr;
        if (!cbits) v.cbits = nullptr;
        return v;
    }
    HostGrid grid(uint64_t slots, uint64_t var_cap) const {
        HostGrid v = g;
        v.slots = slots, v.var_cap = var_cap;
        return v;
    }
};

// A frame in flight from a handle: a device snapshot taken on the handle's
// stream (`snap`), and its copy to pinned memory on the cache's own stream
// (`copied`), which overlaps the handle's next substeps.
struct Slot {
    cudaEvent_t snap = nullptr, copied = nullptr;
    Buffers dev{true}, host{false};
    cudaError_t ensure(uint64_t n, bool cell, bool cbits, uint64_t slots, uint64_t var_cap) {
        cudaError_t e;
        if (!snap && (e = cudaEventCreateWithFlags(&snap, cudaEventDisableTiming))) return e;
        if (!copied && (e = cudaEventCreateWithFlags(&copied, cudaEventDisableTiming | cudaEventBlockingSync))) return e;
        if ((e = dev.ensure(n, cell, cbits, slots, var_cap))) return e;
        return host.ensure(n, cell, cbits, slots, var_cap);
    }
    void release() {
        if (snap) cudaEventDestroy(snap);
        if (copied) cudaEventDestroy(copied);
        snap = copied = nullptr;
        dev.release(), host.release();
    }
};

struct Job {
    uint32_t frame = 0;
    int slot = -1;  // >= 0: a handle's copies in that slot; else `host`
    int device = 0;
    // handle jobs
    uint64_t n = 0;
    double time = 0.0;
    bool store_grid = false;
    UnpackInfo unpack;
    GridLayout layout{};
    HostParticles hp;
    HostGrid hg;
    // host jobs
    std::shared_ptr<FrameData> host;
};

}  // namespace

struct sv_cache {
    std::string dir, version;
    FrameData statics;
    uint32_t next_frame = 0;
    std::vector<Slot> slots;
    std::vector<bool> slot_busy;
    std::deque<Job> queue;
    std::mutex m;
    std::condition_variable cv;
    bool stop = false;
    bool busy = false;  // the writer holds a job
    std::string error;  // first failure of the writer
    std::atomic<uint64_t> frames{0}, bytes{0};
    std::thread worker;
    cudaStream_t copy_stream = nullptr;  // device snapshot -> pinned memory
    int stream_device = -1;

    // One frame: a handle's copies (unpacked here) or a host frame.
    std::string write(Job &j) {
        char name[32];
        std::snprintf(name, sizeof(name), "frame_%05u.bin", j.frame);
        const std::string path = dir + "/" + name;
        uint64_t written = 0;
        std::string err;
        if (j.slot < 0) {
            sv_frame f = view_of(*j.host);
            err = write_frame_file(path.c_str(), f, version, written);
        } else {
            // the slot goes back to sv_cache_store once its buffers are read
            struct Release {
                sv_cache *c;
                int k;
                bool done = false;
                void operator()() {
                    if (done) return;
                    done = true;
                    c->release_slot(k);
                }
                ~Release() { (*this)(); }
            } release{this, j.slot};
            cudaSetDevice(j.device);
            const cudaError_t e = cudaEventSynchronize(slots[j.slot].copied);
            if (e != cudaSuccess) return std::string("frame cache: copy failed: ") + cudaGetErrorString(e);
            FrameData d;
            const uint64_t n = j.n;
            d.time = j.time, d.n = n;
            d.flags.resize(n), d.energy.resize(n), d.collider_bits.resize(n);
            d.x.resize(3 * n), d.F.resize(9 * n), d.v.resize(3 * n), d.C.resize(9 * n);
            sv_particles o{};
            o.n = n;
            o.flags = d.flags.data(), o.positions = d.x.data(), o.position_gradients = d.F.data();
            o.velocities = d.v.data(), o.velocity_gradients = d.C.data(), o.elastic_energies = d.energy.data();
            o.collider_bits = d.collider_bits.data();
            if (!unpack_particles(j.hp, j.unpack, &o)) return "frame cache: corrupt original index";
            if (j.store_grid) {
                const std::vector<GridNode> nodes = grid_nodes(j.hg, j.layout);
                const uint64_t m = nodes.size();
                d.has_grid = true, d.m = m;
                d.node_ids.resize(3 * m), d.node_bits.resize(m), d.node_m.resize(m), d.node_v.resize(3 * m);
                for (uint64_t i = 0; i < m; ++i) {
                    std::memcpy(&d.node_ids[3 * i], nodes[i].id, 12);
                    d.node_bits[i] = nodes[i].bits;
                    d.node_m[i] = nodes[i].v.w;
                    d.node_v[3 * i] = nodes[i].v.x, d.node_v[3 * i + 1] = nodes[i].v.y, d.node_v[3 * i + 2] = nodes[i].v.z;
                }
            }
            release();  // the pinned buffers are free again
            sv_frame f = view_of(d);
            // what the substep never changes comes from the statics
            sv_frame s = view_of(statics);
            f.mass = s.mass, f.initial_volume = s.initial_volume, f.viscosity_dynamic = s.viscosity_dynamic;
            f.viscosity_bulk = s.viscosity_bulk, f.mu = s.mu, f.lambda = s.lambda, f.sand_alpha = s.sand_alpha;
            f.exponent = s.exponent, f.bulk_modulus = s.bulk_modulus, f.initial_positions = s.initial_positions;
            err = write_frame_file(path.c_str(), f, version, written);
        }
        if (err.empty()) bytes += written, frames += 1;
        return err;
    }

    void release_slot(int k) {
        {
            std::lock_guard<std::mutex> lk(m);
            slot_busy[k] = false;
        }
        cv.notify_all();
    }

    void run() {
        std::unique_lock<std::mutex> lk(m);
        while (true) {
            cv.wait(lk, [&] { return stop || !queue.empty(); });
            if (queue.empty()) break;  // stop requested and nothing left
            Job j = std::move(queue.front());
            queue.pop_front();
            busy = true;
            const bool failed = !error.empty();
            lk.unlock();
            std::string err;
            if (!failed) {
                err = write(j);  // releases a handle job's slot itself
            } else if (j.slot >= 0) {
                // after a failure the queue drains unwritten (StoreThread's
                // loop ends at its first error); its copies still finish
                cudaSetDevice(j.device);
                cudaEventSynchronize(slots[j.slot].copied);
                release_slot(j.slot);
            }
            lk.lock();
            if (!err.empty() && error.empty()) error = err;
            busy = false;
            cv.notify_all();
        }
    }
};

namespace {

int writer_error(sv_cache *c) {
    std::lock_guard<std::mutex> lk(c->m);
    if (c->error.empty()) return 0;
    return cfail(c->error);
}

}  // namespace

extern "C" {

int sv_frame_write(const char *path, const sv_frame *frame, const char *version, uint64_t *bytes_written) {
    if (!path || !frame) return cfail("sv_frame_write: NULL argument");
    uint64_t bytes = 0;
    const std::string err = write_frame_file(path, *frame, version_or_default(version), bytes);
    if (!err.empty()) return cfail(err);
    if (bytes_written) *bytes_written = bytes;
    return 0;
}

int sv_frame_read(const char *path, const char *version, sv_frame *frame) {
    if (!path || !frame) return cfail("sv_frame_read: NULL argument");
    const std::string err = read_frame_file(path, version_or_default(version), *frame);
    if (!err.empty()) return cfail(err);
    return 0;
}

int sv_cache_open(const char *dir, const char *version, const sv_frame *statics, uint32_t first_frame, uint32_t depth,
                  sv_cache **out) {
    if (!dir || !statics || !out) return cfail("sv_cache_open: NULL argument");
    *out = nullptr;
    const std::string v = version_or_default(version);
    if (v.size() > VERSION_LEN) return cfail("sv_cache_open: version string longer than 64 bytes");
    auto *c = new sv_cache;
    c->dir = dir, c->version = v, c->next_frame = first_frame;
    c->statics = copy_frame(*statics);
    c->statics.has_grid = false, c->statics.m = 0;
    const uint32_t d = depth ? depth : 2;
    c->slots.resize(d);  // their events and buffers come with the first store from a handle
    c->slot_busy.assign(d, false);
    c->worker = std::thread([c] { c->run(); });
    *out = c;
    return 0;
}

int sv_cache_store(sv_cache *c, sv_handle *h, int store_grid) {
    if (!c || !h) return cfail("sv_cache_store: NULL argument");
    if (writer_error(c)) return -1;
    if (h->n != c->statics.n) return cfail("sv_cache_store: the handle's particle count differs from the statics'");
    if (refresh_counters(h)) return -1;
    uint64_t slots = 0, var_cap = 0;
    if (store_grid) grid_sizes(h, slots, var_cap);
    int k = -1;
    {
        // a free slot: the oldest frame in flight has left its buffers
        std::unique_lock<std::mutex> lk(c->m);
        c->cv.wait(lk, [&] {
            for (size_t i = 0; i < c->slots.size(); ++i)
                if (!c->slot_busy[i]) return true;
            return !c->error.empty();
        });
        if (!c->error.empty()) return cfail(c->error);
        for (size_t i = 0; i < c->slots.size(); ++i)
            if (!c->slot_busy[i]) {
                k = (int)i;
                break;
            }
        c->slot_busy[k] = true;
    }
    Slot &s = c->slots[k];
    const bool cell = h->layout.position_form == 1, cbits = h->side[h->cur].cbits_done != nullptr;
    Job j;
    cudaGetDevice(&j.device);
    cudaError_t e = cudaSuccess;
    if (!c->copy_stream) {
        e = cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
        c->stream_device = j.device;
    }
    if (e == cudaSuccess && j.device != c->stream_device) e = cudaErrorInvalidDevice;  // one device per cache
    if (e == cudaSuccess) e = s.ensure(h->n, cell, cbits, slots, var_cap);
    if (e == cudaSuccess) {
        j.slot = k, j.n = h->n, j.time = h->time, j.store_grid = store_grid != 0;
        j.unpack = unpack_info(h, true);
        j.layout = h->layout;
        j.hp = s.host.particles(h->n, cell, cbits);
        j.hg = s.host.grid(slots, var_cap);
        const HostParticles dp = s.dev.particles(h->n, cell, cbits);
        const HostGrid dg = s.dev.grid(slots, var_cap);
        // device snapshot on the handle's stream, so its next substeps only
        // wait for a copy at HBM speed; the host copy runs on the cache's stream
        if ((e = copy_particles(dp, device_view(h), h->stream)) == cudaSuccess &&
            (!store_grid || (e = copy_grid(dg, device_grid_view(h, slots, var_cap), h->stream)) == cudaSuccess) &&
            (e = cudaEventRecord(s.snap, h->stream)) == cudaSuccess &&
            (e = cudaStreamWaitEvent(c->copy_stream, s.snap, 0)) == cudaSuccess &&
            (e = copy_particles(j.hp, dp, c->copy_stream)) == cudaSuccess &&
            (!store_grid || (e = copy_grid(j.hg, dg, c->copy_stream)) == cudaSuccess))
            e = cudaEventRecord(s.copied, c->copy_stream);
    }
    if (e != cudaSuccess) {
        std::lock_guard<std::mutex> lk(c->m);
        c->slot_busy[k] = false;
        return cfail(std::string("sv_cache_store: ") + cudaGetErrorString(e));
    }
    {
        std::lock_guard<std::mutex> lk(c->m);
        j.frame = c->next_frame++;
        c->queue.push_back(std::move(j));
    }
    c->cv.notify_all();
    return 0;
}

int sv_cache_store_frame(sv_cache *c, const sv_frame *frame) {
    if (!c || !frame) return cfail("sv_cache_store_frame: NULL argument");
    if (writer_error(c)) return -1;
    Job j;
    j.host = std::make_shared<FrameData>(copy_frame(*frame));
    {
        std::lock_guard<std::mutex> lk(c->m);
        j.frame = c->next_frame++;
        c->queue.push_back(std::move(j));
    }
    c->cv.notify_all();
    return 0;
}

int sv_cache_check(sv_cache *c) {
    if (!c) return cfail("sv_cache_check: NULL cache");
    return writer_error(c);
}

int sv_cache_flush(sv_cache *c) {
    if (!c) return cfail("sv_cache_flush: NULL cache");
    {
        std::unique_lock<std::mutex> lk(c->m);
        c->cv.wait(lk, [&] { return (c->queue.empty() && !c->busy) || !c->error.empty(); });
    }
    return writer_error(c);
}

int sv_cache_info(sv_cache *c, uint64_t *frames_written, uint64_t *bytes_written) {
    if (!c) return cfail("sv_cache_info: NULL cache");
    if (frames_written) *frames_written = c->frames.load();
    if (bytes_written) *bytes_written = c->bytes.load();
    return 0;
}

int sv_cache_close(sv_cache *c) {
    if (!c) return 0;
    {
        std::lock_guard<std::mutex> lk(c->m);
        c->stop = true;
    }
    c->cv.notify_all();
    if (c->worker.joinable()) c->worker.join();
    const int rc = writer_error(c);
    for (Slot &s : c->slots) s.release();
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    delete c;
    return rc;
}

}  // extern "C"
