// sv_transfer.cu -- particle state to and from the caller's host arrays by
// kernels that access pageable host memory directly.
//
// On a Grace host (NVLink-C2C, address translation through the host page
// tables: cudaDevAttrPageableMemoryAccess) the GPU reads and writes ordinary
// malloc'd memory coherently.  The upload then is one kernel that reads the
// caller's arrays (file_frame's [n][3] / [n][9] layouts) and writes the
// device layout -- packing flags with the material index, converting to the
// cell + offset form, transposing the matrices into element planes -- instead
// of a single-threaded host staging loop and pageable copies.  The download
// inverts the binning permutation on the device and writes the caller's
// arrays in the original particle order (the reference's reverse_sort_map
// restore, cpu_state.rs:71-104) with coalesced stores.  Both give the same
// bits as the staged path in sv_api.cu / sv_cache.cu, which remains for
// devices without pageable-memory access.
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "sv_internal.h"

namespace sv {
namespace {

constexpr int TPB = 256;

// The caller's arrays of one scene, copied to device memory once per
// upload so that no thread chases pointers through host memory.
struct UploadScene {
    const uint32_t *flags;
    const float *positions, *velocities, *position_gradients, *velocity_gradients;
    const float *elastic_energies, *plastic_j;  // may be NULL
    uint64_t first;                              // first particle of the scene
};

struct UploadArgs {
    const UploadScene *sc;       // device: one per scene, plus a sentinel whose first is n
    uint32_t n_scenes;
    const uint32_t *mat_index;   // host: material of each particle
    const SceneInfo *scenes;     // device
    ParticleArrays a;            // device, side 0
    uint64_t n;
    double dx;
};

__device__ __forceinline__ uint32_t scene_of(const UploadScene *sc, uint32_t n_scenes, uint64_t i) {
    uint32_t lo = 0, hi = n_scenes;  // sc[lo].first <= i < sc[hi].first
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (sc[mid].first <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// One particle of the upload: its position, velocity and matrix rows already
// in shared memory, its per-particle scalars in registers.
template <bool CELL>
__device__ __forceinline__ void upload_one(const UploadArgs &u, uint64_t i, uint32_t sc, uint32_t flags, uint32_t mi,
                                           float plastic_j, float energy, const float *rx, const float *rv,
                                           const float *rF, const float *rC) {
    const uint32_t packed = (flags & FLAG_MASK) | (mi << MATERIAL_SHIFT);
    const float x = rx[0], y = rx[1], z = rx[2];
    float4 pos;
    if (!CELL) {
        pos = make_float4(x, y, z, 0.f);
    } else {
        const double q[3] = {(double)x / u.dx, (double)y / u.dx, (double)z / u.dx};
        int ci[3];
        float o[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double f = floor(q[a]);
            ci[a] = (int)f + u.scenes[sc].off[a];
            o[a] = (float)(q[a] - f);
            if (o[a] >= 1.f) o[a] = 0.f, ci[a] += 1;
        }
        pos = make_float4(o[0], o[1], o[2], 0.f);
        u.a.cell[i] = make_int4(ci[0], ci[1], ci[2], 0);
    }
    pos.w = __uint_as_float(packed);
    u.a.pos[i] = pos;
    u.a.vel[i] = make_float4(rv[0], rv[1], rv[2], plastic_j);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        u.a.C[(uint64_t)k * u.n + i] = rC[k];
        u.a.F[(uint64_t)k * u.n + i] = rF[k];
    }
    u.a.energy[i] = energy;
    u.a.orig[i] = (uint32_t)i;
}

// Rows of W floats of a tile (src rows li0 ...): element e = threadIdx.x +
// k * TPB of the tile's count * W words, consecutive threads on consecutive
// words.  All loads of a tile are issued before any store to shared memory,
// so each thread has them in flight together across the host link.
template <int W> struct Rows {
    float r[W];
    __device__ __forceinline__ void load(const float *src, uint64_t li0, int count) {
        const float *in = src + li0 * W;
#pragma unroll
        for (int k = 0; k < W; ++k) {
            const int e = threadIdx.x + k * TPB;
            r[k] = e < count * W ? in[e] : 0.f;
        }
    }
    __device__ __forceinline__ void store(float *stage, int count) const {
#pragma unroll
        for (int k = 0; k < W; ++k) {
            const int e = threadIdx.x + k * TPB;
            if (e < count * W) stage[e] = r[k];
        }
    }
};

// The staged upload's per-particle conversion (sv_api.cu create_impl),
// reading the caller's arrays directly: over tiles of TPB particles, whose
// [n][3] and [n][9] rows arrive through shared memory with coalesced loads.
template <bool CELL> __global__ void __launch_bounds__(TPB) k_upload(UploadArgs u) {
    __shared__ float sx[TPB * 3], sv[TPB * 3], sF[TPB * 9], sC[TPB * 9];
    for (uint64_t i0 = (uint64_t)blockIdx.x * TPB; i0 < u.n; i0 += (uint64_t)gridDim.x * TPB) {
        const int count = (int)(u.n - i0 < (uint64_t)TPB ? u.n - i0 : (uint64_t)TPB);
        const int t = threadIdx.x;
        const uint64_t i = i0 + t;
        const uint32_t s0 = scene_of(u.sc, u.n_scenes, i0), s1 = scene_of(u.sc, u.n_scenes, i0 + count - 1);
        // this thread's particle: its scene and scalars
        const uint32_t sc = s0 == s1 ? s0 : (t < count ? scene_of(u.sc, u.n_scenes, i) : s0);
        const UploadScene p = u.sc[sc];
        const uint64_t li = i - p.first;
        uint32_t flags = 0, mi = 0;
        float pj = 1.f, en = 0.f;
        if (t < count) {
            flags = p.flags[li], mi = u.mat_index[i];
            if (p.plastic_j) pj = p.plastic_j[li];
            if (p.elastic_energies) en = p.elastic_energies[li];
        }
        if (s0 == s1) {
            const uint64_t li0 = i0 - p.first;
            Rows<3> x, v;
            Rows<9> F, C;
            x.load(p.positions, li0, count), v.load(p.velocities, li0, count);
            F.load(p.position_gradients, li0, count), C.load(p.velocity_gradients, li0, count);
            x.store(sx, count), v.store(sv, count), F.store(sF, count), C.store(sC, count);
        } else if (t < count) {
            // a tile across scenes: each thread its own rows
#pragma unroll
            for (int k = 0; k < 3; ++k) sx[3 * t + k] = p.positions[3 * li + k], sv[3 * t + k] = p.velocities[3 * li + k];
#pragma unroll
            for (int k = 0; k < 9; ++k)
                sF[9 * t + k] = p.position_gradients[9 * li + k], sC[9 * t + k] = p.velocity_gradients[9 * li + k];
        }
        __syncthreads();
        if (t < count) upload_one<CELL>(u, i, sc, flags, mi, pj, en, sx + 3 * t, sv + 3 * t, sF + 9 * t, sC + 9 * t);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(TPB) k_invert(const uint32_t *orig, uint32_t *inv, uint64_t n, uint32_t *bad) {
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = orig[s];
        if (i >= n || atomicExch(&inv[i], (uint32_t)s) != 0xFFFFFFFFu) atomicOr(bad, 1u);
    }
}

struct DownloadArgs {
    ParticleArrays a;          // device, the current side
    const uint32_t *inv;       // device: slot of each original particle
    const Material *mats;      // device
    const SceneInfo *scenes;   // device
    const uint32_t *bits0;     // host: collider bits the particles were created with (no frame input)
    bool stepped;
    sv_particles o;            // host arrays (NULL ones are skipped) of particles first .. first + count
    uint64_t first, count;
    uint64_t n;
    uint32_t n_materials;
    double dx;
};

// Writes a tile's rows of `width` floats, staged in shared memory, to
// dst[i0 * width ...] with consecutive threads on consecutive words, so that
// every host-memory transaction covers whole cache lines.
__device__ __forceinline__ void flush_rows(float *dst, const float *stage, uint64_t i0, int count, int width) {
    float *out = dst + i0 * width;
    for (int e = threadIdx.x; e < count * width; e += TPB) out[e] = stage[e];
}

// unpack_particles (sv_cache.cu) over tiles of TPB particles in original
// order: each thread gathers its particle from the device state, the tile's
// [n][3] and [n][9] rows are staged in shared memory and leave coalesced.
template <bool CELL> __global__ void __launch_bounds__(TPB) k_download(DownloadArgs d) {
    __shared__ float sx[TPB * 3], sv[TPB * 3], sF[TPB * 9], sC[TPB * 9];
    const sv_particles &o = d.o;
    for (uint64_t i0 = (uint64_t)blockIdx.x * TPB; i0 < d.count; i0 += (uint64_t)gridDim.x * TPB) {
        const int count = (int)(d.count - i0 < (uint64_t)TPB ? d.count - i0 : (uint64_t)TPB);
        const int t = threadIdx.x;
        const uint64_t i = i0 + t;  // in the caller's arrays; original particle d.first + i
        const uint64_t s = t < count ? d.inv[d.first + i] : d.n;
        if (s < d.n) {  // else unset (reported through the flag of k_invert) or past the end
            const float4 p = d.a.pos[s], v = d.a.vel[s];
            const uint32_t packed = __float_as_uint(p.w);
            if (o.flags) o.flags[i] = packed & FLAG_MASK;
            float x = p.x, y = p.y, z = p.z;
            if (CELL) {
                // back to the scene's own coordinates
                const uint32_t mi = packed >> MATERIAL_SHIFT;
                const SceneInfo &sc = d.scenes[mi < d.n_materials ? d.mats[mi].scene : 0];
                const int4 c = d.a.cell[s];
                x = (float)(((double)(c.x - sc.off[0]) + p.x) * d.dx);
                y = (float)(((double)(c.y - sc.off[1]) + p.y) * d.dx);
                z = (float)(((double)(c.z - sc.off[2]) + p.z) * d.dx);
            }
            sx[3 * t] = x, sx[3 * t + 1] = y, sx[3 * t + 2] = z;
            sv[3 * t] = v.x, sv[3 * t + 1] = v.y, sv[3 * t + 2] = v.z;
            if (o.plastic_j) o.plastic_j[i] = v.w;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                sF[9 * t + k] = d.a.F[(uint64_t)k * d.n + s];
                sC[9 * t + k] = d.a.C[(uint64_t)k * d.n + s];
            }
            if (o.elastic_energies) o.elastic_energies[i] = d.a.energy[s];
            if (o.collider_bits) {
                // without colliders every substep's Collide clears a live
                // particle's bits (collide.rs:53-56)
                if (d.a.cbits_done) o.collider_bits[i] = d.a.cbits_done[s];
                else o.collider_bits[i] = (d.stepped && !(packed & SV_TOMBSTONED)) ? 0u : (d.bits0 ? d.bits0[d.first + i] : 0u);
            }
        } else if (t < count) {
            // an unset row keeps what the caller's array held
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                sx[3 * t + k] = o.positions ? o.positions[3 * i + k] : 0.f;
                sv[3 * t + k] = o.velocities ? o.velocities[3 * i + k] : 0.f;
            }
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                sF[9 * t + k] = o.position_gradients ? o.position_gradients[9 * i + k] : 0.f;
                sC[9 * t + k] = o.velocity_gradients ? o.velocity_gradients[9 * i + k] : 0.f;
            }
        }
        __syncthreads();
        if (o.positions) flush_rows(o.positions, sx, i0, count, 3);
        if (o.velocities) flush_rows(o.velocities, sv, i0, count, 3);
        if (o.position_gradients) flush_rows(o.position_gradients, sF, i0, count, 9);
        if (o.velocity_gradients) flush_rows(o.velocity_gradients, sC, i0, count, 9);
        __syncthreads();
    }
}

// Populates the pages of the caller's output arrays from host threads (one
// read-and-write of the same byte per page, so the contents stay).  A page
// the GPU touches first is populated through a device-side fault serviced
// by the host, tens of microseconds each; freshly allocated arrays (numpy's
// zeros map pages lazily) would otherwise cost more than the copy itself.
// True when every page of the range is mapped (mincore); arrays the caller
// reuses, or that produce_next_state prepared while the substeps ran, need
// no second pass, whose thread start-up alone is about 0.3 ms.  A page that
// is mapped but still read-only (never written) only costs the GPU a fault.
bool all_resident(const std::pair<void *, size_t> &a, size_t page) {
    const uintptr_t b0 = (uintptr_t)a.first / page * page;
    const uintptr_t b1 = ((uintptr_t)a.first + a.second + page - 1) / page * page;
    std::vector<unsigned char> v((b1 - b0) / page);
    if (v.empty()) return true;
    if (mincore((void *)b0, b1 - b0, v.data()) != 0) return false;
    for (unsigned char c : v)
        if (!(c & 1)) return false;
    return true;
}

void populate(const std::vector<std::pair<void *, size_t>> &all) {
    const size_t page = (size_t)std::max(4096L, sysconf(_SC_PAGESIZE));
    std::vector<std::pair<void *, size_t>> arrays;
    for (const auto &a : all)
        if (!all_resident(a, page)) arrays.push_back(a);
    if (arrays.empty()) return;
    size_t total = 0;
    for (const auto &a : arrays) total += a.second;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned T = (unsigned)std::max<size_t>(1, std::min<size_t>(std::min(hw, 16u), total / (8u << 20)));
    auto work = [&](unsigned t) {
        for (const auto &a : arrays) {
            const uintptr_t b0 = (uintptr_t)a.first / page * page;
            const uintptr_t b1 = ((uintptr_t)a.first + a.second + page - 1) / page * page;
            const size_t pages = (b1 - b0) / page;
            const uintptr_t c0 = b0 + pages * t / T * page, c1 = b0 + pages * (t + 1) / T * page;
            if (c1 <= c0) continue;
            // one call populates the range writable (Linux 5.14+); else touch each page
            if (madvise((void *)c0, c1 - c0, MADV_POPULATE_WRITE) == 0) continue;
            for (uintptr_t q = std::max<uintptr_t>(c0, (uintptr_t)a.first); q < c1 && q < (uintptr_t)a.first + a.second;
                 q = (q / page + 1) * page) {
                volatile uint8_t *p = reinterpret_cast<volatile uint8_t *>(q);
                *p = *p;
            }
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < T; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
}

unsigned blocks_for(uint64_t n) {
    const uint64_t b = (n + TPB - 1) / TPB;
    const uint64_t cap = (uint64_t)sm_count() * 8;
    return (unsigned)std::max<uint64_t>(1, std::min(b, cap));
}

}  // namespace

bool pageable_access() {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
    return v == 1;
}

cudaError_t upload_direct(sv_handle *h, const sv_particles *ps, uint32_t n_scenes, const uint64_t *first,
                          const uint32_t *mat_index) {
    if (h->n == 0) return cudaSuccess;
    std::vector<UploadScene> table(n_scenes + 1);
    for (uint32_t s = 0; s <= n_scenes; ++s) {
        UploadScene &t = table[s];
        t = UploadScene{};
        t.first = first[s];
        if (s == n_scenes) break;
        t.flags = ps[s].flags, t.positions = ps[s].positions, t.velocities = ps[s].velocities;
        t.position_gradients = ps[s].position_gradients, t.velocity_gradients = ps[s].velocity_gradients;
        t.elastic_energies = ps[s].elastic_energies, t.plastic_j = ps[s].plastic_j;
    }
    UploadScene *dtable = nullptr;
    const size_t bytes = table.size() * sizeof(UploadScene);
    cudaError_t e = cudaMallocAsync((void **)&dtable, bytes, h->stream);
    if (e != cudaSuccess) return e;
    UploadArgs u;
    u.sc = dtable, u.n_scenes = n_scenes, u.mat_index = mat_index;
    u.scenes = h->scenes, u.a = h->side[0], u.n = h->n, u.dx = h->layout.dx;
    if ((e = cudaMemcpyAsync(dtable, table.data(), bytes, cudaMemcpyHostToDevice, h->stream)) == cudaSuccess) {
        if (h->layout.position_form == 1) k_upload<true><<<blocks_for(h->n), TPB, 0, h->stream>>>(u);
        else k_upload<false><<<blocks_for(h->n), TPB, 0, h->stream>>>(u);
        h->launches += 1;
        e = cudaGetLastError();
    }
    const cudaError_t ef = cudaFreeAsync(dtable, h->stream);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);  // the caller's arrays may go away
    return e;
}

int download_direct(sv_handle *h, sv_particles *o, uint64_t first, uint64_t count) {
    const uint64_t n = h->n;
    if (n == 0 || count == 0) return 0;
    cudaError_t e;
    uint32_t *bad = h->counters + C_TRANSFER_BAD;  // an original index out of range or repeated
    DownloadArgs d;
    d.a = h->side[h->cur], d.inv = h->inv, d.mats = h->materials, d.scenes = h->scenes;
    d.bits0 = h->collider_bits.empty() ? nullptr : h->collider_bits.data();
    d.stepped = h->substeps_total > 0;
    d.o = *o, d.first = first, d.count = count, d.n = n, d.n_materials = h->n_materials, d.dx = h->layout.dx;
    // unset entries (a corrupt state) stay 0xFFFFFFFF and are skipped
    if ((e = cudaMemsetAsync(bad, 0, 4, h->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(h->inv, 0xFF, n * 4, h->stream)) != cudaSuccess) {
        set_last_error(std::string("sv_download: ") + cudaGetErrorString(e));
        return -1;
    }
    k_invert<<<blocks_for(n), TPB, 0, h->stream>>>(h->side[h->cur].orig, h->inv, n, bad);
    {
        std::vector<std::pair<void *, size_t>> out;
        auto add = [&](void *p, size_t bytes) {
            if (p) out.push_back({p, bytes});
        };
        add(o->flags, count * 4), add(o->positions, count * 12), add(o->position_gradients, count * 36);
        add(o->velocities, count * 12), add(o->velocity_gradients, count * 36), add(o->elastic_energies, count * 4);
        add(o->collider_bits, count * 4), add(o->plastic_j, count * 4);
        populate(out);  // overlaps k_invert
    }
    if (h->layout.position_form == 1) k_download<true><<<blocks_for(count), TPB, 0, h->stream>>>(d);
    else k_download<false><<<blocks_for(count), TPB, 0, h->stream>>>(d);
    h->launches += 2;
    uint32_t flag = 0;
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(&flag, bad, 4, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) {
        set_last_error(std::string("sv_download: ") + cudaGetErrorString(e));
        return -1;
    }
    if (flag) {
        set_last_error("sv_download: corrupt original index");
        return -1;
    }
    return 0;
}

}  // namespace sv

extern "C" int sv_prepare_host(void *const *arrays, const uint64_t *bytes, uint32_t count) {
    if (count && (!arrays || !bytes)) {
        sv::set_last_error("sv_prepare_host: NULL argument");
        return -1;
    }
    std::vector<std::pair<void *, size_t>> list;
    for (uint32_t k = 0; k < count; ++k)
        if (arrays[k] && bytes[k]) list.push_back({arrays[k], (size_t)bytes[k]});
    sv::populate(list);
    return 0;
}
