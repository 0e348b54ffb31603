// sv_sort.cu -- stable LSD radix sort and exclusive scan, written for
// sm_103a: digits of up to 10 bits, split evenly over the fewest passes
// (25-bit binning keys take three passes of 9, 8 and 8 bits, not four),
// per-tile histograms scanned digit-major, and a stable scatter whose
// in-tile ranks come from __match_any_sync peer groups processed row by row
// (so equal digits keep input order).
#include "sv_sort.cuh"

#include <cstring>
#include <mutex>

namespace sv {

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

constexpr int SORT_WARPS = 8;
constexpr int SORT_THREADS = SORT_WARPS * 32;
constexpr int SORT_ITEMS = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;
constexpr int MAX_DIGIT_BITS = 10;
constexpr int MAX_RADIX = 1 << MAX_DIGIT_BITS;

// Digit width of each pass for a key of `key_bits` bits: the fewest passes
// of at most MAX_DIGIT_BITS bits, as even as possible.
inline int sort_passes(int key_bits) { return (key_bits + MAX_DIGIT_BITS - 1) / MAX_DIGIT_BITS; }
inline int pass_bits(int key_bits, int pass) {
    const int passes = sort_passes(key_bits);
    return key_bits / passes + (pass < key_bits % passes ? 1 : 0);
}

inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Block-wide exclusive scan of SCAN_ITEMS consecutive values per thread.
// Returns the block total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t (&v)[SCAN_ITEMS], uint32_t *warp_sums) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t local = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        uint32_t t = v[i];
        v[i] = local;
        local += t;
    }
    uint32_t inc = warp_inclusive_scan(local, lane);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = warp_sums[lane];
        uint32_t si = warp_inclusive_scan(s, lane);
        warp_sums[lane] = si - s;
        if (lane == 31) warp_sums[32] = si;
    }
    __syncthreads();
    uint32_t off = warp_sums[warp] + inc - local;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) v[i] += off;
    uint32_t total = warp_sums[32];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t *in, uint64_t n, uint32_t *sums) {
    __shared__ uint32_t red[32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i)
        if (base + i < n) s += in[base + i];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = red[lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) sums[blockIdx.x] = t;
    }
}

// Scans one SCAN_TILE per block and adds the block's offset (offsets may be
// null for a single block).
__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan_tile(const uint32_t *in, uint32_t *out, uint64_t n, const uint32_t *offsets) {
    __shared__ uint32_t warp_sums[33];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) v[i] = base + i < n ? in[base + i] : 0u;
    block_exclusive_scan(v, warp_sums);
    uint32_t off = offsets ? offsets[blockIdx.x] : 0u;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i)
        if (base + i < n) out[base + i] = v[i] + off;
}

// Per-tile digit histogram, stored digit-major: hist[d * tiles + tile].
// RADIX is the shared table size, a power of two above `mask`.
template <int RADIX>
__global__ void __launch_bounds__(SORT_THREADS)
    k_radix_hist(const uint32_t *keys, uint64_t n, int shift, uint32_t mask, uint32_t *hist, uint32_t tiles) {
    __shared__ uint32_t h[RADIX];
    for (int i = threadIdx.x; i < RADIX; i += SORT_THREADS) h[i] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * SORT_TILE;
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint64_t e = base + (uint64_t)j * SORT_THREADS + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & mask], 1u);
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d <= mask; d += SORT_THREADS) hist[(uint64_t)d * tiles + blockIdx.x] = h[d];
}

// Stable scatter (vals_in == nullptr means "value = element index").  Warp w owns elements [w*32*ITEMS, (w+1)*32*ITEMS) of the
// tile; row j of lane l is element w*32*ITEMS + j*32 + l, so walking rows in
// order and lanes in order visits the warp's elements in input order.
template <int RADIX>
__global__ void __launch_bounds__(SORT_THREADS)
    k_radix_scatter(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out, uint32_t *vals_out,
                    uint64_t n, int shift, uint32_t mask, const uint32_t *scanned, uint32_t tiles) {
    __shared__ uint32_t wcnt[SORT_WARPS][RADIX];
    __shared__ uint32_t gbase[RADIX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&wcnt[0][0])[i] = 0;
    for (uint32_t d = threadIdx.x; d <= mask; d += SORT_THREADS) gbase[d] = scanned[(uint64_t)d * tiles + blockIdx.x];
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
    uint64_t base = (uint64_t)blockIdx.x * SORT_TILE + (uint64_t)warp * 32 * SORT_ITEMS + lane;
    uint32_t key[SORT_ITEMS], val[SORT_ITEMS], rank[SORT_ITEMS];
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint64_t e = base + (uint64_t)j * 32;
        bool valid = e < n;
        key[j] = valid ? keys_in[e] : 0u;
        val[j] = valid ? (vals_in ? vals_in[e] : (uint32_t)e) : 0u;
        uint32_t digit = valid ? (key[j] >> shift) & mask : 0xFFFFFFFFu;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        int leader = __ffs(peers) - 1;
        uint32_t before = 0;
        if (lane == leader && valid) {
            before = wcnt[warp][digit];
            wcnt[warp][digit] = before + __popc(peers);
        }
        before = __shfl_sync(0xffffffffu, before, leader);
        rank[j] = before + __popc(peers & lt);
        __syncwarp();
    }
    __syncthreads();
    for (uint32_t d = threadIdx.x; d <= mask; d += SORT_THREADS) {
        uint32_t run = gbase[d];
#pragma unroll
        for (int w = 0; w < SORT_WARPS; ++w) {
            uint32_t c = wcnt[w][d];
            wcnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SORT_ITEMS; ++j) {
        uint64_t e = base + (uint64_t)j * 32;
        if (e < n) {
            uint32_t digit = (key[j] >> shift) & mask;
            uint32_t dst = wcnt[warp][digit] + rank[j];
            keys_out[dst] = key[j];
            vals_out[dst] = val[j];
        }
    }
}

}  // namespace

size_t scan_temp_bytes(uint64_t n) {
    size_t total = 0;
    while (n > (uint64_t)SCAN_TILE) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        total += align_up(n * sizeof(uint32_t));
    }
    return total + 256;
}

cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, uint64_t n, void *temp, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (n <= (uint64_t)SCAN_TILE) {
        k_scan_tile<<<1, SCAN_THREADS, 0, stream>>>(in, out, n, nullptr);
        return cudaGetLastError();
    }
    uint64_t blocks = (n + SCAN_TILE - 1) / SCAN_TILE;
    uint32_t *sums = static_cast<uint32_t *>(temp);
    void *rest = static_cast<char *>(temp) + align_up(blocks * sizeof(uint32_t));
    k_scan_reduce<<<(unsigned)blocks, SCAN_THREADS, 0, stream>>>(in, n, sums);
    cudaError_t err = exclusive_scan_u32(sums, sums, blocks, rest, stream);
    if (err != cudaSuccess) return err;
    k_scan_tile<<<(unsigned)blocks, SCAN_THREADS, 0, stream>>>(in, out, n, sums);
    return cudaGetLastError();
}

int scan_launches(uint64_t n) {
    if (n == 0) return 0;
    if (n <= (uint64_t)SCAN_TILE) return 1;
    return 2 + scan_launches((n + SCAN_TILE - 1) / SCAN_TILE);
}

int radix_sort_launches(uint64_t n, int key_bits) {
    if (n == 0) return 0;
    if (key_bits <= 0) return 0;
    if (key_bits > 32) key_bits = 32;
    uint64_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    int total = 0;
    for (int p = 0; p < sort_passes(key_bits); ++p) total += 2 + scan_launches(((uint64_t)1 << pass_bits(key_bits, p)) * tiles);
    return total;
}

size_t radix_sort_temp_bytes(uint64_t n) {
    uint64_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    uint64_t hist = tiles * MAX_RADIX;
    return 2 * align_up(n * sizeof(uint32_t)) + 2 * align_up(hist * sizeof(uint32_t)) + scan_temp_bytes(hist);
}

cudaError_t radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                             uint32_t *vals_out, uint64_t n, int key_bits, void *temp, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    if (n >= (1ull << 32)) return cudaErrorInvalidValue;
    if (key_bits <= 0) {
        cudaError_t e = cudaMemcpyAsync(keys_out, keys_in, n * 4, cudaMemcpyDeviceToDevice, stream);
        if (e != cudaSuccess) return e;
        return cudaMemcpyAsync(vals_out, vals_in, n * 4, cudaMemcpyDeviceToDevice, stream);
    }
    if (key_bits > 32) key_bits = 32;
    uint32_t tiles = (uint32_t)((n + SORT_TILE - 1) / SORT_TILE);
    uint64_t hist_n = (uint64_t)tiles * MAX_RADIX;
    char *t = static_cast<char *>(temp);
    uint32_t *alt_keys = reinterpret_cast<uint32_t *>(t);
    t += align_up(n * 4);
    uint32_t *alt_vals = reinterpret_cast<uint32_t *>(t);
    t += align_up(n * 4);
    uint32_t *hist = reinterpret_cast<uint32_t *>(t);
    t += align_up(hist_n * 4);
    uint32_t *scanned = reinterpret_cast<uint32_t *>(t);
    t += align_up(hist_n * 4);
    void *scan_temp = t;

    const int passes = sort_passes(key_bits);
    const uint32_t *src_k = keys_in, *src_v = vals_in;
    int shift = 0;
    for (int p = 0; p < passes; ++p) {
        const int bits = pass_bits(key_bits, p);
        uint32_t mask = (1u << bits) - 1u;
        bool to_out = ((passes - 1 - p) % 2) == 0;
        uint32_t *dk = to_out ? keys_out : alt_keys, *dv = to_out ? vals_out : alt_vals;
        uint64_t used = (uint64_t)(mask + 1) * tiles;
        if (bits <= 8) k_radix_hist<256><<<tiles, SORT_THREADS, 0, stream>>>(src_k, n, shift, mask, hist, tiles);
        else if (bits == 9) k_radix_hist<512><<<tiles, SORT_THREADS, 0, stream>>>(src_k, n, shift, mask, hist, tiles);
        else k_radix_hist<MAX_RADIX><<<tiles, SORT_THREADS, 0, stream>>>(src_k, n, shift, mask, hist, tiles);
        cudaError_t err = exclusive_scan_u32(hist, scanned, used, scan_temp, stream);
        if (err != cudaSuccess) return err;
        if (bits <= 8)
            k_radix_scatter<256><<<tiles, SORT_THREADS, 0, stream>>>(src_k, src_v, dk, dv, n, shift, mask, scanned, tiles);
        else if (bits == 9)
            k_radix_scatter<512><<<tiles, SORT_THREADS, 0, stream>>>(src_k, src_v, dk, dv, n, shift, mask, scanned, tiles);
        else
            k_radix_scatter<MAX_RADIX><<<tiles, SORT_THREADS, 0, stream>>>(src_k, src_v, dk, dv, n, shift, mask, scanned, tiles);
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        src_k = dk, src_v = dv;
        shift += bits;
    }
    return cudaSuccess;
}

}  // namespace sv

// ---------------------------------------------------------------------------
// Allocation-free sort (sv_sort_pairs_noalloc in the C ABI).
//
// Some callers cannot call cudaMalloc: a plugin inside a host application
// that owns the whole device-memory budget through its own pool (an
// allocation behind its back breaks that accounting), or a loop with a time
// budget per iteration that cannot take the device-wide synchronisation a
// cudaMalloc or cudaFree may cause.  For them the sort's scratch (the sorted keys,
// the ping-pong pair buffers, the digit histograms and the scan partials)
// lives in one file-scope device array of fixed size instead, so the call
// allocates nothing.  The array exists on every GPU that loads the library
// for the life of the process.
namespace sv {
namespace {

constexpr uint64_t NOALLOC_MAX_KEYS = 1ull << 20;  // SV_NOALLOC_MAX_KEYS in the C header

constexpr size_t ce_align(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t ce_scan_temp(uint64_t n) {
    return n > (uint64_t)SCAN_TILE ? ce_align(((n + SCAN_TILE - 1) / SCAN_TILE) * 4) + ce_scan_temp((n + SCAN_TILE - 1) / SCAN_TILE)
                                   : 256;
}
constexpr size_t ce_sort_temp(uint64_t n) {
    return 2 * ce_align(n * 4) + 2 * ce_align(((n + SORT_TILE - 1) / SORT_TILE) * MAX_RADIX * 4) +
           ce_scan_temp(((n + SORT_TILE - 1) / SORT_TILE) * MAX_RADIX);
}
// sorted keys, then the radix sort's temporary storage
constexpr size_t NOALLOC_KEYS_BYTES = ce_align(NOALLOC_MAX_KEYS * 4);
constexpr size_t NOALLOC_BYTES = NOALLOC_KEYS_BYTES + ce_sort_temp(NOALLOC_MAX_KEYS);
// 4 MiB of sorted keys + 8 MiB of ping-pong pairs + 4 MiB of digit
// histograms + 768 B of scan partials; the C header states this figure
static_assert(NOALLOC_BYTES == 16777984, "no-alloc scratch size changed: update SV_NOALLOC_SCRATCH_BYTES");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Device address of g_noalloc_scratch per device, looked up once per device
// with that device current (the host-side name is only a stand-in).
constexpr int NOALLOC_MAX_DEVICES = 64;
void *g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};
std::mutex g_noalloc_mutex;

}  // namespace

}  // namespace sv

extern "C" {

int sv_sort_pairs_noalloc(const uint32_t *keys, uint32_t *perm, uint64_t n, void *stream, char *error, uint64_t error_capacity) {
    using namespace sv;
    auto report = [&](const char *msg) {
        if (error && error_capacity) {
            std::strncpy(error, msg, error_capacity - 1);
            error[error_capacity - 1] = 0;
        }
        return -1;
    };
    if (n == 0) return 0;
    if (n > NOALLOC_MAX_KEYS) return report("sv_sort_pairs_noalloc: n exceeds SV_NOALLOC_MAX_KEYS (1048576)");
    if (!keys || !perm) return report("sv_sort_pairs_noalloc: NULL argument");
    if (radix_sort_temp_bytes(n) > NOALLOC_BYTES - NOALLOC_KEYS_BYTES)
        return report("sv_sort_pairs_noalloc: internal scratch size mismatch");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return report("sv_sort_pairs_noalloc: no usable current device");
    void *base;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_addr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return report(cudaGetErrorString(e));
            g_noalloc_addr[dev] = p;
        }
        base = g_noalloc_addr[dev];
    }
    // Nothing in the scratch needs to start at zero: every histogram, scan
    // and pair buffer is fully written before it is read.
    uint32_t *sorted_keys = static_cast<uint32_t *>(base);
    void *temp = static_cast<unsigned char *>(base) + NOALLOC_KEYS_BYTES;
    cudaError_t e = radix_sort_pairs(keys, nullptr, sorted_keys, perm, n, 32, temp, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return report(cudaGetErrorString(e));
    return 0;
}

}  // extern "C"
