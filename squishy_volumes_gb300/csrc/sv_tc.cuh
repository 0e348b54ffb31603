// sv_tc.cuh -- Blackwell tensor-core (tcgen05) primitives and the layout of
// the learned stress closure's small MLP.
//
// tcgen05 in one paragraph: one thread of a CTA issues tcgen05.mma; A and B
// come from shared memory through 64-bit matrix descriptors, the fp32
// accumulator D lives in tensor memory (TMEM: 128 lanes x 512 columns of 32
// bits per SM, allocated per CTA in power-of-two column counts), completion
// is signalled by tcgen05.commit on an mbarrier, and warp w of the CTA reads
// TMEM lanes 32(w%4)..32(w%4)+31 with tcgen05.ld -- so for M = 128, thread t
// of a 128-thread CTA reads row t of D.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "sv_eig.cuh"

namespace sv {
namespace tc {

// ------------------------------------------------------------------ MLP shape
// x (NIN, input NIN-1 reserved and zero) -> four hidden layers of width NH,
// h = silu(W h_prev + b) on the tensor cores (bf16 operands, fp32
// accumulation) -> an fp32 head y = W5 h4 + b5 (NOUT outputs, the first
// N_USED_OUT used) on the CUDA cores, reading the last hidden layer in fp32.
constexpr int NIN = 16;   // padded input width (one K = 16 MMA step)
constexpr int NH = 64;    // hidden width
constexpr int N_HIDDEN = 4;
constexpr int NOUT = 8;   // head outputs
constexpr int N_USED_OUT = 6;
// fp32 master parameters: W1 [NH x NIN], b1, then W2..W4 [NH x NH] with
// their biases, then W5 [NOUT x NH], b5 (row-major, out x in)
constexpr int P_W1 = 0, P_B1 = P_W1 + NH * NIN;
constexpr int P_W2 = P_B1 + NH, P_B2 = P_W2 + NH * NH;
constexpr int P_W3 = P_B2 + NH, P_B3 = P_W3 + NH * NH;
constexpr int P_W4 = P_B3 + NH, P_B4 = P_W4 + NH * NH;
constexpr int P_W5 = P_B4 + NH, P_B5 = P_W5 + NOUT * NH;
constexpr int N_PARAMS = P_B5 + NOUT;
__host__ __device__ constexpr int p_weight(int layer) { return layer == 1 ? P_W1 : layer == 2 ? P_W2 : layer == 3 ? P_W3 : P_W4; }
__host__ __device__ constexpr int p_bias(int layer) { return layer == 1 ? P_B1 : layer == 2 ? P_B2 : layer == 3 ? P_B3 : P_B4; }

// Byte offset of element (r, k) of an R x K bf16 matrix in the canonical
// K-major layout without swizzle: 8-row x 16-byte core matrices, the core
// matrices of one 8-row group adjacent along K (leading byte offset 128), the
// groups K * 16 bytes apart (stride byte offset).
__host__ __device__ constexpr int kmaj(int r, int k, int K) {
    return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Packed weight image (copied verbatim into shared memory).  The forward
// part first (all an inference pass reads): W1 [NH x NIN] and W2..W4
// [NH x NH] as bf16 B operands (N = output units, K = input units), the
// hidden biases b1..b4 in fp32, the head W5 [NOUT x NH] and b5 in fp32.
// Then, for the backward pass, W2^T..W4^T [NH x NH] as bf16 B operands of the
// input-gradient products (N = input units, K = output units).
constexpr int IMG_W1 = 0;
constexpr int IMG_W2 = IMG_W1 + NH * NIN * 2;
constexpr int IMG_W3 = IMG_W2 + NH * NH * 2;
constexpr int IMG_W4 = IMG_W3 + NH * NH * 2;
constexpr int IMG_BH = IMG_W4 + NH * NH * 2;        // b1..b4, fp32 [4][NH]
constexpr int IMG_W5 = IMG_BH + N_HIDDEN * NH * 4;  // fp32 [NOUT][NH]
constexpr int IMG_B5 = IMG_W5 + NOUT * NH * 4;      // fp32 [NOUT]
constexpr int IMG_FWD_BYTES = (IMG_B5 + NOUT * 4 + 127) / 128 * 128;
constexpr int IMG_W2T = IMG_FWD_BYTES;
constexpr int IMG_W3T = IMG_W2T + NH * NH * 2;
constexpr int IMG_W4T = IMG_W3T + NH * NH * 2;
constexpr int IMG_BYTES = IMG_W4T + NH * NH * 2;
__host__ __device__ constexpr int img_weight(int layer) { return layer == 1 ? IMG_W1 : layer == 2 ? IMG_W2 : layer == 3 ? IMG_W3 : IMG_W4; }
__host__ __device__ constexpr int img_weight_t(int layer) { return layer == 2 ? IMG_W2T : layer == 3 ? IMG_W3T : IMG_W4T; }
static_assert(IMG_W2 % 128 == 0 && IMG_W3 % 128 == 0 && IMG_W4 % 128 == 0 && IMG_W2T % 128 == 0 &&
                  IMG_W3T % 128 == 0 && IMG_W4T % 128 == 0 && IMG_BH % 16 == 0 && IMG_W5 % 16 == 0,
              "operand images must stay 128-byte aligned");

// silu(z) = z sigmoid(z) and its derivative sigmoid(z) (1 + z (1 - sigmoid(z)))
__device__ __forceinline__ float sigmoid_f(float z) { return __frcp_rn(1.f + __expf(-z)); }

// Instruction descriptor of tcgen05.mma kind::f16: D fp32 (bits 4-5 = 1),
// A and B bf16 (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset >> 4 (bits 16-29), stride byte offset >> 4 (bits 32-45), the
// fixed version 1 (bits 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {  // one full warp
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {  // the allocating warp
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Waits for the mbarrier phase with parity `parity` to complete, for at most
// `max_cycles` SM clocks; false when the limit was hit.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long max_cycles) {
    const uint32_t a = smem_u32(bar);
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > max_cycles) return false;
    }
}

// D[128 x N] (+)= A[128 x K] B[N x K]^T, all K-major bf16 in the layout of
// kmaj(); issued by one thread.  K is a multiple of 16.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint32_t a_smem, uint32_t b_smem, int K, int N,
                                         bool accumulate) {
    const uint32_t idesc = idesc_bf16(128, N);
    const uint32_t sbo = (uint32_t)K * 16u;
    for (int kk = 0; kk < K / 16; ++kk) {
        const uint64_t ad = smem_desc(a_smem + kk * 256, 128, sbo);
        const uint64_t bd = smem_desc(b_smem + kk * 256, 128, sbo);
        const uint32_t acc = (accumulate || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                d_tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
    }
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive fp32 columns of this thread's TMEM lane (row).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// TMEM address of this warp's lane quarter, column `col`.
__device__ __forceinline__ uint32_t tmem_lane_addr(uint32_t base, int col) {
    const uint32_t quarter = (threadIdx.x >> 5) & 3;
    return base + ((quarter * 32u) << 16) + (uint32_t)col;
}

// Writes 8 values as one 16-byte chunk of row r of a K-major operand.
__device__ __forceinline__ void store_row8(uint8_t *base, int r, int k0, int K, const float v[8]) {
    __nv_bfloat162 q[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) q[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4 *>(base + kmaj(r, k0, K)) = *reinterpret_cast<uint4 *>(q);
}

}  // namespace tc

}  // namespace sv
