// sv_tc.cuh -- Blackwell tensor-core (tcgen05) primitives, the layout of the
// learned stress closure's small MLP, and the closed-form eigen-solver that
// gives the closure its principal stretches without an iterative SVD.
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

namespace sv {
namespace tc {

// ------------------------------------------------------------------ MLP shape
// x (NIN) -> relu(W1 x + b1) (NH) -> relu(W2 h + b2) (NH) -> W3 h + b3 (NOUT)
constexpr int NIN = 16;   // padded input width (one K = 16 MMA step)
constexpr int NH = 32;    // hidden width
constexpr int NOUT = 16;  // padded output width (M = 128 needs N % 16 == 0)
constexpr int N_USED_OUT = 6;
constexpr int N_PARAMS = NH * NIN + NH + NH * NH + NH + NOUT * NH + NOUT;  // fp32 master parameters
// parameter offsets in the fp32 master vector
constexpr int P_W1 = 0, P_B1 = P_W1 + NH * NIN, P_W2 = P_B1 + NH, P_B2 = P_W2 + NH * NH, P_W3 = P_B2 + NH,
              P_B3 = P_W3 + NOUT * NH;

// Byte offset of element (r, k) of an R x K bf16 matrix in the canonical
// K-major layout without swizzle: 8-row x 16-byte core matrices, the core
// matrices of one 8-row group adjacent along K (leading byte offset 128), the
// groups K * 16 bytes apart (stride byte offset).
__host__ __device__ constexpr int kmaj(int r, int k, int K) {
    return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Packed bf16 weight image (copied verbatim into shared memory):
//   W1 [NH x NIN], W2 [NH x NH], W3 [NOUT x NH] as B operands of the forward
//   pass (N = output units, K = input units), W2^T [NH x NH] and W3^T
//   [NH x NOUT] as B operands of the backward pass, then b1, b2, b3 in fp32.
constexpr int IMG_W1 = 0;
constexpr int IMG_W2 = IMG_W1 + NH * NIN * 2;
constexpr int IMG_W3 = IMG_W2 + NH * NH * 2;
constexpr int IMG_W2T = IMG_W3 + NOUT * NH * 2;
constexpr int IMG_W3T = IMG_W2T + NH * NH * 2;
constexpr int IMG_B1 = IMG_W3T + NH * NOUT * 2;
constexpr int IMG_B2 = IMG_B1 + NH * 4;
constexpr int IMG_B3 = IMG_B2 + NH * 4;
constexpr int IMG_BYTES = IMG_B3 + NOUT * 4;
constexpr int IMG_FWD_BYTES = IMG_W2T;  // forward weights only (inference)
static_assert(IMG_W2 % 128 == 0 && IMG_W3 % 128 == 0 && IMG_W2T % 128 == 0 && IMG_W3T % 128 == 0 && IMG_B1 % 16 == 0,
              "operand images must stay 128-byte aligned");

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

// ------------------------------------------------------------------ eigen
// Eigen-decomposition of a symmetric 3x3 matrix in closed form, after
// D. Eberly, "A Robust Eigensolver for 3x3 Symmetric Matrices" (Geometric
// Tools, 2014): eigenvalues from the trigonometric solution of the
// characteristic cubic of the scaled, shifted matrix; the eigenvector of the
// best-separated eigenvalue from the longest cross product of two rows of
// A - lambda I; the next one from the 2x2 problem in that vector's orthogonal
// complement; the last by a cross product.  a = (a00, a01, a02, a11, a12,
// a22).  Eigenvalues come out descending, V's columns (column-major a[c*3+r])
// are the matching unit eigenvectors.
__host__ __device__ inline void sym_eig3(const float a_in[6], float lam[3], float V[9]) {
    float m = fmaxf(fmaxf(fmaxf(fabsf(a_in[0]), fabsf(a_in[1])), fmaxf(fabsf(a_in[2]), fabsf(a_in[3]))),
                    fmaxf(fabsf(a_in[4]), fabsf(a_in[5])));
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.f : 0.f;
    if (!(m > 0.f)) {
        lam[0] = lam[1] = lam[2] = 0.f;
        return;
    }
    const float s = 1.f / m;
    const float a00 = a_in[0] * s, a01 = a_in[1] * s, a02 = a_in[2] * s, a11 = a_in[3] * s, a12 = a_in[4] * s,
                a22 = a_in[5] * s;
    const float norm = a01 * a01 + a02 * a02 + a12 * a12;
    const float q = (a00 + a11 + a22) / 3.f;
    const float b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
    const float p = sqrtf((b00 * b00 + b11 * b11 + b22 * b22 + 2.f * norm) / 6.f);
    if (!(p > 0.f)) {
        lam[0] = lam[1] = lam[2] = q * m;
        return;
    }
    // det((A - qI) / p), formed from the divided entries so that a tiny p
    // (A close to a multiple of I) cannot underflow
    const float ip = 1.f / p;
    const float d00 = b00 * ip, d11 = b11 * ip, d22 = b22 * ip, d01 = a01 * ip, d02 = a02 * ip, d12 = a12 * ip;
    const float det = d00 * (d11 * d22 - d12 * d12) - d01 * (d01 * d22 - d12 * d02) + d02 * (d01 * d12 - d11 * d02);
    const float half = fminf(fmaxf(0.5f * det, -1.f), 1.f);
    const float ang = acosf(half) / 3.f;
    const float two_thirds_pi = 2.09439510239319549f;
    const float beta2 = 2.f * cosf(ang), beta0 = 2.f * cosf(ang + two_thirds_pi);
    const float beta1 = -(beta0 + beta2);
    // ascending eigenvalues of the scaled matrix
    const float al[3] = {q + p * beta0, q + p * beta1, q + p * beta2};
    const float A[3][3] = {{a00, a01, a02}, {a01, a11, a12}, {a02, a12, a22}};
    auto cross = [](const float u[3], const float v[3], float w[3]) {
        w[0] = u[1] * v[2] - u[2] * v[1];
        w[1] = u[2] * v[0] - u[0] * v[2];
        w[2] = u[0] * v[1] - u[1] * v[0];
    };
    // eigenvector of the eigenvalue `e` that is well separated from the others
    auto vec0 = [&](float e, float out[3]) {
        // rows of A - e I, scaled to a largest entry of 1 so that their cross
        // products cannot underflow when A is close to a multiple of I
        float r0[3] = {A[0][0] - e, A[0][1], A[0][2]};
        float r1[3] = {A[1][0], A[1][1] - e, A[1][2]};
        float r2[3] = {A[2][0], A[2][1], A[2][2] - e};
        float rm = 0.f;
        for (int k = 0; k < 3; ++k) rm = fmaxf(rm, fmaxf(fabsf(r0[k]), fmaxf(fabsf(r1[k]), fabsf(r2[k]))));
        if (!(rm > 0.f)) {
            out[0] = 1.f, out[1] = 0.f, out[2] = 0.f;
            return;
        }
        const float irm = 1.f / rm;
        for (int k = 0; k < 3; ++k) r0[k] *= irm, r1[k] *= irm, r2[k] *= irm;
        float x0[3], x1[3], x2[3];
        cross(r0, r1, x0);
        cross(r0, r2, x1);
        cross(r1, r2, x2);
        const float d0 = x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2];
        const float d1 = x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2];
        const float d2 = x2[0] * x2[0] + x2[1] * x2[1] + x2[2] * x2[2];
        const float *best = x0;
        float dm = d0;
        if (d1 > dm) best = x1, dm = d1;
        if (d2 > dm) best = x2, dm = d2;
        if (!(dm > 0.f)) {
            out[0] = 1.f, out[1] = 0.f, out[2] = 0.f;
            return;
        }
        const float inv = 1.f / sqrtf(dm);
        out[0] = best[0] * inv, out[1] = best[1] * inv, out[2] = best[2] * inv;
    };
    // eigenvector of `e` orthogonal to the unit vector w
    auto vec1 = [&](const float w[3], float e, float out[3]) {
        float u[3], v[3];
        if (fabsf(w[0]) > fabsf(w[1])) {
            const float inv = 1.f / sqrtf(w[0] * w[0] + w[2] * w[2]);
            u[0] = -w[2] * inv, u[1] = 0.f, u[2] = w[0] * inv;
        } else {
            const float inv = 1.f / sqrtf(w[1] * w[1] + w[2] * w[2]);
            u[0] = 0.f, u[1] = w[2] * inv, u[2] = -w[1] * inv;
        }
        cross(w, u, v);
        float au[3], av[3];
        for (int r = 0; r < 3; ++r) {
            au[r] = A[r][0] * u[0] + A[r][1] * u[1] + A[r][2] * u[2];
            av[r] = A[r][0] * v[0] + A[r][1] * v[1] + A[r][2] * v[2];
        }
        float m00 = u[0] * au[0] + u[1] * au[1] + u[2] * au[2] - e;
        float m01 = u[0] * av[0] + u[1] * av[1] + u[2] * av[2];
        float m11 = v[0] * av[0] + v[1] * av[1] + v[2] * av[2] - e;
        const float x00 = fabsf(m00), x01 = fabsf(m01), x11 = fabsf(m11);
        float cu = 1.f, cv = 0.f;  // out = cu u + cv v
        if (x00 >= x11) {
            if (fmaxf(x00, x01) > 0.f) {
                if (x00 >= x01) {
                    m01 /= m00;
                    m00 = 1.f / sqrtf(1.f + m01 * m01);
                    m01 *= m00;
                } else {
                    m00 /= m01;
                    m01 = 1.f / sqrtf(1.f + m00 * m00);
                    m00 *= m01;
                }
                cu = m01, cv = -m00;
            }
        } else {
            if (fmaxf(x11, x01) > 0.f) {
                if (x11 >= x01) {
                    m01 /= m11;
                    m11 = 1.f / sqrtf(1.f + m01 * m01);
                    m01 *= m11;
                } else {
                    m11 /= m01;
                    m01 = 1.f / sqrtf(1.f + m11 * m11);
                    m11 *= m01;
                }
                cu = m11, cv = -m01;
            }
        }
        out[0] = cu * u[0] + cv * v[0], out[1] = cu * u[1] + cv * v[1], out[2] = cu * u[2] + cv * v[2];
    };
    float e0[3], e1[3], e2[3];  // eigenvectors of al[0], al[1], al[2]
    if (half >= 0.f) {
        vec0(al[2], e2);
        vec1(e2, al[1], e1);
        cross(e1, e2, e0);
    } else {
        vec0(al[0], e0);
        vec1(e0, al[1], e1);
        cross(e0, e1, e2);
    }
    // eigenvalues as Rayleigh quotients of the eigenvectors: the cubic's
    // trigonometric roots lose accuracy at a double root, the vectors do not
    auto rq = [&](const float v[3]) {
        float s = 0.f;
        for (int r = 0; r < 3; ++r) s += v[r] * (A[r][0] * v[0] + A[r][1] * v[1] + A[r][2] * v[2]);
        return s;
    };
    lam[0] = rq(e2) * m, lam[1] = rq(e1) * m, lam[2] = rq(e0) * m;
    for (int r = 0; r < 3; ++r) V[r] = e2[r], V[3 + r] = e1[r], V[6 + r] = e0[r];
}

}  // namespace sv
