// sv_mlp.cuh -- per-CTA control of the tensor-core MLP (TMEM allocation,
// the MMA-completion mbarrier with bounded waits) and the 128-row inference
// tile shared by the standalone forward kernel and the particle kernel.
#pragma once
#include <cuda_runtime.h>

#include "sv_tc.cuh"

namespace sv {
namespace mlp {

constexpr int TMEM_COLS_INFER = 64;  // one NH-wide fp32 accumulator
constexpr long long MMA_WAIT_CYCLES = 2000000000ll;  // about one second

// Shared per-CTA state.  `abort` is only written between two barriers, so
// every thread reads the same value right after a barrier.
struct Ctl {
    uint64_t bar;
    uint32_t tmem;
    int abort;
    uint32_t fail_parity;
};

// Per-thread MMA phase tracking.
struct Phase {
    uint32_t parity = 0;
    bool ok = true;
};

// All threads of the CTA; warp 0 allocates `cols` TMEM columns.
__device__ __forceinline__ void ctl_init(Ctl &c, uint32_t cols) {
    if (threadIdx.x < 32) tc::tmem_alloc(&c.tmem, cols);
    if (threadIdx.x == 0) {
        tc::mbar_init(&c.bar, 1);
        c.abort = 0;
        c.fail_parity = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
}

// Publishes this thread's operand writes to the tensor core, lets thread 0
// issue `fn` (MMAs) and commit them, and waits (bounded) for completion.
// Returns false, uniformly over the CTA, when an earlier wait already gave
// up; a wait that gives up now marks the CTA aborted and `ph.ok` false.
template <class Fn> __device__ __forceinline__ bool issue(Ctl &c, Phase &ph, Fn fn) {
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (c.abort) return false;
    if (threadIdx.x == 0) {
        fn();
        tc::mma_commit(&c.bar);
    }
    const bool ok = tc::mbar_wait(&c.bar, ph.parity, MMA_WAIT_CYCLES);
    if (!ok) {
        c.abort = 1;
        c.fail_parity = ph.parity;
        ph.ok = false;
    }
    ph.parity ^= 1u;
    tc::fence_after();
    return true;
}

// All threads.  After an abort, waits (bounded by `wait_cycles`) once more
// for the MMA that did not finish, then frees the TMEM and raises `err`.
__device__ __forceinline__ void ctl_finish(Ctl &c, uint32_t cols, uint32_t *err, long long wait_cycles = MMA_WAIT_CYCLES) {
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (c.abort) {
        if (threadIdx.x == 0) {
            tc::mbar_wait(&c.bar, c.fail_parity, wait_cycles);
            if (err) atomicOr(err, 1u);
        }
        __syncthreads();
    }
    if (threadIdx.x < 32) tc::tmem_dealloc(c.tmem, cols);
}

// One 128-row tile through the network: thread t's input row x, outputs
// y[0 .. nout).  a0 [128 x NIN] and a1 [128 x NH] are operand buffers
// (16-byte aligned), img the packed weight image (forward part) in shared
// memory.  Each hidden layer's accumulator is read from TMEM 16 columns at a
// time, given its bias and SiLU, and written as the next layer's bf16
// operand; the last one feeds the fp32 head.  Returns this thread's status:
// false when a wait gave up (y is then meaningless).
__device__ __forceinline__ bool infer_tile(Ctl &c, Phase &ph, const uint8_t *img, uint8_t *a0, uint8_t *a1,
                                           const float x[tc::NIN], float *y, int nout = tc::NOUT) {
    using namespace tc;
    const int t = threadIdx.x;
    const uint32_t tm = c.tmem;
    store_row8(a0, t, 0, NIN, x);
    store_row8(a0, t, 8, NIN, x + 8);
    const float *bh = reinterpret_cast<const float *>(img + IMG_BH);
    const float *w5 = reinterpret_cast<const float *>(img + IMG_W5);
    const float *b5 = reinterpret_cast<const float *>(img + IMG_B5);
    for (int o = 0; o < nout; ++o) y[o] = b5[o];
    if (!issue(c, ph, [&] { mma_bf16(tm, smem_u32(a0), smem_u32(img + IMG_W1), NIN, NH, false); })) return false;
#pragma unroll 1
    for (int layer = 1; layer <= N_HIDDEN; ++layer) {
        const float *b = bh + (layer - 1) * NH;
#pragma unroll
        for (int q = 0; q < NH / 16; ++q) {
            float h[16];
            tmem_ld16(tmem_lane_addr(tm, 16 * q), h);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float z = h[j] + b[16 * q + j];
                h[j] = z * sigmoid_f(z);
            }
            if (layer < N_HIDDEN) {
                store_row8(a1, t, 16 * q, NH, h);
                store_row8(a1, t, 16 * q + 8, NH, h + 8);
            } else {
                for (int o = 0; o < nout; ++o) {
                    float acc = y[o];
#pragma unroll
                    for (int j = 0; j < 16; ++j) acc = fmaf(w5[o * NH + 16 * q + j], h[j], acc);
                    y[o] = acc;
                }
            }
        }
        if (layer < N_HIDDEN &&
            !issue(c, ph, [&] { mma_bf16(tm, smem_u32(a1), smem_u32(img + img_weight(layer + 1)), NH, NH, false); }))
            return false;
    }
    tc::fence_before();
    return ph.ok;
}

// Host-side launchers (sv_mlp.cu).
cudaError_t pack_image(const float *params, uint8_t *img, cudaStream_t s);
cudaError_t forward(const uint8_t *img, const float *X, uint64_t n, float *Y, uint32_t *err, cudaStream_t s);
cudaError_t grad(const uint8_t *img, const float *X, const float *Ytgt, const float *Wt, uint64_t n, float *g,
                 float *loss, float *Yout, uint32_t *err, cudaStream_t s);
cudaError_t adam(float *params, float *g, float *m, float *v, uint8_t *img, float lr, int step, cudaStream_t s);
int train_blocks();

}  // namespace mlp
}  // namespace sv
