// sv_mlp.cuh -- per-CTA control of the tensor-core MLP (TMEM allocation,
// the MMA-completion mbarrier with bounded waits) and the 128-row inference
// tile shared by the standalone forward kernel and the particle kernel.
#pragma once
#include <cuda_runtime.h>

#include "sv_tc.cuh"

namespace sv {
namespace mlp {

constexpr int TMEM_COLS_INFER = 32;
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

// One 128-row tile through the network: thread t's input row x, output y.
// a0 [128 x NIN] and a1 [128 x NH] are operand buffers (1 KB aligned), img
// the packed weight image in shared memory.  Returns this thread's status:
// false when a wait gave up (y is then meaningless).
__device__ __forceinline__ bool infer_tile(Ctl &c, Phase &ph, const uint8_t *img, uint8_t *a0, uint8_t *a1,
                                           const float x[tc::NIN], float y[tc::NOUT]) {
    using namespace tc;
    const int t = threadIdx.x;
    const uint32_t tm = c.tmem;
    store_row8(a0, t, 0, NIN, x);
    store_row8(a0, t, 8, NIN, x + 8);
    if (!issue(c, ph, [&] { mma_bf16(tm, smem_u32(a0), smem_u32(img + IMG_W1), NIN, NH, false); })) {
#pragma unroll
        for (int k = 0; k < NOUT; ++k) y[k] = 0.f;
        return false;
    }
    float h[NH];
    tmem_ld16(tmem_lane_addr(tm, 0), h);
    tmem_ld16(tmem_lane_addr(tm, 16), h + 16);
    const float *b1 = reinterpret_cast<const float *>(img + IMG_B1);
#pragma unroll
    for (int j = 0; j < NH; ++j) h[j] = fmaxf(h[j] + b1[j], 0.f);
#pragma unroll
    for (int k = 0; k < NH / 8; ++k) store_row8(a1, t, 8 * k, NH, h + 8 * k);
    if (!issue(c, ph, [&] { mma_bf16(tm, smem_u32(a1), smem_u32(img + IMG_W2), NH, NH, false); })) {
#pragma unroll
        for (int k = 0; k < NOUT; ++k) y[k] = 0.f;
        return false;
    }
    tmem_ld16(tmem_lane_addr(tm, 0), h);
    tmem_ld16(tmem_lane_addr(tm, 16), h + 16);
    const float *b2 = reinterpret_cast<const float *>(img + IMG_B2);
#pragma unroll
    for (int j = 0; j < NH; ++j) h[j] = fmaxf(h[j] + b2[j], 0.f);
#pragma unroll
    for (int k = 0; k < NH / 8; ++k) store_row8(a1, t, 8 * k, NH, h + 8 * k);
    if (!issue(c, ph, [&] { mma_bf16(tm, smem_u32(a1), smem_u32(img + IMG_W3), NH, NOUT, false); })) {
#pragma unroll
        for (int k = 0; k < NOUT; ++k) y[k] = 0.f;
        return false;
    }
    tmem_ld16(tmem_lane_addr(tm, 0), y);
    const float *b3 = reinterpret_cast<const float *>(img + IMG_B3);
#pragma unroll
    for (int k = 0; k < NOUT; ++k) y[k] += b3[k];
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
