// sv_mlp.cu -- the learned stress closure's MLP on the tensor cores: forward
// (inference) and training (forward + backward) kernels built on tcgen05, the
// Adam update that also writes the packed bf16 weight image, and the
// stateless C entry points sv_mlp_forward / sv_mlp_grad used to check the
// kernels against a CPU evaluation of the same network.
//
// Precision: weights and activations enter the tensor core as bf16, every
// product is accumulated in fp32 (TMEM), biases, ReLU, the loss and the Adam
// state are fp32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "sv_internal.h"
#include "sv_mlp.cuh"

namespace sv {
namespace mlp {

using namespace tc;

namespace {

constexpr int T = 128;                 // threads per CTA = samples per tile = MMA M

// ------------------------------------------------------------------ image
__device__ __forceinline__ void put_bf16(uint8_t *img, int off, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(img + off) = __float2bfloat16_rn(v);
}

// Writes master parameter `idx` (value v) into the packed image.
__device__ __forceinline__ void image_write(uint8_t *img, int idx, float v) {
    if (idx < P_B1) {
        const int r = idx / NIN, k = idx % NIN;
        put_bf16(img, IMG_W1 + kmaj(r, k, NIN), v);
    } else if (idx < P_W2) {
        reinterpret_cast<float *>(img + IMG_B1)[idx - P_B1] = v;
    } else if (idx < P_B2) {
        const int e = idx - P_W2, r = e / NH, k = e % NH;  // W2[r][k]: out r, in k
        put_bf16(img, IMG_W2 + kmaj(r, k, NH), v);
        put_bf16(img, IMG_W2T + kmaj(k, r, NH), v);
    } else if (idx < P_W3) {
        reinterpret_cast<float *>(img + IMG_B2)[idx - P_B2] = v;
    } else if (idx < P_B3) {
        const int e = idx - P_W3, r = e / NH, k = e % NH;  // W3[r][k]: out r, in k
        put_bf16(img, IMG_W3 + kmaj(r, k, NH), v);
        put_bf16(img, IMG_W3T + kmaj(k, r, NOUT), v);
    } else {
        reinterpret_cast<float *>(img + IMG_B3)[idx - P_B3] = v;
    }
}

__global__ void k_pack_image(const float *params, uint8_t *img) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N_PARAMS; i += gridDim.x * blockDim.x)
        image_write(img, i, params[i]);
}

// Adam (Kingma & Ba 2015) with bias correction; clears the gradient and
// refreshes the image.
__global__ void k_adam(float *params, float *grad, float *m, float *v, uint8_t *img, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N_PARAMS; i += gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi, v[i] = vi;
        const float p = params[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        params[i] = p;
        grad[i] = 0.f;
        image_write(img, i, p);
    }
}

__device__ __forceinline__ void copy_to_smem(uint8_t *dst, const uint8_t *src, int bytes) {
    for (int i = threadIdx.x * 16; i < bytes; i += blockDim.x * 16)
        *reinterpret_cast<uint4 *>(dst + i) = *reinterpret_cast<const uint4 *>(src + i);
}

// ------------------------------------------------------------------ forward
__global__ void __launch_bounds__(T) k_mlp_forward(const uint8_t *img, const float *X, uint64_t n, float *Y,
                                                   uint32_t *err) {
    __shared__ __align__(1024) uint8_t s_img[IMG_BYTES];
    __shared__ __align__(1024) uint8_t s_a0[T * NIN * 2];
    __shared__ __align__(1024) uint8_t s_a1[T * NH * 2];
    __shared__ Ctl ctl;
    copy_to_smem(s_img, img, IMG_BYTES);
    ctl_init(ctl, TMEM_COLS_INFER);
    Phase ph;
    const uint64_t tiles = (n + T - 1) / T;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t row = tile * T + threadIdx.x;
        float x[NIN], y[NOUT];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = row < n ? X[row * NIN + k] : 0.f;
        infer_tile(ctl, ph, s_img, s_a0, s_a1, x, y);
        if (row < n)
#pragma unroll
            for (int k = 0; k < NOUT; ++k) Y[row * NOUT + k] = y[k];
    }
    ctl_finish(ctl, TMEM_COLS_INFER, err);
}

// ------------------------------------------------------------------ training
// Dynamic shared memory of the training kernel (operand buffers 1 KB aligned).
constexpr int TR_IMG = 0;
constexpr int TR_A0 = 8192;                     // X tile          [128 x NIN]
constexpr int TR_A1 = TR_A0 + T * NIN * 2;      // H1              [128 x NH]
constexpr int TR_A2 = TR_A1 + T * NH * 2;       // H2              [128 x NH]
constexpr int TR_G3 = TR_A2 + T * NH * 2;       // dY              [128 x NOUT]
constexpr int TR_G2 = TR_G3 + T * NOUT * 2;     // dZ2             [128 x NH]
constexpr int TR_TA = TR_G2 + T * NH * 2;       // dY^T / dZ2^T / dZ1^T [128 rows x 128 samples]
constexpr int TR_TB2 = TR_TA + T * T * 2;       // H2^T            [NH x 128]
constexpr int TR_TB1 = TR_TB2 + NH * T * 2;     // H1^T            [NH x 128]
constexpr int TR_TB0 = TR_TB1 + NH * T * 2;     // X^T             [NIN x 128]
constexpr int TR_DB = TR_TB0 + NIN * T * 2;     // bias gradient sums (fp32)
constexpr int TR_BYTES = TR_DB + (NH + NH + NOUT + 1) * 4;
static_assert(IMG_BYTES <= TR_A0, "image slot");
// TMEM columns: layer outputs / backward products, then the three weight
// gradient accumulators (rows = output units of the layer).
constexpr int TM_OUT = 0, TM_DW2 = 32, TM_DW3 = 64, TM_DW1 = 96, TM_COLS = 128;

__device__ __forceinline__ void store_col_t(uint8_t *buf, int t, const float *v, int rows) {
    // column t (sample) of a [rows x 128] K-major operand
    for (int r = 0; r < rows; ++r) put_bf16(buf, kmaj(r, t, T), v[r]);
}

__global__ void __launch_bounds__(T) k_mlp_train(const uint8_t *img, const float *X, const float *Ytgt,
                                                 const float *Wt, uint64_t n, float inv_n, float *grad, float *loss,
                                                 float *Yout, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ Ctl ctl;
    uint8_t *s_img = sm + TR_IMG;
    float *s_db = reinterpret_cast<float *>(sm + TR_DB);
    copy_to_smem(s_img, img, IMG_BYTES);
    for (int i = threadIdx.x; i < NH + NH + NOUT + 1; i += T) s_db[i] = 0.f;
    ctl_init(ctl, TM_COLS);
    Phase ph;
    const int t = threadIdx.x;
    const uint32_t tm = ctl.tmem;
    const uint64_t tiles = (n + T - 1) / T;
    bool first = true;
    float lsum = 0.f;
    const float *b1 = reinterpret_cast<const float *>(s_img + IMG_B1);
    const float *b2 = reinterpret_cast<const float *>(s_img + IMG_B2);
    const float *b3 = reinterpret_cast<const float *>(s_img + IMG_B3);
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t row = tile * T + t;
        const bool valid = row < n;
        float x[NIN];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = valid ? X[row * NIN + k] : 0.f;
        store_row8(sm + TR_A0, t, 0, NIN, x);
        store_row8(sm + TR_A0, t, 8, NIN, x + 8);
        store_col_t(sm + TR_TB0, t, x, NIN);
        // layer 1
        if (!issue(ctl, ph, [&] { mma_bf16(tm + TM_OUT, smem_u32(sm + TR_A0), smem_u32(s_img + IMG_W1), NIN, NH, false); }))
            break;
        float h1[NH];
        tmem_ld16(tmem_lane_addr(tm, TM_OUT), h1);
        tmem_ld16(tmem_lane_addr(tm, TM_OUT + 16), h1 + 16);
        uint32_t mask1 = 0;
#pragma unroll
        for (int j = 0; j < NH; ++j) {
            const float z = h1[j] + b1[j];
            mask1 |= (z > 0.f ? 1u : 0u) << j;
            h1[j] = fmaxf(z, 0.f);
        }
#pragma unroll
        for (int c = 0; c < NH / 8; ++c) store_row8(sm + TR_A1, t, 8 * c, NH, h1 + 8 * c);
        store_col_t(sm + TR_TB1, t, h1, NH);
        // layer 2
        if (!issue(ctl, ph, [&] { mma_bf16(tm + TM_OUT, smem_u32(sm + TR_A1), smem_u32(s_img + IMG_W2), NH, NH, false); }))
            break;
        float h2[NH];
        tmem_ld16(tmem_lane_addr(tm, TM_OUT), h2);
        tmem_ld16(tmem_lane_addr(tm, TM_OUT + 16), h2 + 16);
        uint32_t mask2 = 0;
#pragma unroll
        for (int j = 0; j < NH; ++j) {
            const float z = h2[j] + b2[j];
            mask2 |= (z > 0.f ? 1u : 0u) << j;
            h2[j] = fmaxf(z, 0.f);
        }
#pragma unroll
        for (int c = 0; c < NH / 8; ++c) store_row8(sm + TR_A2, t, 8 * c, NH, h2 + 8 * c);
        store_col_t(sm + TR_TB2, t, h2, NH);
        // layer 3
        if (!issue(ctl, ph, [&] { mma_bf16(tm + TM_OUT, smem_u32(sm + TR_A2), smem_u32(s_img + IMG_W3), NH, NOUT, false); }))
            break;
        float y[NOUT];
        tmem_ld16(tmem_lane_addr(tm, TM_OUT), y);
        // loss = sum_rows w sum_{o < N_USED_OUT} (y - t)^2 * inv_n
        float dy[NOUT];
        const float wr = valid ? Wt[row] : 0.f;
#pragma unroll
        for (int o = 0; o < NOUT; ++o) {
            y[o] += b3[o];
            const float tg = (valid && o < N_USED_OUT) ? Ytgt[row * NOUT + o] : y[o];
            const float d = y[o] - tg;
            lsum += wr * d * d * inv_n;
            dy[o] = (o < N_USED_OUT) ? 2.f * wr * d * inv_n : 0.f;
        }
        if (Yout && valid)
#pragma unroll
            for (int o = 0; o < NOUT; ++o) Yout[row * NOUT + o] = y[o];
#pragma unroll
        for (int o = 0; o < NOUT; ++o) atomicAdd(&s_db[NH + NH + o], dy[o]);
        store_row8(sm + TR_G3, t, 0, NOUT, dy);
        store_row8(sm + TR_G3, t, 8, NOUT, dy + 8);
        store_col_t(sm + TR_TA, t, dy, NOUT);
        // dH2 = dY W3, dW3 (+)= dY^T H2
        if (!issue(ctl, ph, [&] {
                mma_bf16(tm + TM_OUT, smem_u32(sm + TR_G3), smem_u32(s_img + IMG_W3T), NOUT, NH, false);
                mma_bf16(tm + TM_DW3, smem_u32(sm + TR_TA), smem_u32(sm + TR_TB2), T, NH, !first);
            }))
            break;
        float g2[NH];
        tmem_ld16(tmem_lane_addr(tm, TM_OUT), g2);
        tmem_ld16(tmem_lane_addr(tm, TM_OUT + 16), g2 + 16);
#pragma unroll
        for (int j = 0; j < NH; ++j) {
            g2[j] = ((mask2 >> j) & 1u) ? g2[j] : 0.f;
            atomicAdd(&s_db[NH + j], g2[j]);
        }
#pragma unroll
        for (int c = 0; c < NH / 8; ++c) store_row8(sm + TR_G2, t, 8 * c, NH, g2 + 8 * c);
        store_col_t(sm + TR_TA, t, g2, NH);
        // dH1 = dZ2 W2, dW2 (+)= dZ2^T H1
        if (!issue(ctl, ph, [&] {
                mma_bf16(tm + TM_OUT, smem_u32(sm + TR_G2), smem_u32(s_img + IMG_W2T), NH, NH, false);
                mma_bf16(tm + TM_DW2, smem_u32(sm + TR_TA), smem_u32(sm + TR_TB1), T, NH, !first);
            }))
            break;
        float g1[NH];
        tmem_ld16(tmem_lane_addr(tm, TM_OUT), g1);
        tmem_ld16(tmem_lane_addr(tm, TM_OUT + 16), g1 + 16);
#pragma unroll
        for (int j = 0; j < NH; ++j) {
            g1[j] = ((mask1 >> j) & 1u) ? g1[j] : 0.f;
            atomicAdd(&s_db[j], g1[j]);
        }
        store_col_t(sm + TR_TA, t, g1, NH);
        // dW1 (+)= dZ1^T X
        if (!issue(ctl, ph, [&] { mma_bf16(tm + TM_DW1, smem_u32(sm + TR_TA), smem_u32(sm + TR_TB0), T, NIN, !first); }))
            break;
        first = false;
    }
    // weight gradients: warp 0 reads rows 0..31 of the accumulators
    fence_before();
    __syncthreads();
    fence_after();
    if (!first && !ctl.abort && threadIdx.x < 32) {  // abort is uniform after the barrier
        float r[16];
        for (int c = 0; c < NH; c += 16) {  // dW2[t][c..c+15]
            tmem_ld16(tmem_lane_addr(tm, TM_DW2 + c), r);
            for (int k = 0; k < 16; ++k) atomicAdd(&grad[P_W2 + t * NH + c + k], r[k]);
        }
        for (int c = 0; c < NH; c += 16) {  // dW3[t][..] for t < NOUT
            tmem_ld16(tmem_lane_addr(tm, TM_DW3 + c), r);
            if (t < NOUT)
                for (int k = 0; k < 16; ++k) atomicAdd(&grad[P_W3 + t * NH + c + k], r[k]);
        }
        tmem_ld16(tmem_lane_addr(tm, TM_DW1), r);  // dW1[t][0..15]
        for (int k = 0; k < 16; ++k) atomicAdd(&grad[P_W1 + t * NIN + k], r[k]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NH + NH + NOUT; i += T) {
        const int dst = i < NH ? P_B1 + i : i < 2 * NH ? P_B2 + (i - NH) : P_B3 + (i - 2 * NH);
        atomicAdd(&grad[dst], s_db[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, lsum);
    ctl_finish(ctl, TM_COLS, err);
}

}  // namespace

int train_blocks() { return sm_count() * 2; }

cudaError_t pack_image(const float *params, uint8_t *img, cudaStream_t s) {
    k_pack_image<<<(N_PARAMS + 255) / 256, 256, 0, s>>>(params, img);
    return cudaGetLastError();
}

cudaError_t forward(const uint8_t *img, const float *X, uint64_t n, float *Y, uint32_t *err, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t tiles = (n + T - 1) / T;
    const unsigned blocks = (unsigned)std::min<uint64_t>(tiles, (uint64_t)sm_count() * 8);
    k_mlp_forward<<<blocks, T, 0, s>>>(img, X, n, Y, err);
    return cudaGetLastError();
}

cudaError_t grad(const uint8_t *img, const float *X, const float *Ytgt, const float *Wt, uint64_t n, float *g,
                 float *loss, float *Yout, uint32_t *err, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, TR_BYTES);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const uint64_t tiles = (n + T - 1) / T;
    const unsigned blocks = (unsigned)std::min<uint64_t>(tiles, (uint64_t)train_blocks());
    k_mlp_train<<<blocks, T, TR_BYTES, s>>>(img, X, Ytgt, Wt, n, 1.f / (float)n, g, loss, Yout, err);
    return cudaGetLastError();
}

cudaError_t adam(float *params, float *g, float *m, float *v, uint8_t *img, float lr, int step, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<(N_PARAMS + 255) / 256, 256, 0, s>>>(params, g, m, v, img, lr, b1, b2, 1e-8f, c1, c2);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace sv

// ------------------------------------------------------------------ C ABI
namespace {

int mlp_fail(const std::string &m) {
    sv::set_last_error(m);
    return -1;
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() { cudaFree(p); }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 16); }
};

}  // namespace

extern "C" int sv_mlp_param_count(void) { return sv::tc::N_PARAMS; }

extern "C" int sv_mlp_forward(const float *params, const float *x, uint64_t n, float *y) {
    using namespace sv;
    if (!params || (n && (!x || !y))) return mlp_fail("sv_mlp_forward: NULL argument");
    DevBuf dp, dimg, dx, dy, derr;
    cudaError_t e;
    if ((e = dp.alloc(tc::N_PARAMS * 4)) || (e = dimg.alloc(tc::IMG_BYTES)) || (e = dx.alloc(n * tc::NIN * 4)) ||
        (e = dy.alloc(n * tc::NOUT * 4)) || (e = derr.alloc(4)))
        return mlp_fail(std::string("sv_mlp_forward: ") + cudaGetErrorString(e));
    uint32_t herr = 0;
    if ((e = cudaMemcpy(dp.p, params, tc::N_PARAMS * 4, cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(dx.p, x, n * tc::NIN * 4, cudaMemcpyHostToDevice)) || (e = cudaMemset(derr.p, 0, 4)) ||
        (e = mlp::pack_image((float *)dp.p, (uint8_t *)dimg.p, 0)) ||
        (e = mlp::forward((uint8_t *)dimg.p, (float *)dx.p, n, (float *)dy.p, (uint32_t *)derr.p, 0)) ||
        (e = cudaMemcpy(y, dy.p, n * tc::NOUT * 4, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(&herr, derr.p, 4, cudaMemcpyDeviceToHost)))
        return mlp_fail(std::string("sv_mlp_forward: ") + cudaGetErrorString(e));
    if (herr) return mlp_fail("sv_mlp_forward: tensor-core wait timed out");
    return 0;
}

extern "C" int sv_mlp_grad(const float *params, const float *x, const float *t, const float *w, uint64_t n, float *y,
                           float *grad, float *loss) {
    using namespace sv;
    if (!params || !grad || !loss || (n && (!x || !t || !w))) return mlp_fail("sv_mlp_grad: NULL argument");
    DevBuf dp, dimg, dx, dt, dw, dy, dg, dl, derr;
    cudaError_t e;
    if ((e = dp.alloc(tc::N_PARAMS * 4)) || (e = dimg.alloc(tc::IMG_BYTES)) || (e = dx.alloc(n * tc::NIN * 4)) ||
        (e = dt.alloc(n * tc::NOUT * 4)) || (e = dw.alloc(n * 4)) || (e = dy.alloc(n * tc::NOUT * 4)) ||
        (e = dg.alloc(tc::N_PARAMS * 4)) || (e = dl.alloc(4)) || (e = derr.alloc(4)))
        return mlp_fail(std::string("sv_mlp_grad: ") + cudaGetErrorString(e));
    uint32_t herr = 0;
    if ((e = cudaMemcpy(dp.p, params, tc::N_PARAMS * 4, cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(dx.p, x, n * tc::NIN * 4, cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(dt.p, t, n * tc::NOUT * 4, cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(dw.p, w, n * 4, cudaMemcpyHostToDevice)) || (e = cudaMemset(dg.p, 0, tc::N_PARAMS * 4)) ||
        (e = cudaMemset(dl.p, 0, 4)) || (e = cudaMemset(derr.p, 0, 4)) ||
        (e = mlp::pack_image((float *)dp.p, (uint8_t *)dimg.p, 0)) ||
        (e = mlp::grad((uint8_t *)dimg.p, (float *)dx.p, (float *)dt.p, (float *)dw.p, n, (float *)dg.p, (float *)dl.p,
                       y ? (float *)dy.p : nullptr, (uint32_t *)derr.p, 0)) ||
        (e = cudaMemcpy(grad, dg.p, tc::N_PARAMS * 4, cudaMemcpyDeviceToHost)) ||
        (e = cudaMemcpy(loss, dl.p, 4, cudaMemcpyDeviceToHost)) ||
        (y && (e = cudaMemcpy(y, dy.p, n * tc::NOUT * 4, cudaMemcpyDeviceToHost))) ||
        (e = cudaMemcpy(&herr, derr.p, 4, cudaMemcpyDeviceToHost)))
        return mlp_fail(std::string("sv_mlp_grad: ") + cudaGetErrorString(e));
    if (herr) return mlp_fail("sv_mlp_grad: tensor-core wait timed out");
    return 0;
}
