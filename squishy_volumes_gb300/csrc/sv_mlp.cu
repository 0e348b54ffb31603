// sv_mlp.cu -- the learned stress closure's MLP on the tensor cores: forward
// (inference) and training (forward + backward) kernels built on tcgen05, the
// Adam update that also writes the packed bf16 weight image, and the
// stateless C entry points sv_mlp_forward / sv_mlp_grad used to check the
// kernels against a CPU evaluation of the same network.
//
// Precision: weights and activations of the hidden layers enter the tensor
// core as bf16, every product is accumulated in fp32 (TMEM); biases, SiLU,
// the head (which reads the last hidden layer in fp32), the loss and the
// Adam state are fp32.
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
        const int r = idx / NIN, k = idx % NIN;  // W1[r][k]: out r, in k
        put_bf16(img, IMG_W1 + kmaj(r, k, NIN), v);
        return;
    }
    if (idx >= P_W5) {
        if (idx < P_B5) reinterpret_cast<float *>(img + IMG_W5)[idx - P_W5] = v;
        else reinterpret_cast<float *>(img + IMG_B5)[idx - P_B5] = v;
        return;
    }
    for (int layer = 1; layer <= N_HIDDEN; ++layer) {
        const int pb = p_bias(layer);
        if (idx >= pb && idx < pb + NH) {
            reinterpret_cast<float *>(img + IMG_BH)[(layer - 1) * NH + idx - pb] = v;
            return;
        }
        if (layer >= 2) {
            const int pw = p_weight(layer);
            if (idx >= pw && idx < pw + NH * NH) {
                const int e = idx - pw, r = e / NH, k = e % NH;  // out r, in k
                put_bf16(img, img_weight(layer) + kmaj(r, k, NH), v);
                put_bf16(img, img_weight_t(layer) + kmaj(k, r, NH), v);
                return;
            }
        }
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
// Dynamic shared memory: the forward image, then the two operand buffers.
constexpr int FW_A0 = IMG_FWD_BYTES;
constexpr int FW_A1 = FW_A0 + T * NIN * 2;
constexpr int FW_BYTES = FW_A1 + T * NH * 2;

__global__ void __launch_bounds__(T) k_mlp_forward(const uint8_t *img, const float *X, uint64_t n, float *Y,
                                                   uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ Ctl ctl;
    copy_to_smem(sm, img, IMG_FWD_BYTES);
    ctl_init(ctl, TMEM_COLS_INFER);
    Phase ph;
    const uint64_t tiles = (n + T - 1) / T;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t row = tile * T + threadIdx.x;
        float x[NIN], y[NOUT];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = (row < n && k < NIN - 1) ? X[row * NIN + k] : 0.f;  // input 15 reserved
        infer_tile(ctl, ph, sm, sm + FW_A0, sm + FW_A1, x, y);
        if (row < n)
#pragma unroll
            for (int k = 0; k < NOUT; ++k) Y[row * NOUT + k] = y[k];
    }
    ctl_finish(ctl, TMEM_COLS_INFER, err);
}

// ------------------------------------------------------------------ training
// Dynamic shared memory of the training kernel.  K-major bf16 operands:
//   A0   X              [128 samples x NIN]     layer 1 (forward, recompute)
//   AH   H_l            [128 x NH]              the next layer's A operand
//   G    dZ_l           [128 x NH]              A operand of dH_(l-1) = dZ_l W_l
//   TA   H4^T, dZ_l^T   [128 rows x 128 samples] A operand of the weight
//        gradients (rows = units; row NH is ones: dW5^T's row NH is db5)
//   DYT  dY^T           [16 x 128 samples]      B operand of dW5^T
//   TB0  X^T            [NIN x 128]             row NIN-1 is ones (db1)
//   TB1..TB3 H_l^T      [NH + 16 x 128]          row NH is ones (db2..db4)
constexpr int TB_ROWS = NH + 16;
constexpr int TR_IMG = 0;
constexpr int TR_A0 = IMG_BYTES;
constexpr int TR_AH = TR_A0 + T * NIN * 2;
constexpr int TR_G = TR_AH + T * NH * 2;
constexpr int TR_TA = TR_G + T * NH * 2;
constexpr int TR_DYT = TR_TA + T * T * 2;
constexpr int TR_TB0 = TR_DYT + 16 * T * 2;
constexpr int TR_TB1 = TR_TB0 + NIN * T * 2;
constexpr int TR_TB2 = TR_TB1 + TB_ROWS * T * 2;
constexpr int TR_TB3 = TR_TB2 + TB_ROWS * T * 2;
constexpr int TR_BYTES = TR_TB3 + TB_ROWS * T * 2;
static_assert(TR_A0 % 128 == 0 && TR_TA % 128 == 0 && TR_BYTES <= 227 * 1024, "training shared memory");
// TMEM columns: the pre-activations z2..z4 (z1 lands in Z3's columns in the
// forward pass and is recomputed there in the backward pass; each input
// gradient reuses the columns of the layer it was taken from), then the
// weight-gradient accumulators (rows = output units; their last used column
// is the bias gradient).
constexpr int TM_Z2 = 0, TM_Z3 = 64, TM_Z4 = 128;
constexpr int TM_DW2 = 192, TM_DW3 = TM_DW2 + TB_ROWS, TM_DW4 = TM_DW3 + TB_ROWS;
constexpr int TM_DW1 = TM_DW4 + TB_ROWS, TM_DW5 = TM_DW1 + 16, TM_COLS = 512;
static_assert(TM_DW5 + 16 <= TM_COLS, "TMEM columns");

__device__ __forceinline__ void put_col(uint8_t *buf, int t, int r, float v) { put_bf16(buf, kmaj(r, t, T), v); }

__global__ void __launch_bounds__(T) k_mlp_train(const uint8_t *img, const float *X, const float *Ytgt,
                                                 const float *Wt, uint64_t n, float inv_n, float *grad, float *loss,
                                                 float *Yout, uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ Ctl ctl;
    const int t = threadIdx.x;
    uint8_t *s_img = sm + TR_IMG;
    copy_to_smem(s_img, img, IMG_BYTES);
    // the constant rows: ones for the bias gradients, zero padding
    put_col(sm + TR_TB0, t, NIN - 1, 1.f);
    for (int r = NH; r < TB_ROWS; ++r) {
        const float v = r == NH ? 1.f : 0.f;
        put_col(sm + TR_TB1, t, r, v), put_col(sm + TR_TB2, t, r, v), put_col(sm + TR_TB3, t, r, v);
    }
    for (int r = NH; r < T; ++r) put_col(sm + TR_TA, t, r, r == NH ? 1.f : 0.f);
    for (int r = NOUT; r < 16; ++r) put_col(sm + TR_DYT, t, r, 0.f);
    ctl_init(ctl, TM_COLS);
    Phase ph;
    const uint32_t tm = ctl.tmem;
    const float *bh = reinterpret_cast<const float *>(s_img + IMG_BH);
    const float *w5 = reinterpret_cast<const float *>(s_img + IMG_W5);
    const float *b5 = reinterpret_cast<const float *>(s_img + IMG_B5);
    const uint64_t tiles = (n + T - 1) / T;
    bool first = true;
    float lsum = 0.f;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t row = tile * T + t;
        const bool valid = row < n;
        float x[NIN];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = (valid && k < NIN - 1) ? X[row * NIN + k] : 0.f;  // input 15 reserved
        store_row8(sm + TR_A0, t, 0, NIN, x);
        store_row8(sm + TR_A0, t, 8, NIN, x + 8);
        for (int r = 0; r < NIN - 1; ++r) put_col(sm + TR_TB0, t, r, x[r]);
        // ---- forward: hidden layers 1..3 into AH and TB1..TB3
        if (!issue(ctl, ph, [&] { mma_bf16(tm + TM_Z3, smem_u32(sm + TR_A0), smem_u32(s_img + IMG_W1), NIN, NH, false); }))
            break;
        bool ok = true;
#pragma unroll 1
        for (int layer = 1; layer <= 3 && ok; ++layer) {
            const int zc = layer == 1 ? TM_Z3 : layer == 2 ? TM_Z2 : TM_Z3;
            uint8_t *tb = sm + (layer == 1 ? TR_TB1 : layer == 2 ? TR_TB2 : TR_TB3);
            for (int q = 0; q < NH / 16; ++q) {
                float h[16];
                tmem_ld16(tmem_lane_addr(tm, zc + 16 * q), h);
                for (int j = 0; j < 16; ++j) {
                    const float z = h[j] + bh[(layer - 1) * NH + 16 * q + j];
                    h[j] = z * sigmoid_f(z);
                    put_col(tb, t, 16 * q + j, h[j]);
                }
                store_row8(sm + TR_AH, t, 16 * q, NH, h);
                store_row8(sm + TR_AH, t, 16 * q + 8, NH, h + 8);
            }
            const int dst = layer == 1 ? TM_Z2 : layer == 2 ? TM_Z3 : TM_Z4;
            ok = issue(ctl, ph, [&] {
                mma_bf16(tm + dst, smem_u32(sm + TR_AH), smem_u32(s_img + img_weight(layer + 1)), NH, NH, false);
            });
        }
        if (!ok) break;
        // ---- layer 4 and the fp32 head; h4^T into TA for dW5^T
        float y[NOUT];
        for (int o = 0; o < NOUT; ++o) y[o] = b5[o];
        for (int q = 0; q < NH / 16; ++q) {
            float h[16];
            tmem_ld16(tmem_lane_addr(tm, TM_Z4 + 16 * q), h);
            for (int j = 0; j < 16; ++j) {
                const float z = h[j] + bh[3 * NH + 16 * q + j];
                h[j] = z * sigmoid_f(z);
                put_col(sm + TR_TA, t, 16 * q + j, h[j]);
            }
            for (int o = 0; o < NOUT; ++o) {
                float acc = y[o];
                for (int j = 0; j < 16; ++j) acc = fmaf(w5[o * NH + 16 * q + j], h[j], acc);
                y[o] = acc;
            }
        }
        // loss = sum_rows w sum_{o < N_USED_OUT} (y - t)^2 * inv_n
        float dy[NOUT];
        const float wr = valid ? (Wt ? Wt[row] : 1.f) : 0.f;
        for (int o = 0; o < NOUT; ++o) {
            const float tg = (valid && o < N_USED_OUT) ? Ytgt[row * NOUT + o] : y[o];
            const float d = y[o] - tg;
            lsum += wr * d * d * inv_n;
            dy[o] = (o < N_USED_OUT) ? 2.f * wr * d * inv_n : 0.f;
            put_col(sm + TR_DYT, t, o, dy[o]);
        }
        if (Yout && valid)
            for (int o = 0; o < NOUT; ++o) Yout[row * NOUT + o] = y[o];
        // dW5^T (+)= H4^T dY (row NH: db5)
        if (!issue(ctl, ph, [&] {
                mma_bf16(tm + TM_DW5, smem_u32(sm + TR_TA), smem_u32(sm + TR_DYT), T, 16, !first);
            }))
            break;
        // ---- backward through layers 4..1
#pragma unroll 1
        for (int layer = 4; layer >= 1 && ok; --layer) {
            // the layer's pre-activation and the gradient of its output
            const int zc = layer == 4 ? TM_Z4 : layer == 3 ? TM_Z3 : layer == 2 ? TM_Z2 : TM_Z3;
            const int gc = layer == 3 ? TM_Z4 : layer == 2 ? TM_Z3 : TM_Z2;  // dH_layer (layers 1..3)
            for (int q = 0; q < NH / 16; ++q) {
                float z[16], dh[16];
                tmem_ld16(tmem_lane_addr(tm, zc + 16 * q), z);
                if (layer == 4) {
                    for (int j = 0; j < 16; ++j) {
                        float a = 0.f;
                        for (int o = 0; o < N_USED_OUT; ++o) a = fmaf(dy[o], w5[o * NH + 16 * q + j], a);
                        dh[j] = a;
                    }
                } else {
                    tmem_ld16(tmem_lane_addr(tm, gc + 16 * q), dh);
                }
                for (int j = 0; j < 16; ++j) {
                    const float zz = z[j] + bh[(layer - 1) * NH + 16 * q + j];
                    const float sg = sigmoid_f(zz);
                    dh[j] *= sg * (1.f + zz * (1.f - sg));  // dZ
                    put_col(sm + TR_TA, t, 16 * q + j, dh[j]);
                }
                if (layer > 1) {
                    store_row8(sm + TR_G, t, 16 * q, NH, dh);
                    store_row8(sm + TR_G, t, 16 * q + 8, NH, dh + 8);
                }
            }
            if (layer == 4) {
                ok = issue(ctl, ph, [&] {
                    mma_bf16(tm + TM_Z4, smem_u32(sm + TR_G), smem_u32(s_img + IMG_W4T), NH, NH, false);
                    mma_bf16(tm + TM_DW4, smem_u32(sm + TR_TA), smem_u32(sm + TR_TB3), T, TB_ROWS, !first);
                });
            } else if (layer == 3) {
                ok = issue(ctl, ph, [&] {
                    mma_bf16(tm + TM_Z3, smem_u32(sm + TR_G), smem_u32(s_img + IMG_W3T), NH, NH, false);
                    mma_bf16(tm + TM_DW3, smem_u32(sm + TR_TA), smem_u32(sm + TR_TB2), T, TB_ROWS, !first);
                });
            } else if (layer == 2) {
                // dH1, dW2, and z1 recomputed into Z3's columns
                ok = issue(ctl, ph, [&] {
                    mma_bf16(tm + TM_Z2, smem_u32(sm + TR_G), smem_u32(s_img + IMG_W2T), NH, NH, false);
                    mma_bf16(tm + TM_DW2, smem_u32(sm + TR_TA), smem_u32(sm + TR_TB1), T, TB_ROWS, !first);
                    mma_bf16(tm + TM_Z3, smem_u32(sm + TR_A0), smem_u32(s_img + IMG_W1), NIN, NH, false);
                });
            } else {
                ok = issue(ctl, ph, [&] {
                    mma_bf16(tm + TM_DW1, smem_u32(sm + TR_TA), smem_u32(sm + TR_TB0), T, NIN, !first);
                });
            }
        }
        if (!ok) break;
        first = false;
    }
    // weight gradients: threads t < NH read row t of each accumulator (the
    // rows of the output units); column NH (NIN - 1 for layer 1) is the bias
    fence_before();
    __syncthreads();
    fence_after();
    if (!first && !ctl.abort && t < 96) {  // warps 0..2 (abort is uniform after the barrier)
        float r[16];
        for (int layer = 2; layer <= 4; ++layer) {
            const int col0 = layer == 2 ? TM_DW2 : layer == 3 ? TM_DW3 : TM_DW4;
            for (int c = 0; c < TB_ROWS; c += 16) {
                tmem_ld16(tmem_lane_addr(tm, col0 + c), r);
                if (t < NH)
                    for (int k = 0; k < 16; ++k) {
                        if (c + k < NH) atomicAdd(&grad[p_weight(layer) + t * NH + c + k], r[k]);
                        else if (c + k == NH) atomicAdd(&grad[p_bias(layer) + t], r[k]);
                    }
            }
        }
        tmem_ld16(tmem_lane_addr(tm, TM_DW1), r);
        if (t < NH) {
            for (int k = 0; k < NIN - 1; ++k) atomicAdd(&grad[P_W1 + t * NIN + k], r[k]);
            atomicAdd(&grad[P_B1 + t], r[NIN - 1]);
        }
        tmem_ld16(tmem_lane_addr(tm, TM_DW5), r);  // row j: dW5[o][j]; row NH: db5[o]
        if (t < NH)
            for (int o = 0; o < NOUT; ++o) atomicAdd(&grad[P_W5 + o * NH + t], r[o]);
        else if (t == NH)
            for (int o = 0; o < NOUT; ++o) atomicAdd(&grad[P_B5 + o], r[o]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, lsum);
    ctl_finish(ctl, TM_COLS, err);
}

}  // namespace

int train_blocks() { return sm_count(); }  // one CTA per SM: all of its TMEM and most of its shared memory

cudaError_t pack_image(const float *params, uint8_t *img, cudaStream_t s) {
    k_pack_image<<<(N_PARAMS + 255) / 256, 256, 0, s>>>(params, img);
    return cudaGetLastError();
}

cudaError_t forward(const uint8_t *img, const float *X, uint64_t n, float *Y, uint32_t *err, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t tiles = (n + T - 1) / T;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, FW_BYTES);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const unsigned blocks = (unsigned)std::min<uint64_t>(tiles, (uint64_t)sm_count() * 4);
    k_mlp_forward<<<blocks, T, FW_BYTES, s>>>(img, X, n, Y, err);
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
