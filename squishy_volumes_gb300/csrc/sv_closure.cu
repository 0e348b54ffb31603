// sv_closure.cu -- the learned stress closure's data, training and error
// evaluation (the closure itself runs inside the particle kernel):
//
//   sv_closure_harvest  trial deformation gradients F + dt C F of the snow
//                       and sand particles of the handle's current state --
//                       states the plain solver produced -- into a pool,
//                       optionally widened by a random symmetric stretch;
//   sv_closure_train    labels the pool with the fp64 SVD + return map,
//                       records the feature hull, trains the MLP on the GPU
//                       (tcgen05 forward/backward kernels, Adam);
//   sv_closure_set_mode switches sv_step between the return maps and the
//                       learned closure;
//   sv_closure_evaluate stress and projected-F errors of both paths against
//                       the fp64 return map on the current state.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "sv_closure.cuh"
#include "sv_internal.h"
#include "sv_mlp.cuh"

namespace sv {

namespace {

constexpr int CL_SAMPLE = 12;  // trial F (9), plastic J, material index bits, spare
constexpr uint64_t CL_MAX_SAMPLES = 1ull << 22;
constexpr int EVAL_SUMS = 8;

// lowbias32 integer hash (C. Wellons)
__host__ __device__ inline uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ inline float unit(uint32_t h) { return (float)(h >> 8) * (2.f / 16777216.f) - 1.f; }  // [-1, 1)

__device__ inline void trial_f(const ParticleArrays &s, uint64_t n, uint64_t i, float dt, m3f &F) {
    m3f C;
#pragma unroll
    for (int k = 0; k < 9; ++k) F.a[k] = s.F[(uint64_t)k * n + i], C.a[k] = s.C[(uint64_t)k * n + i];
    const m3f CF = mat_mul(C, F);
#pragma unroll
    for (int k = 0; k < 9; ++k) F.a[k] += CF.a[k] * dt;
}

__global__ void k_harvest(ParticleArrays s, const Material *mats, uint64_t n, float dt, uint32_t threshold,
                          uint32_t seed, float augment, float *out, uint64_t *count, uint64_t cap) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t packed = __float_as_uint(s.pos[i].w);
        if (packed & (SV_TOMBSTONED | SV_FAILED)) continue;
        const uint32_t mi = packed >> MATERIAL_SHIFT;
        const Material m = mats[mi];
        if (!closure::applies(m.kind)) continue;
        const uint32_t h = hash32((uint32_t)i * 2654435761u ^ hash32(seed));
        if (h > threshold) continue;
        m3f F;
        trial_f(s, n, i, dt, F);
        if (augment > 0.f && (hash32(h) & 1u)) {
            // F (I + a R), R symmetric with entries in [-1, 1)
            float R[9];
            uint32_t g = hash32(h ^ 0x9e3779b9u);
            for (int r = 0; r < 3; ++r)
                for (int c = r; c < 3; ++c) {
                    g = hash32(g);
                    R[c * 3 + r] = R[r * 3 + c] = augment * unit(g) + (r == c ? 1.f : 0.f);
                }
            m3f Rm;
            for (int k = 0; k < 9; ++k) Rm.a[k] = R[k];
            F = mat_mul(F, Rm);
        }
        const uint64_t slot = atomicAdd(reinterpret_cast<unsigned long long *>(count), 1ull);
        if (slot >= cap) continue;
        float *o = out + slot * CL_SAMPLE;
        for (int k = 0; k < 9; ++k) o[k] = F.a[k];
        o[9] = m.kind == KIND_SNOW ? s.vel[i].w : 1.f;
        o[10] = __uint_as_float(mi);
        o[11] = 0.f;
    }
}

// Features and targets of each sample, written at position perm[i].
__global__ void k_label(const float *samples, uint64_t n, const Material *mats, const uint32_t *perm, float *X,
                        float *Y, float *W) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float *smp = samples + i * CL_SAMPLE;
        const Material m = mats[__float_as_uint(smp[10])];
        m3d Fd, U, V;
        double S[3];
        for (int k = 0; k < 9; ++k) Fd.a[k] = (double)smp[k];
        svd3<double>(Fd, U, S, V, 12);
        // descending singular values
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2 - a; ++b)
                if (S[b] < S[b + 1]) {
                    const double t = S[b];
                    S[b] = S[b + 1], S[b + 1] = t;
                }
        const uint64_t d = perm[i];
        float x[tc::NIN], y[tc::NOUT];
        const bool valid = S[2] > 1e-6 && det3(Fd) > 0.0;
        float e[3];
        for (int k = 0; k < 3; ++k) e[k] = valid ? (float)log(S[k]) : 0.f;
        closure::features(m, e, x);
        if (valid) closure::targets(m, S, (double)smp[9], y);
        else
            for (int k = 0; k < tc::NOUT; ++k) y[k] = 0.f;
        for (int k = 0; k < tc::NIN; ++k) X[d * tc::NIN + k] = x[k];
        for (int k = 0; k < tc::NOUT; ++k) Y[d * tc::NOUT + k] = y[k];
        W[d] = valid ? 1.f : 0.f;
    }
}

// Per-block min / max of the informative features over valid samples.
__global__ void k_feature_range(const float *X, const float *W, uint64_t n, float *out) {
    __shared__ float lo[closure::N_FEAT][32], hi[closure::N_FEAT][32];
    float l[closure::N_FEAT], u[closure::N_FEAT];
    for (int k = 0; k < closure::N_FEAT; ++k) l[k] = 1e30f, u[k] = -1e30f;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (!(W[i] > 0.f)) continue;
        for (int k = 0; k < closure::N_FEAT; ++k) {
            const float v = X[i * tc::NIN + k];
            l[k] = fminf(l[k], v), u[k] = fmaxf(u[k], v);
        }
    }
    for (int k = 0; k < closure::N_FEAT; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            l[k] = fminf(l[k], __shfl_xor_sync(0xffffffffu, l[k], o));
            u[k] = fmaxf(u[k], __shfl_xor_sync(0xffffffffu, u[k], o));
        }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < closure::N_FEAT; ++k) lo[k][w] = l[k], hi[k][w] = u[k];
    __syncthreads();
    if (threadIdx.x < closure::N_FEAT) {
        float a = 1e30f, b = -1e30f;
        for (int j = 0; j < (int)(blockDim.x >> 5); ++j) a = fminf(a, lo[threadIdx.x][j]), b = fmaxf(b, hi[threadIdx.x][j]);
        out[blockIdx.x * 2 * closure::N_FEAT + threadIdx.x] = a;
        out[blockIdx.x * 2 * closure::N_FEAT + closure::N_FEAT + threadIdx.x] = b;
    }
}

__device__ inline void add_sq(double &acc, const double a[9], const double b[9]) {
    for (int k = 0; k < 9; ++k) acc += (a[k] - b[k]) * (a[k] - b[k]);
}

// Errors of the learned and plain fp32 closures against the fp64 return map
// on the trial F of every snow/sand particle of a state.  One CTA = 128
// particles per tile, the network evaluated as in the particle kernel.
__global__ void __launch_bounds__(128) k_closure_eval(ParticleArrays s, const Material *mats, uint64_t n, float dt,
                                                      const uint8_t *img, const closure::Hull *hull_g, int use_learned,
                                                      double *sums, uint32_t *err) {
    __shared__ __align__(16) uint8_t s_img[tc::IMG_BYTES];
    __shared__ __align__(1024) uint8_t s_a0[128 * tc::NIN * 2];
    __shared__ __align__(1024) uint8_t s_a1[128 * tc::NH * 2];
    __shared__ closure::Hull hull;
    __shared__ mlp::Ctl ctl;
    for (int t = threadIdx.x * 16; t < tc::IMG_BYTES; t += 128 * 16)
        *reinterpret_cast<uint4 *>(s_img + t) = *reinterpret_cast<const uint4 *>(img + t);
    for (int t = threadIdx.x; t < 2 * tc::NIN; t += 128) (&hull.lo[0])[t] = (&hull_g->lo[0])[t];
    mlp::ctl_init(ctl, mlp::TMEM_COLS_INFER);
    mlp::Phase ph;
    double acc[EVAL_SUMS] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint64_t tiles = (n + 127) / 128;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t i = tile * 128 + threadIdx.x;
        bool work = false;
        Material m;
        m3f F;
        float jp = 1.f;
        if (i < n) {
            const uint32_t packed = __float_as_uint(s.pos[i].w);
            if (!(packed & (SV_TOMBSTONED | SV_FAILED))) {
                m = mats[packed >> MATERIAL_SHIFT];
                if (closure::applies(m.kind)) {
                    work = true;
                    trial_f(s, n, i, dt, F);
                    if (m.kind == KIND_SNOW) jp = s.vel[i].w;
                }
            }
        }
        float x[tc::NIN], sig[3], V[9], y[tc::NOUT];
        bool want = false;
        if (work && use_learned) want = closure::learned_features(m, F, hull, sig, V, x);
        if (!want)
            for (int k = 0; k < tc::NIN; ++k) x[k] = 0.f;
        bool net_ok = false;
        if (__syncthreads_or(want) && !ctl.abort) net_ok = mlp::infer_tile(ctl, ph, s_img, s_a0, s_a1, x, y);
        if (!work) continue;
        // fp64 reference: SVD + return map
        double tau_ref[9], f_ref[9];
        {
            m3d Fd, U, Vd;
            double S[3], sd[3], tau[3], jpo;
            for (int k = 0; k < 9; ++k) Fd.a[k] = (double)F.a[k];
            svd3<double>(Fd, U, S, Vd, 12);
            closure::return_map<double>(m, S, sd);
            const double h = closure::hardening<double>(m, S, sd, (double)jp, jpo);
            closure::kirchhoff<double>(m, sd, h, tau);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    double t = 0, f = 0;
                    for (int k = 0; k < 3; ++k) {
                        t += U.a[k * 3 + r] * tau[k] * U.a[k * 3 + c];
                        f += U.a[k * 3 + r] * sd[k] * Vd.a[k * 3 + c];
                    }
                    tau_ref[c * 3 + r] = t, f_ref[c * 3 + r] = f;
                }
        }
        // plain fp32 path as the particle kernel runs it
        double tau_32[9], f_32[9];
        {
            m3f U, Vf;
            float S[3], sf[3], tau[3], jpo;
            uint32_t dummy = 0;
            particle_svd(F, U, S, Vf, 1, dummy);
            closure::return_map<float>(m, S, sf);
            const float h = closure::hardening<float>(m, S, sf, jp, jpo);
            closure::kirchhoff<float>(m, sf, h, tau);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    float t = 0, f = 0;
                    for (int k = 0; k < 3; ++k) {
                        t += U.a[k * 3 + r] * tau[k] * U.a[k * 3 + c];
                        f += U.a[k * 3 + r] * sf[k] * Vf.a[k * 3 + c];
                    }
                    tau_32[c * 3 + r] = t, f_32[c * 3 + r] = f;
                }
        }
        double tau_l[9], f_l[9];
        bool used = false;
        if (want && net_ok) {
            m3f Fn, tt;
            float e_l, jp_l, J_l;
            if (closure::learned_apply(m, F, sig, V, y, jp, Fn, tt, e_l, jp_l, J_l)) {
                used = true;
                for (int k = 0; k < 9; ++k) tau_l[k] = tt.a[k], f_l[k] = Fn.a[k];
            }
        }
        if (!used)
            for (int k = 0; k < 9; ++k) tau_l[k] = tau_32[k], f_l[k] = f_32[k];
        add_sq(acc[0], tau_l, tau_ref);
        add_sq(acc[1], tau_32, tau_ref);
        const double zero[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        add_sq(acc[2], tau_ref, zero);
        add_sq(acc[3], f_l, f_ref);
        add_sq(acc[4], f_32, f_ref);
        add_sq(acc[5], f_ref, zero);
        acc[6] += 1.0;
        acc[7] += used ? 0.0 : 1.0;
    }
    for (int k = 0; k < EVAL_SUMS; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&sums[k], v);
    }
    mlp::ctl_finish(ctl, mlp::TMEM_COLS_INFER, err);
}

template <class T> cudaError_t grow(T **p, uint64_t &cap, uint64_t need, size_t per) {
    if (need <= cap && *p) return cudaSuccess;
    T *q = nullptr;
    cudaError_t e = cudaMalloc((void **)&q, std::max<uint64_t>(need, 1) * per * sizeof(T));
    if (e != cudaSuccess) return e;
    if (*p && cap) cudaMemcpy(q, *p, cap * per * sizeof(T), cudaMemcpyDeviceToDevice);
    cudaFree(*p);
    *p = q;
    cap = need;
    return cudaSuccess;
}

int fail(const std::string &m) {
    set_last_error(m);
    return -1;
}

#define CL_CUDA(expr)                                                                             \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) return fail(std::string("closure: ") + #expr + ": " + cudaGetErrorString(e_)); \
    } while (0)

int ensure_net(sv_handle *h, uint32_t seed) {
    if (h->cl_params) return 0;
    const int P = tc::N_PARAMS;
    CL_CUDA(cudaMalloc(&h->cl_params, P * 4));
    CL_CUDA(cudaMalloc(&h->cl_grad, P * 4));
    CL_CUDA(cudaMalloc(&h->cl_m, P * 4));
    CL_CUDA(cudaMalloc(&h->cl_v, P * 4));
    CL_CUDA(cudaMalloc(&h->cl_img, tc::IMG_BYTES));
    CL_CUDA(cudaMalloc(&h->cl_hull, sizeof(closure::Hull)));
    CL_CUDA(cudaMalloc(&h->cl_loss, 4));
    CL_CUDA(cudaMalloc(&h->cl_err, 4));
    CL_CUDA(cudaMalloc(&h->cl_sums, EVAL_SUMS * sizeof(double)));
    // He initialisation for the ReLU layers, a smaller output layer, zero biases
    std::mt19937_64 rng(seed);
    std::vector<float> p(P, 0.f);
    auto fill = [&](int off, int rows, int cols, double sd) {
        std::normal_distribution<double> nd(0.0, sd);
        for (int k = 0; k < rows * cols; ++k) p[off + k] = (float)nd(rng);
    };
    fill(tc::P_W1, tc::NH, tc::NIN, std::sqrt(2.0 / closure::N_FEAT));
    fill(tc::P_W2, tc::NH, tc::NH, std::sqrt(2.0 / tc::NH));
    fill(tc::P_W3, tc::NOUT, tc::NH, 0.5 * std::sqrt(1.0 / tc::NH));
    CL_CUDA(cudaMemcpy(h->cl_params, p.data(), P * 4, cudaMemcpyHostToDevice));
    CL_CUDA(cudaMemset(h->cl_grad, 0, P * 4));
    CL_CUDA(cudaMemset(h->cl_m, 0, P * 4));
    CL_CUDA(cudaMemset(h->cl_v, 0, P * 4));
    CL_CUDA(cudaMemset(h->cl_err, 0, 4));
    CL_CUDA(mlp::pack_image(h->cl_params, h->cl_img, h->stream));
    h->cl_step = 0;
    return 0;
}

}  // namespace

void free_closure(sv_handle *h) {
    cudaFree(h->cl_params), cudaFree(h->cl_grad), cudaFree(h->cl_m), cudaFree(h->cl_v), cudaFree(h->cl_img);
    cudaFree(h->cl_hull), cudaFree(h->cl_samples), cudaFree(h->cl_X), cudaFree(h->cl_Y), cudaFree(h->cl_W);
    cudaFree(h->cl_loss), cudaFree(h->cl_err), cudaFree(h->cl_count), cudaFree(h->cl_sums);
}

}  // namespace sv

using namespace sv;

extern "C" int sv_closure_harvest(sv_handle *h, float dt, uint32_t max_samples, float augment, uint32_t seed,
                                  uint64_t *total_out) {
    if (!h) return fail("sv_closure_harvest: NULL handle");
    if (!(dt > 0.f)) return fail("sv_closure_harvest: dt must be positive");
    if (!(augment >= 0.f && augment < 0.5f)) return fail("sv_closure_harvest: augment must be in [0, 0.5)");
    if (!h->cl_count) CL_CUDA(cudaMalloc(&h->cl_count, sizeof(uint64_t)));
    const uint64_t room = CL_MAX_SAMPLES - std::min(CL_MAX_SAMPLES, h->cl_n);
    const uint64_t want = std::min<uint64_t>(max_samples, room);
    if (want > 0 && h->n > 0) {
        CL_CUDA(grow(&h->cl_samples, h->cl_cap, h->cl_n + want, CL_SAMPLE));
        const double keep = std::min(1.0, (double)want / (double)h->n);
        const uint32_t threshold = keep >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(keep * 4294967295.0);
        CL_CUDA(cudaMemsetAsync(h->cl_count, 0, sizeof(uint64_t), h->stream));
        const unsigned blocks = (unsigned)std::min<uint64_t>((h->n + 255) / 256, (uint64_t)sm_count() * 8);
        k_harvest<<<blocks, 256, 0, h->stream>>>(h->side[h->cur], h->materials, h->n, dt, threshold, seed, augment,
                                                 h->cl_samples + h->cl_n * CL_SAMPLE, h->cl_count, want);
        CL_CUDA(cudaGetLastError());
        uint64_t got = 0;
        CL_CUDA(cudaMemcpyAsync(&got, h->cl_count, sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
        CL_CUDA(cudaStreamSynchronize(h->stream));
        h->cl_n += std::min(got, want);
    }
    if (total_out) *total_out = h->cl_n;
    return 0;
}

extern "C" int sv_closure_train(sv_handle *h, uint32_t iterations, uint32_t batch, float lr, uint32_t seed,
                                float *loss_out) {
    if (!h) return fail("sv_closure_train: NULL handle");
    if (h->cl_n < 128) return fail("sv_closure_train: fewer than 128 harvested samples");
    if (!(lr > 0.f)) return fail("sv_closure_train: lr must be positive");
    if (ensure_net(h, seed)) return -1;
    const uint64_t n = h->cl_n;
    CL_CUDA(grow(&h->cl_X, h->cl_xy_cap, n, tc::NIN));
    {
        uint64_t cap = 0;
        CL_CUDA(grow(&h->cl_Y, cap, n, tc::NOUT));
        cap = 0;
        cudaFree(h->cl_W);
        h->cl_W = nullptr;
        CL_CUDA(grow(&h->cl_W, cap, n, 1));
    }
    // labels in a shuffled order, so contiguous minibatches are random
    std::vector<uint32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0u);
    std::mt19937_64 rng(seed * 7919ull + 17);
    std::shuffle(perm.begin(), perm.end(), rng);
    uint32_t *dperm = nullptr;
    CL_CUDA(cudaMalloc(&dperm, n * 4));
    cudaError_t e = cudaMemcpy(dperm, perm.data(), n * 4, cudaMemcpyHostToDevice);
    const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count() * 8);
    if (e == cudaSuccess) {
        k_label<<<blocks, 256, 0, h->stream>>>(h->cl_samples, n, h->materials, dperm, h->cl_X, h->cl_Y, h->cl_W);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(dperm);
    CL_CUDA(e);
    // feature hull: the range seen in training, widened a little
    {
        float *dr = nullptr;
        CL_CUDA(cudaMalloc(&dr, (size_t)blocks * 2 * closure::N_FEAT * 4));
        k_feature_range<<<blocks, 256, 0, h->stream>>>(h->cl_X, h->cl_W, n, dr);
        std::vector<float> r((size_t)blocks * 2 * closure::N_FEAT);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(r.data(), dr, r.size() * 4, cudaMemcpyDeviceToHost);
        cudaFree(dr);
        CL_CUDA(e);
        closure::Hull hull;
        for (int k = 0; k < tc::NIN; ++k) hull.lo[k] = 0.f, hull.hi[k] = 0.f;
        for (int k = 0; k < closure::N_FEAT; ++k) {
            float a = 1e30f, b = -1e30f;
            for (unsigned j = 0; j < blocks; ++j)
                a = std::min(a, r[j * 2 * closure::N_FEAT + k]), b = std::max(b, r[j * 2 * closure::N_FEAT + closure::N_FEAT + k]);
            const float pad = 0.02f * (b - a) + 1e-3f;
            hull.lo[k] = a - pad, hull.hi[k] = b + pad;
        }
        CL_CUDA(cudaMemcpy(h->cl_hull, &hull, sizeof(hull), cudaMemcpyHostToDevice));
    }
    // minibatch Adam with a cosine learning-rate decay to 1 %
    uint32_t b = std::max<uint32_t>(128, std::min<uint64_t>(batch ? batch : 8192, n) / 128 * 128);
    std::uniform_int_distribution<uint64_t> pick(0, n - b);
    for (uint32_t it = 0; it < iterations; ++it) {
        const uint64_t off = pick(rng);
        const double c = 0.5 * (1.0 + std::cos(M_PI * (double)it / std::max<uint32_t>(1, iterations)));
        const float lr_it = (float)(lr * (0.01 + 0.99 * c));
        CL_CUDA(cudaMemsetAsync(h->cl_loss, 0, 4, h->stream));
        CL_CUDA(mlp::grad(h->cl_img, h->cl_X + off * tc::NIN, h->cl_Y + off * tc::NOUT, h->cl_W + off, b, h->cl_grad,
                          h->cl_loss, nullptr, h->cl_err, h->stream));
        CL_CUDA(mlp::adam(h->cl_params, h->cl_grad, h->cl_m, h->cl_v, h->cl_img, lr_it, ++h->cl_step, h->stream));
    }
    // loss over the whole pool
    CL_CUDA(cudaMemsetAsync(h->cl_loss, 0, 4, h->stream));
    CL_CUDA(mlp::grad(h->cl_img, h->cl_X, h->cl_Y, h->cl_W, n, h->cl_grad, h->cl_loss, nullptr, h->cl_err, h->stream));
    CL_CUDA(cudaMemsetAsync(h->cl_grad, 0, tc::N_PARAMS * 4, h->stream));
    float loss = 0.f;
    uint32_t err = 0;
    CL_CUDA(cudaMemcpyAsync(&loss, h->cl_loss, 4, cudaMemcpyDeviceToHost, h->stream));
    CL_CUDA(cudaMemcpyAsync(&err, h->cl_err, 4, cudaMemcpyDeviceToHost, h->stream));
    CL_CUDA(cudaStreamSynchronize(h->stream));
    if (err) return fail("sv_closure_train: a tensor-core wait timed out");
    h->cl_trained = true;
    if (loss_out) *loss_out = loss;
    return 0;
}

namespace sv {
namespace {
// The learned closure's bounded tensor-core wait made to run out: one CTA
// sets up the closure's per-CTA control (TMEM columns and the MMA-completion
// mbarrier), waits at most `max_cycles` for an MMA commit that is never
// issued, and ends like a particle pass whose wait gave up (ctl_finish: a
// second bounded wait, the TMEM freed, C_CLOSURE_ERR raised).
__global__ void __launch_bounds__(128) k_closure_wait_timeout(uint32_t *counters, long long max_cycles) {
    __shared__ mlp::Ctl ctl;
    mlp::ctl_init(ctl, mlp::TMEM_COLS_INFER);
    if (threadIdx.x == 0 && !tc::mbar_wait(&ctl.bar, 0, max_cycles)) ctl.abort = 1, ctl.fail_parity = 0;
    mlp::ctl_finish(ctl, mlp::TMEM_COLS_INFER, &counters[C_CLOSURE_ERR], max_cycles);
}
}  // namespace
}  // namespace sv

extern "C" int sv_debug_closure_wait_timeout(sv_handle *h, uint64_t max_cycles) {
    using namespace sv;
    if (!h) return fail("sv_debug_closure_wait_timeout: NULL handle");
    if (max_cycles == 0 || max_cycles > 4000000000ull)
        return fail("sv_debug_closure_wait_timeout: max_cycles must be in [1, 4e9]");
    k_closure_wait_timeout<<<1, 128, 0, h->stream>>>(h->counters, (long long)max_cycles);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(std::string("sv_debug_closure_wait_timeout: ") + cudaGetErrorString(e));
    return 0;
}

extern "C" int sv_closure_set_mode(sv_handle *h, int mode) {
    if (!h) return fail("sv_closure_set_mode: NULL handle");
    if (mode != 0 && mode != 1) return fail("sv_closure_set_mode: mode must be 0 or 1");
    if (mode == 1 && !h->cl_trained) return fail("sv_closure_set_mode: the closure has not been trained");
    if (mode == 1 && h->deterministic) return fail("sv_closure_set_mode: not with the deterministic P2G mode");
    if (mode != h->closure_mode) {
        CL_CUDA(cudaStreamSynchronize(h->stream));
        drop_graphs(h);
    }
    h->closure_mode = mode;
    return 0;
}

extern "C" int sv_closure_evaluate(sv_handle *h, float dt, double out[8]) {
    if (!h || !out) return fail("sv_closure_evaluate: NULL argument");
    if (!h->cl_trained) return fail("sv_closure_evaluate: the closure has not been trained");
    CL_CUDA(cudaMemsetAsync(h->cl_sums, 0, EVAL_SUMS * sizeof(double), h->stream));
    CL_CUDA(cudaMemsetAsync(h->cl_err, 0, 4, h->stream));
    const uint64_t tiles = (h->n + 127) / 128;
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)sm_count() * 4));
    k_closure_eval<<<blocks, 128, 0, h->stream>>>(h->side[h->cur], h->materials, h->n, dt, h->cl_img,
                                                  reinterpret_cast<const closure::Hull *>(h->cl_hull), 1, h->cl_sums,
                                                  h->cl_err);
    CL_CUDA(cudaGetLastError());
    double s[EVAL_SUMS];
    uint32_t err = 0;
    CL_CUDA(cudaMemcpyAsync(s, h->cl_sums, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
    CL_CUDA(cudaMemcpyAsync(&err, h->cl_err, 4, cudaMemcpyDeviceToHost, h->stream));
    CL_CUDA(cudaStreamSynchronize(h->stream));
    if (err) return fail("sv_closure_evaluate: a tensor-core wait timed out");
    const double tr = std::sqrt(std::max(s[2], 1e-300)), fr = std::sqrt(std::max(s[5], 1e-300));
    out[0] = std::sqrt(s[0]) / tr;  // learned (with fallbacks): relative Kirchhoff stress error
    out[1] = std::sqrt(s[1]) / tr;  // plain fp32 return map: relative Kirchhoff stress error
    out[2] = std::sqrt(s[3]) / fr;  // learned: relative projected-F error
    out[3] = std::sqrt(s[4]) / fr;  // plain fp32: relative projected-F error
    out[4] = s[6];                  // snow/sand particles evaluated
    out[5] = s[7];                  // of which fell back to the return map
    out[6] = tr;                    // |tau_ref| (Frobenius over all particles)
    out[7] = fr;                    // |F_ref|
    return 0;
}

extern "C" int sv_closure_get_params(sv_handle *h, float *params) {
    if (!h || !params) return fail("sv_closure_get_params: NULL argument");
    if (!h->cl_params) return fail("sv_closure_get_params: the closure has not been trained");
    CL_CUDA(cudaStreamSynchronize(h->stream));
    CL_CUDA(cudaMemcpy(params, h->cl_params, tc::N_PARAMS * 4, cudaMemcpyDeviceToHost));
    return 0;
}
