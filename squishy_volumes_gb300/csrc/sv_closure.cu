// sv_closure.cu -- the learned stress closure's data, training and error
// evaluation (the closure itself runs inside the particle kernel):
//
//   sv_closure_harvest  trial deformation gradients F + dt C F of the snow
//                       and sand particles of the handle's current state --
//                       states the plain solver produced -- into a pool,
//                       optionally widened by a random symmetric stretch;
//   sv_closure_train    labels the pool with the fp64 SVD + return map (the
//                       yielding samples carry weight), records the feature
//                       hull and the normalisation of inputs and outputs,
//                       trains the MLP on the GPU (tcgen05 forward/backward
//                       kernels, Adam);
//   sv_closure_copy     hands a trained network to another handle;
//   sv_closure_set_mode switches sv_step between the return maps and the
//                       learned closure;
//   sv_closure_evaluate stress and projected-F errors of both paths against
//                       the fp64 return map on the current state;
//   sv_closure_phase_times  the per-phase costs of both paths.
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

// A pool sample carries its material's parameters, so that a pool may
// gather samples from several handles: trial F (9), plastic J, kind bits,
// mu, lambda, alpha, theta_c, theta_s, xi.
constexpr int CL_SAMPLE = 16;
constexpr uint64_t CL_MAX_SAMPLES = 1ull << 26;
constexpr int EVAL_SUMS = 12;

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
        o[10] = __uint_as_float(m.kind);
        o[11] = m.mu, o[12] = m.lambda, o[13] = m.alpha, o[14] = m.theta_c, o[15] = m.theta_s;
    }
}

// Material ranges the labels draw from (sv_closure_set_material_ranges);
// on = 0: every sample keeps the material it was harvested with.
struct MatRanges {
    int on;
    float nu_lo, nu_hi, phi_lo, phi_hi;  // Poisson's ratio, friction angle (radians)
};

// Raw features and targets of each sample, written at position perm[i];
// weight 1 for the samples that yield (the only ones the network sees).
// With material ranges, a sample keeps its harvested deformation and shear
// modulus but takes a Poisson's ratio (lambda = 2 mu nu / (1 - 2 nu)) and,
// for sand, a friction angle (alpha = sqrt(2/3) 2 sin phi / (3 - sin phi))
// drawn uniformly from the ranges by a hash of its index.
__global__ void k_label(const float *samples, uint64_t n, const uint32_t *perm, float *X,
                        float *Y, float *W, MatRanges mr, uint32_t seed) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float *smp = samples + i * CL_SAMPLE;
        Material m{};
        m.kind = __float_as_uint(smp[10]);
        m.mu = smp[11], m.lambda = smp[12], m.alpha = smp[13], m.theta_c = smp[14], m.theta_s = smp[15];
        m.xi = 0.f;  // the targets do not depend on the hardening
        if (mr.on) {
            const uint32_t h1 = hash32((uint32_t)i ^ hash32(seed ^ 0x51ed270bu)), h2 = hash32(h1 ^ 0x2545f491u);
            const double u1 = (double)(h1 >> 8) / 16777216.0, u2 = (double)(h2 >> 8) / 16777216.0;
            const double nu = mr.nu_lo + (mr.nu_hi - mr.nu_lo) * u1;
            m.lambda = (float)(2.0 * (double)m.mu * nu / (1.0 - 2.0 * nu));
            if (m.kind == KIND_SAND) {
                const double sp = sin(mr.phi_lo + (mr.phi_hi - mr.phi_lo) * u2);
                m.alpha = (float)(sqrt(2.0 / 3.0) * 2.0 * sp / (3.0 - sp));
            }
        }
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
        const bool valid = S[2] > 1e-6 && det3(Fd) > 0.0 && m.mu > 0.f && closure::yields<double>(m, S);
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

// Sums of the weighted samples' targets and their squares (the output
// normalisation), and the count of weighted samples.
__global__ void k_target_moments(const float *Y, const float *W, uint64_t n, double *out) {
    double a[2 * tc::N_USED_OUT + 1] = {};
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (W && !(W[i] > 0.f)) continue;
        for (int k = 0; k < tc::N_USED_OUT; ++k) {
            const double v = Y[i * tc::NOUT + k];
            a[k] += v, a[tc::N_USED_OUT + k] += v * v;
        }
        a[2 * tc::N_USED_OUT] += 1.0;
    }
    for (int k = 0; k < 2 * tc::N_USED_OUT + 1; ++k) {
        double v = a[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&out[k], v);
    }
}

// Raw features and targets to the network's normalised ones, in place.
__global__ void k_normalize(float *X, float *Y, uint64_t n, const closure::Hull *hull) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        for (int k = 0; k < tc::NIN; ++k)
            X[i * tc::NIN + k] = k < closure::N_FEAT ? (X[i * tc::NIN + k] - hull->xm[k]) * hull->xs[k] : 0.f;
        for (int k = 0; k < tc::NOUT; ++k)
            Y[i * tc::NOUT + k] = k < tc::N_USED_OUT ? (Y[i * tc::NOUT + k] - hull->ym[k]) / hull->ys[k] : 0.f;
    }
}

// Per-block min / max of the informative features over valid samples.
__global__ void k_feature_range(const float *X, const float *W, uint64_t n, float *out) {
    __shared__ float lo[closure::N_FEAT][32], hi[closure::N_FEAT][32];
    float l[closure::N_FEAT], u[closure::N_FEAT];
    for (int k = 0; k < closure::N_FEAT; ++k) l[k] = 1e30f, u[k] = -1e30f;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (W && !(W[i] > 0.f)) continue;
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

// Stable compaction of the weighted samples: block g takes the contiguous
// range [g chunk, (g + 1) chunk), counts them, then writes them in order at
// its offset (an exclusive scan of the counts).
__global__ void k_compact_count(const float *W, uint64_t n, uint64_t chunk, uint64_t *cnt) {
    __shared__ uint32_t part[8];
    const uint64_t lo = (uint64_t)blockIdx.x * chunk, hi = std::min<uint64_t>(n, lo + chunk);
    uint32_t c = 0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) c += W[i] > 0.f ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        cnt[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(256) k_compact_write(const float *X, const float *Y, const float *W, uint64_t n,
                                                       uint64_t chunk, const uint64_t *off, float *Xo, float *Yo) {
    __shared__ uint32_t wc[8];
    __shared__ uint64_t base;
    const uint64_t lo = (uint64_t)blockIdx.x * chunk, hi = std::min<uint64_t>(n, lo + chunk);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) base = off[blockIdx.x];
    __syncthreads();
    for (uint64_t i0 = lo; i0 < hi; i0 += 256) {
        const uint64_t i = i0 + threadIdx.x;
        const bool f = i < hi && W[i] > 0.f;
        const uint32_t ball = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wc[w] = __popc(ball);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int k = 0; k < 8; ++k) before += k < w ? wc[k] : 0u, total += wc[k];
        if (f) {
            const uint64_t d = base + before + __popc(ball & ((1u << lane) - 1u));
            for (int k = 0; k < tc::NIN; ++k) Xo[d * tc::NIN + k] = X[i * tc::NIN + k];
            for (int k = 0; k < tc::NOUT; ++k) Yo[d * tc::NOUT + k] = Y[i * tc::NOUT + k];
        }
        __syncthreads();
        if (threadIdx.x == 0) base += total;
        __syncthreads();
    }
}

__device__ inline void add_sq(double &acc, const double a[9], const double b[9]) {
    for (int k = 0; k < 9; ++k) acc += (a[k] - b[k]) * (a[k] - b[k]);
}

// Errors of the learned and plain fp32 closures against the fp64 return map
// on the trial F of every snow/sand particle of a state.  One CTA = 128
// particles per tile, the network evaluated as in the particle kernel.
// Dynamic shared memory: the forward image, then the two operand buffers.
constexpr int EV_A0 = tc::IMG_FWD_BYTES;
constexpr int EV_A1 = EV_A0 + 128 * tc::NIN * 2;
constexpr int EV_BYTES = EV_A1 + 128 * tc::NH * 2;

__global__ void __launch_bounds__(128) k_closure_eval(ParticleArrays s, const Material *mats, uint64_t n, float dt,
                                                      const uint8_t *img, const closure::Hull *hull_g, double *sums,
                                                      uint32_t *err) {
    extern __shared__ __align__(1024) uint8_t ev_sm[];
    __shared__ closure::Hull hull;
    __shared__ mlp::Ctl ctl;
    for (int t = threadIdx.x * 16; t < tc::IMG_FWD_BYTES; t += 128 * 16)
        *reinterpret_cast<uint4 *>(ev_sm + t) = *reinterpret_cast<const uint4 *>(img + t);
    for (int t = threadIdx.x; t < (int)(sizeof(closure::Hull) / 4); t += 128)
        reinterpret_cast<float *>(&hull)[t] = reinterpret_cast<const float *>(hull_g)[t];
    mlp::ctl_init(ctl, mlp::TMEM_COLS_INFER);
    mlp::Phase ph;
    double acc[EVAL_SUMS] = {};
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
        int cls = closure::L_PLAIN;
        if (work) cls = closure::learned_features(m, F, hull, sig, V, x);
        const bool want = cls == closure::L_NET;
        if (!want)
            for (int k = 0; k < tc::NIN; ++k) x[k] = 0.f;
        if (__syncthreads_or(want)) {
            bool ok = false;
            if (!ctl.abort) ok = mlp::infer_tile(ctl, ph, ev_sm, ev_sm + EV_A0, ev_sm + EV_A1, x, y);
            if (want && !ok) cls = closure::L_PLAIN;
        }
        if (want) acc[8] += 1.0;
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
        if (cls != closure::L_PLAIN) {
            m3f Fn, tt;
            float e_l, jp_l, J_l;
            if (closure::learned_apply(m, F, sig, V, cls == closure::L_NET ? y : nullptr, hull, jp, Fn, tt, e_l, jp_l,
                                       J_l)) {
                used = true;
                for (int k = 0; k < 9; ++k) tau_l[k] = tt.a[k], f_l[k] = Fn.a[k];
            }
        }
        if (!used)
            for (int k = 0; k < 9; ++k) tau_l[k] = tau_32[k], f_l[k] = f_32[k];
        add_sq(acc[0], tau_l, tau_ref);
        if (used) add_sq(acc[cls == closure::L_NET ? 10 : 11], tau_l, tau_ref);
        add_sq(acc[1], tau_32, tau_ref);
        const double zero[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        add_sq(acc[2], tau_ref, zero);
        add_sq(acc[3], f_l, f_ref);
        add_sq(acc[4], f_32, f_ref);
        add_sq(acc[5], f_ref, zero);
        acc[6] += 1.0;
        acc[7] += used ? 0.0 : 1.0;
        acc[9] += (want && !used) ? 1.0 : 0.0;
    }
    for (int k = 0; k < EVAL_SUMS; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&sums[k], v);
    }
    mlp::ctl_finish(ctl, mlp::TMEM_COLS_INFER, err);
}

// Per-phase costs of the two constitutive paths on the trial F of the snow
// and sand particles of a state, one thread per particle; each thread
// writes one checksum so that none of the work can be dropped.
//   CLOSED = false: the plain path -- fp32 SVD (with its fp64 redo policy),
//                   return map, hardening, Kirchhoff stress tensor and the
//                   projected F;
//   CLOSED = true:  the learned path without the network -- eigen-
//                   decomposition of F^T F, yield test, features, then the
//                   closed-form stress and projected F of the stretches.
template <bool CLOSED>
__global__ void __launch_bounds__(256) k_phase(ParticleArrays s, const Material *mats, uint64_t n, float dt,
                                               const closure::Hull *hull, float *out, unsigned long long *n_net) {
    uint32_t nets = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t packed = __float_as_uint(s.pos[i].w);
        if (packed & (SV_TOMBSTONED | SV_FAILED)) continue;
        const Material m = mats[packed >> MATERIAL_SHIFT];
        if (!closure::applies(m.kind)) continue;
        m3f F;
        trial_f(s, n, i, dt, F);
        const float jp = m.kind == KIND_SNOW ? s.vel[i].w : 1.f;
        float sum = 0.f;
        if constexpr (CLOSED) {
            float x[tc::NIN], sig[3], V[9];
            const int cls = closure::learned_features(m, F, *hull, sig, V, x);
            nets += cls == closure::L_NET ? 1u : 0u;
            m3f Fn, tt;
            float e_l, jp_l, J_l;
            closure::learned_apply(m, F, sig, V, nullptr, *hull, jp, Fn, tt, e_l, jp_l, J_l);
            for (int k = 0; k < 9; ++k) sum += Fn.a[k] + tt.a[k];
            sum += x[0];
        } else {
            m3f U, V;
            float S[3], sf[3], tau[3], jpo;
            uint32_t fp64 = 0;
            particle_svd(F, U, S, V, 1, fp64);
            closure::return_map<float>(m, S, sf);
            const float h = closure::hardening<float>(m, S, sf, jp, jpo);
            closure::kirchhoff<float>(m, sf, h, tau);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) {
                    float t = 0.f, f = 0.f;
                    for (int k = 0; k < 3; ++k) {
                        t += U.a[k * 3 + r] * tau[k] * U.a[k * 3 + c];
                        f += U.a[k * 3 + r] * sf[k] * V.a[k * 3 + c];
                    }
                    sum += t + f;
                }
        }
        out[i] = sum;
    }
    if (CLOSED) {
        for (int o = 16; o > 0; o >>= 1) nets += __shfl_xor_sync(0xffffffffu, nets, o);
        if ((threadIdx.x & 31) == 0 && nets) atomicAdd(n_net, (unsigned long long)nets);
    }
}

__global__ void k_count_applies(ParticleArrays s, const Material *mats, uint64_t n, unsigned long long *count) {
    uint32_t c = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t packed = __float_as_uint(s.pos[i].w);
        if (!(packed & (SV_TOMBSTONED | SV_FAILED)) && closure::applies(mats[packed >> MATERIAL_SHIFT].kind)) ++c;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, (unsigned long long)c);
}

// All transfers of this file run on the handle's stream (non-blocking, so
// not ordered with the legacy default stream), synchronised where the host
// reads a result.
template <class T> cudaError_t grow(T **p, uint64_t &cap, uint64_t need, size_t per, cudaStream_t s) {
    if (need <= cap && *p) return cudaSuccess;
    T *q = nullptr;
    cudaError_t e = cudaMalloc((void **)&q, std::max<uint64_t>(need, 1) * per * sizeof(T));
    if (e != cudaSuccess) return e;
    if (*p && cap) {
        e = cudaMemcpyAsync(q, *p, cap * per * sizeof(T), cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            cudaFree(q);
            return e;
        }
    }
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
    // He initialisation of the hidden layers, a smaller head, zero biases
    std::mt19937_64 rng(seed);
    std::vector<float> p(P, 0.f);
    auto fill = [&](int off, int rows, int cols, double sd) {
        std::normal_distribution<double> nd(0.0, sd);
        for (int k = 0; k < rows * cols; ++k) p[off + k] = (float)nd(rng);
    };
    fill(tc::P_W1, tc::NH, tc::NIN, std::sqrt(2.0 / closure::N_FEAT));
    for (int l = 2; l <= tc::N_HIDDEN; ++l) fill(tc::p_weight(l), tc::NH, tc::NH, std::sqrt(2.0 / tc::NH));
    fill(tc::P_W5, tc::NOUT, tc::NH, 0.5 * std::sqrt(1.0 / tc::NH));
    CL_CUDA(cudaMemcpyAsync(h->cl_params, p.data(), P * 4, cudaMemcpyHostToDevice, h->stream));
    CL_CUDA(cudaMemsetAsync(h->cl_grad, 0, P * 4, h->stream));
    CL_CUDA(cudaMemsetAsync(h->cl_m, 0, P * 4, h->stream));
    CL_CUDA(cudaMemsetAsync(h->cl_v, 0, P * 4, h->stream));
    CL_CUDA(cudaMemsetAsync(h->cl_err, 0, 4, h->stream));
    CL_CUDA(mlp::pack_image(h->cl_params, h->cl_img, h->stream));
    h->cl_step = 0;
    return 0;
}

}  // namespace

void free_closure(sv_handle *h) {
    cudaFree(h->cl_params), cudaFree(h->cl_grad), cudaFree(h->cl_m), cudaFree(h->cl_v), cudaFree(h->cl_img);
    cudaFree(h->cl_hull), cudaFree(h->cl_samples), cudaFree(h->cl_X), cudaFree(h->cl_Y);
    cudaFree(h->cl_loss), cudaFree(h->cl_err), cudaFree(h->cl_count), cudaFree(h->cl_sums);
}

}  // namespace sv

using namespace sv;

extern "C" int sv_closure_harvest_from(sv_handle *h, sv_handle *src, float dt, uint32_t max_samples, float augment,
                                       uint32_t seed, uint64_t *total_out) {
    if (!h || !src) return fail("sv_closure_harvest: NULL handle");
    if (!(dt > 0.f)) return fail("sv_closure_harvest: dt must be positive");
    if (!(augment >= 0.f && augment < 0.5f)) return fail("sv_closure_harvest: augment must be in [0, 0.5)");
    if (!h->cl_count) CL_CUDA(cudaMalloc(&h->cl_count, sizeof(uint64_t)));
    const uint64_t room = CL_MAX_SAMPLES - std::min(CL_MAX_SAMPLES, h->cl_n);
    const uint64_t want = std::min<uint64_t>(max_samples, room);
    if (want > 0 && src->n > 0) {
        CL_CUDA(grow(&h->cl_samples, h->cl_cap, h->cl_n + want, CL_SAMPLE, h->stream));
        // the source's state is read on the pool's stream once the source's
        // queued work is done
        if (src != h) CL_CUDA(cudaStreamSynchronize(src->stream));
        const double keep = std::min(1.0, (double)want / (double)src->n);
        const uint32_t threshold = keep >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(keep * 4294967295.0);
        CL_CUDA(cudaMemsetAsync(h->cl_count, 0, sizeof(uint64_t), h->stream));
        const unsigned blocks = (unsigned)std::min<uint64_t>((src->n + 255) / 256, (uint64_t)sm_count() * 8);
        k_harvest<<<blocks, 256, 0, h->stream>>>(src->side[src->cur], src->materials, src->n, dt, threshold, seed,
                                                 augment, h->cl_samples + h->cl_n * CL_SAMPLE, h->cl_count, want);
        CL_CUDA(cudaGetLastError());
        uint64_t got = 0;
        CL_CUDA(cudaMemcpyAsync(&got, h->cl_count, sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
        CL_CUDA(cudaStreamSynchronize(h->stream));
        h->cl_n += std::min(got, want);
    }
    if (total_out) *total_out = h->cl_n;
    return 0;
}

extern "C" int sv_closure_harvest(sv_handle *h, float dt, uint32_t max_samples, float augment, uint32_t seed,
                                  uint64_t *total_out) {
    return sv_closure_harvest_from(h, h, dt, max_samples, augment, seed, total_out);
}

extern "C" int sv_closure_train(sv_handle *h, uint32_t iterations, uint32_t batch, float lr, uint32_t seed,
                                float *loss_out) {
    if (!h) return fail("sv_closure_train: NULL handle");
    if (h->cl_n < 128) return fail("sv_closure_train: fewer than 128 harvested samples");
    if (!(lr > 0.f)) return fail("sv_closure_train: lr must be positive");
    if (ensure_net(h, seed)) return -1;
    const uint64_t n = h->cl_n;
    const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count() * 8);
    // 1. labels of the whole pool, in a shuffled order so that contiguous
    //    minibatches are random
    float *rX = nullptr, *rY = nullptr, *rW = nullptr;
    uint32_t *dperm = nullptr;
    uint64_t *dcnt = nullptr;
    auto release = [&] { cudaFree(rX), cudaFree(rY), cudaFree(rW), cudaFree(dperm), cudaFree(dcnt); };
    cudaError_t e = cudaMalloc(&rX, n * tc::NIN * 4);
    if (e == cudaSuccess) e = cudaMalloc(&rY, n * tc::NOUT * 4);
    if (e == cudaSuccess) e = cudaMalloc(&rW, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dperm, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dcnt, (size_t)blocks * 8);
    std::mt19937_64 rng(seed * 7919ull + 17);
    if (e == cudaSuccess) {
        std::vector<uint32_t> perm(n);
        std::iota(perm.begin(), perm.end(), 0u);
        std::shuffle(perm.begin(), perm.end(), rng);
        e = cudaMemcpyAsync(dperm, perm.data(), n * 4, cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) {
        const MatRanges mr{h->cl_ranges_on, h->cl_ranges[0], h->cl_ranges[1], h->cl_ranges[2], h->cl_ranges[3]};
        k_label<<<blocks, 256, 0, h->stream>>>(h->cl_samples, n, dperm, rX, rY, rW, mr, seed);
        e = cudaGetLastError();
    }
    // 2. the yielding samples, compacted in order
    const uint64_t chunk = (n + blocks - 1) / blocks;
    std::vector<uint64_t> cnt(blocks), off(blocks);
    if (e == cudaSuccess) {
        k_compact_count<<<blocks, 256, 0, h->stream>>>(rW, n, chunk, dcnt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), dcnt, (size_t)blocks * 8, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    uint64_t m = 0;
    for (unsigned g = 0; g < blocks; ++g) off[g] = m, m += cnt[g];
    if (e == cudaSuccess && m < 128) {
        release();
        return fail("sv_closure_train: fewer than 128 yielding samples in the pool");
    }
    if (e == cudaSuccess) e = grow(&h->cl_X, h->cl_xy_cap, m, tc::NIN, h->stream);
    if (e == cudaSuccess) {
        uint64_t cap = 0;
        cudaFree(h->cl_Y);
        h->cl_Y = nullptr;
        e = grow(&h->cl_Y, cap, m, tc::NOUT, h->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(dcnt, off.data(), (size_t)blocks * 8, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        k_compact_write<<<blocks, 256, 0, h->stream>>>(rX, rY, rW, n, chunk, dcnt, h->cl_X, h->cl_Y);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    release();
    CL_CUDA(e);
    h->cl_yielding = m;
    // 3. feature hull: the range of the yielding samples, widened a little;
    //    the inputs mapped to about [-1, 1], the outputs to zero mean and
    //    unit variance
    {
        const unsigned rb = (unsigned)std::min<uint64_t>((m + 255) / 256, (uint64_t)sm_count() * 8);
        float *dr = nullptr;
        double *dm = nullptr;
        const int NM = 2 * tc::N_USED_OUT + 1;
        CL_CUDA(cudaMalloc(&dr, (size_t)rb * 2 * closure::N_FEAT * 4));
        e = cudaMalloc(&dm, NM * sizeof(double));
        if (e == cudaSuccess) e = cudaMemsetAsync(dm, 0, NM * sizeof(double), h->stream);
        if (e == cudaSuccess) {
            k_feature_range<<<rb, 256, 0, h->stream>>>(h->cl_X, nullptr, m, dr);
            k_target_moments<<<rb, 256, 0, h->stream>>>(h->cl_Y, nullptr, m, dm);
            e = cudaGetLastError();
        }
        std::vector<float> r((size_t)rb * 2 * closure::N_FEAT);
        double mom[2 * tc::N_USED_OUT + 1];
        if (e == cudaSuccess) e = cudaMemcpyAsync(r.data(), dr, r.size() * 4, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(mom, dm, sizeof(mom), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        cudaFree(dr);
        cudaFree(dm);
        CL_CUDA(e);
        const double c = mom[2 * tc::N_USED_OUT];
        closure::Hull hull;
        for (int k = 0; k < tc::NIN; ++k) hull.lo[k] = hull.hi[k] = hull.xm[k] = hull.xs[k] = 0.f;
        for (int k = 0; k < tc::NOUT; ++k) hull.ym[k] = 0.f, hull.ys[k] = 1.f;
        for (int k = 0; k < closure::N_FEAT; ++k) {
            float a = 1e30f, b = -1e30f;
            for (unsigned j = 0; j < rb; ++j)
                a = std::min(a, r[j * 2 * closure::N_FEAT + k]), b = std::max(b, r[j * 2 * closure::N_FEAT + closure::N_FEAT + k]);
            const float pad = 0.02f * (b - a) + 1e-4f * std::max(1.f, std::fabs(a) + std::fabs(b));
            hull.lo[k] = a - pad, hull.hi[k] = b + pad;
            hull.xm[k] = 0.5f * (hull.lo[k] + hull.hi[k]);
            hull.xs[k] = 2.f / (hull.hi[k] - hull.lo[k]);
        }
        for (int k = 0; k < tc::N_USED_OUT; ++k) {
            const double mean = mom[k] / c;
            const double var = std::max(0.0, mom[tc::N_USED_OUT + k] / c - mean * mean);
            hull.ym[k] = (float)mean;
            hull.ys[k] = (float)std::max(std::sqrt(var), 1e-6);
        }
        CL_CUDA(cudaMemcpyAsync(h->cl_hull, &hull, sizeof(hull), cudaMemcpyHostToDevice, h->stream));
        k_normalize<<<rb, 256, 0, h->stream>>>(h->cl_X, h->cl_Y, m, reinterpret_cast<const closure::Hull *>(h->cl_hull));
        CL_CUDA(cudaGetLastError());
    }
    // 4. minibatch Adam with a cosine learning-rate decay to 1 %
    const uint32_t b = (uint32_t)std::max<uint64_t>(128, std::min<uint64_t>(batch ? batch : 65536, m) / 128 * 128);
    std::uniform_int_distribution<uint64_t> pick(0, m - b);
    for (uint32_t it = 0; it < iterations; ++it) {
        const uint64_t o = pick(rng);
        const double c = 0.5 * (1.0 + std::cos(M_PI * (double)it / std::max<uint32_t>(1, iterations)));
        const float lr_it = (float)(lr * (0.01 + 0.99 * c));
        CL_CUDA(mlp::grad(h->cl_img, h->cl_X + o * tc::NIN, h->cl_Y + o * tc::NOUT, nullptr, b, h->cl_grad,
                          h->cl_loss, nullptr, h->cl_err, h->stream));
        CL_CUDA(mlp::adam(h->cl_params, h->cl_grad, h->cl_m, h->cl_v, h->cl_img, lr_it, ++h->cl_step, h->stream));
    }
    // loss (normalised units) over the yielding samples
    CL_CUDA(cudaMemsetAsync(h->cl_loss, 0, 4, h->stream));
    CL_CUDA(mlp::grad(h->cl_img, h->cl_X, h->cl_Y, nullptr, m, h->cl_grad, h->cl_loss, nullptr, h->cl_err, h->stream));
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

extern "C" int sv_closure_copy(sv_handle *dst, sv_handle *src) {
    if (!dst || !src) return fail("sv_closure_copy: NULL handle");
    if (!src->cl_trained) return fail("sv_closure_copy: the source closure has not been trained");
    if (dst == src) return 0;
    if (ensure_net(dst, 0)) return -1;
    CL_CUDA(cudaStreamSynchronize(src->stream));
    CL_CUDA(cudaMemcpyAsync(dst->cl_params, src->cl_params, tc::N_PARAMS * 4, cudaMemcpyDeviceToDevice, dst->stream));
    CL_CUDA(cudaMemcpyAsync(dst->cl_m, src->cl_m, tc::N_PARAMS * 4, cudaMemcpyDeviceToDevice, dst->stream));
    CL_CUDA(cudaMemcpyAsync(dst->cl_v, src->cl_v, tc::N_PARAMS * 4, cudaMemcpyDeviceToDevice, dst->stream));
    CL_CUDA(cudaMemcpyAsync(dst->cl_img, src->cl_img, tc::IMG_BYTES, cudaMemcpyDeviceToDevice, dst->stream));
    CL_CUDA(cudaMemcpyAsync(dst->cl_hull, src->cl_hull, sizeof(closure::Hull), cudaMemcpyDeviceToDevice, dst->stream));
    CL_CUDA(cudaStreamSynchronize(dst->stream));
    dst->cl_step = src->cl_step;
    dst->cl_yielding = src->cl_yielding;
    dst->cl_trained = true;
    if (dst->closure_mode == 1) drop_graphs(dst);  // the captured graphs read the old image
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

extern "C" int sv_closure_evaluate(sv_handle *h, float dt, double out[12]) {
    if (!h || !out) return fail("sv_closure_evaluate: NULL argument");
    if (!h->cl_trained) return fail("sv_closure_evaluate: the closure has not been trained");
    CL_CUDA(cudaMemsetAsync(h->cl_sums, 0, EVAL_SUMS * sizeof(double), h->stream));
    CL_CUDA(cudaMemsetAsync(h->cl_err, 0, 4, h->stream));
    const uint64_t tiles = (h->n + 127) / 128;
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles, (uint64_t)sm_count() * 4));
    CL_CUDA(cudaFuncSetAttribute(k_closure_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, EV_BYTES));
    k_closure_eval<<<blocks, 128, EV_BYTES, h->stream>>>(h->side[h->cur], h->materials, h->n, dt, h->cl_img,
                                                         reinterpret_cast<const closure::Hull *>(h->cl_hull), h->cl_sums,
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
    out[8] = s[8];                  // particles handed to the network (yielding, inside the hull)
    out[9] = s[9];                  // of which the residual check sent back to the return map
    out[10] = std::sqrt(s[10]) / tr;  // out[0]'s part from the network's particles
    out[11] = std::sqrt(s[11]) / tr;  // out[0]'s part from the elastic (eigen-decomposition) particles
    return 0;
}

extern "C" int sv_closure_get_params(sv_handle *h, float *params) {
    if (!h || !params) return fail("sv_closure_get_params: NULL argument");
    if (!h->cl_params) return fail("sv_closure_get_params: the closure has not been trained");
    CL_CUDA(cudaStreamSynchronize(h->stream));
    CL_CUDA(cudaMemcpy(params, h->cl_params, tc::N_PARAMS * 4, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int sv_closure_phase_times(sv_handle *h, float dt, double out[6]) {
    if (!h || !out) return fail("sv_closure_phase_times: NULL argument");
    if (!h->cl_trained) return fail("sv_closure_phase_times: the closure has not been trained");
    const uint64_t n = std::max<uint64_t>(h->n, 1);
    float *chk = nullptr, *X = nullptr, *Y = nullptr;
    unsigned long long *cnt = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto release = [&] {
        cudaFree(chk), cudaFree(X), cudaFree(Y), cudaFree(cnt);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e = cudaMalloc(&chk, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&X, n * tc::NIN * 4);
    if (e == cudaSuccess) e = cudaMalloc(&Y, n * tc::NOUT * 4);
    if (e == cudaSuccess) e = cudaMalloc(&cnt, 16);
    if (e == cudaSuccess) e = cudaMemsetAsync(X, 0, n * tc::NIN * 4, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, 16, h->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        release();
        return fail(std::string("sv_closure_phase_times: ") + cudaGetErrorString(e));
    }
    const ParticleArrays st = h->side[h->cur];
    const closure::Hull *hull = reinterpret_cast<const closure::Hull *>(h->cl_hull);
    const unsigned blocks = (unsigned)std::min<uint64_t>((h->n + 255) / 256, (uint64_t)sm_count() * 8);
    const int reps = 5;
    // mean of `reps` launches after one untimed launch
    auto time = [&](auto launch, double &ms) {
        launch();
        cudaEventRecord(e0, h->stream);
        for (int r = 0; r < reps; ++r) launch();
        cudaEventRecord(e1, h->stream);
        e = cudaEventSynchronize(e1);
        float t = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        ms = (double)t / reps;
        return e == cudaSuccess ? cudaGetLastError() : e;
    };
    double t_plain = 0, t_closed = 0, t_net_all = 0, t_net = 0;
    unsigned long long counts[2] = {0, 0};
    if (h->n > 0) {
        k_count_applies<<<blocks, 256, 0, h->stream>>>(st, h->materials, h->n, cnt);
        e = time([&] { k_phase<false><<<blocks, 256, 0, h->stream>>>(st, h->materials, h->n, dt, hull, chk, nullptr); },
                 t_plain);
        if (e == cudaSuccess)
            e = time([&] { k_phase<true><<<blocks, 256, 0, h->stream>>>(st, h->materials, h->n, dt, hull, chk, cnt + 1); },
                     t_closed);
        if (e == cudaSuccess) e = cudaMemcpyAsync(counts, cnt, 16, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        const uint64_t all = counts[0], nets = counts[1] / (reps + 1);
        if (e == cudaSuccess && all)
            e = time([&] { mlp::forward(h->cl_img, X, all, Y, h->cl_err, h->stream); }, t_net_all);
        if (e == cudaSuccess && nets)
            e = time([&] { mlp::forward(h->cl_img, X, nets, Y, h->cl_err, h->stream); }, t_net);
        counts[1] = nets;
    }
    release();
    if (e != cudaSuccess) return fail(std::string("sv_closure_phase_times: ") + cudaGetErrorString(e));
    out[0] = t_plain;            // ms: SVD + return map + stress (plain path)
    out[1] = t_closed;           // ms: eig + yield test + closed-form stress (learned path without the network)
    out[2] = t_net_all;          // ms: the network over every snow/sand particle
    out[3] = (double)counts[0];  // snow/sand particles
    out[4] = (double)counts[1];  // of which yield inside the hull (the network's share)
    out[5] = t_net;              // ms: the network over the yielding ones only
    return 0;
}

extern "C" int sv_closure_pool(sv_handle *h, uint64_t *pairs, uint64_t *yielding) {
    if (!h) return fail("sv_closure_pool: NULL handle");
    if (pairs) *pairs = h->cl_n;
    if (yielding) *yielding = h->cl_yielding;
    return 0;
}

extern "C" int sv_closure_get_pool(sv_handle *h, uint64_t first, uint64_t count, float *X, float *Y, float *hull) {
    if (!h) return fail("sv_closure_get_pool: NULL handle");
    if (!h->cl_params || !h->cl_X) return fail("sv_closure_get_pool: the closure has not been trained");
    if (first + count > h->cl_yielding || first + count < first) return fail("sv_closure_get_pool: rows out of range");
    CL_CUDA(cudaStreamSynchronize(h->stream));
    if (count && X) CL_CUDA(cudaMemcpy(X, h->cl_X + first * tc::NIN, count * tc::NIN * 4, cudaMemcpyDeviceToHost));
    if (count && Y) CL_CUDA(cudaMemcpy(Y, h->cl_Y + first * tc::NOUT, count * tc::NOUT * 4, cudaMemcpyDeviceToHost));
    if (hull) CL_CUDA(cudaMemcpy(hull, h->cl_hull, sizeof(closure::Hull), cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int sv_closure_set_material_ranges(sv_handle *h, float nu_lo, float nu_hi, float phi_lo_deg,
                                              float phi_hi_deg) {
    if (!h) return fail("sv_closure_set_material_ranges: NULL handle");
    if (nu_lo == 0.f && nu_hi == 0.f && phi_lo_deg == 0.f && phi_hi_deg == 0.f) {
        h->cl_ranges_on = 0;
        return 0;
    }
    if (!(nu_lo >= 0.f && nu_lo <= nu_hi && nu_hi < 0.5f))
        return fail("sv_closure_set_material_ranges: need 0 <= nu_lo <= nu_hi < 0.5");
    if (!(phi_lo_deg >= 0.f && phi_lo_deg <= phi_hi_deg && phi_hi_deg < 90.f))
        return fail("sv_closure_set_material_ranges: need 0 <= phi_lo <= phi_hi < 90 degrees");
    h->cl_ranges_on = 1;
    h->cl_ranges[0] = nu_lo, h->cl_ranges[1] = nu_hi;
    h->cl_ranges[2] = phi_lo_deg * (float)(M_PI / 180.0), h->cl_ranges[3] = phi_hi_deg * (float)(M_PI / 180.0);
    return 0;
}
