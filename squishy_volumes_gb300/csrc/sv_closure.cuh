// sv_closure.cuh -- the learned stress closure of snow and Drucker-Prager
// sand particles (an addition; the reference has the return maps only).
//
// Plain path (the reference's and this library's default): SVD of the trial
// F, the return map on its singular values, the stress from the projected
// ones.  Learned path: the principal stretches come from a closed-form
// eigen-decomposition of F^T F (no iteration); the yield test, closed form
// and cheap, sorts the particle:
//   elastic  -- the return map leaves the stretches alone: the Kirchhoff
//               stress of the stretches, no network;
//   yielding -- the network (4 hidden layers of width 64, SiLU, on the
//               tensor cores; fp32 head) maps the principal Hencky strains
//               and the material parameters to the plastic correction of
//               the strains and the principal Kirchhoff stress of the
//               projected state.  The stress applied is the closed-form
//               Kirchhoff stress of the corrected stretches; the network's
//               own stress output is the residual check.
// A yielding particle outside the training hull, or whose residual check
// fails, takes the plain path.
//
// Raw features (the network sees (x - xm) xs, both from the training pool):
//   x0..2 = e_i    principal Hencky strains ln sigma_i, sigma descending
//   x3 = snow, x4 = sand, x5 = lambda / mu,
//   x6 = theta_c, x7 = theta_s (snow), x8 = alpha (sand),
//   x9..11 = the branch of each stretch under the snow limits (-1 below
//            1 - theta_c, +1 above 1 + theta_s, 0 between; 0 for sand),
//   x12 = 1 on sand's expansion / hydrostatic branch (0 otherwise);
//   x13..15 = 0.  The branch features come from the closed-form yield test:
//   with them the network fits a function that is smooth on each branch
//   instead of locating the branches' kinks itself.
// Raw targets (the network predicts (y - ym) / ys):
//   y0..2 = ln s_i - e_i            plastic correction of the strains
//                                   (measured more accurate than predicting
//                                   ln s_i itself: the error then scales
//                                   with the correction, which is small for
//                                   most yielding particles)
//   y3..5 = tau_i / (mu h)          principal Kirchhoff stress of the
//                                   projected state, h the snow hardening
#pragma once
#include "sv_math.cuh"
#include "sv_tc.cuh"

namespace sv {
namespace closure {

constexpr float RES_TOL = 1e-3f;  // |tau_net - tau(s)| / (mu h), max over i
constexpr int N_FEAT = 13;        // features that carry information

// The accepted feature range (lo, hi) and the normalisation of the inputs
// and outputs, all from the training pool.
struct Hull {
    float lo[tc::NIN], hi[tc::NIN];
    float xm[tc::NIN], xs[tc::NIN];
    float ym[tc::NOUT], ys[tc::NOUT];
};

enum LearnedClass { L_PLAIN = 0, L_ELASTIC = 1, L_NET = 2 };

__host__ __device__ inline bool applies(uint32_t kind) { return kind == KIND_SNOW || kind == KIND_SAND; }

__host__ __device__ inline void features(const Material &m, const float e[3], float x[tc::NIN]) {
    for (int k = 0; k < tc::NIN; ++k) x[k] = 0.f;
    x[0] = e[0], x[1] = e[1], x[2] = e[2];
    const bool snow = m.kind == KIND_SNOW;
    x[3] = snow ? 1.f : 0.f;
    x[4] = snow ? 0.f : 1.f;
    x[5] = m.mu > 0.f ? m.lambda / m.mu : 0.f;
    if (snow) {
        x[6] = m.theta_c;
        x[7] = m.theta_s;
        const float lo = logf(1.f - m.theta_c), hi = logf(1.f + m.theta_s);
        for (int k = 0; k < 3; ++k) x[9 + k] = e[k] < lo ? -1.f : (e[k] > hi ? 1.f : 0.f);
    } else {
        x[8] = m.alpha;
        const float e_tr = e[0] + e[1] + e[2];
        float eh2 = 0.f;
        for (int k = 0; k < 3; ++k) eh2 += (e[k] - e_tr / 3.f) * (e[k] - e_tr / 3.f);
        x[12] = (e_tr < 0.f && eh2 > 0.f) ? 0.f : 1.f;
    }
}

// The return maps on the principal stretches (sigma in, s out), as the
// particle kernel applies them to the SVD: snow clamps to
// [1 - theta_c, 1 + theta_s] (Stomakhin et al. 2013); sand follows the
// Drucker-Prager projection in Hencky strain of
// rust/crates/cpu/src/phase/advance_particles.rs:48-71.
template <class T> __host__ __device__ inline void return_map(const Material &m, const T sig[3], T s[3]) {
    if (m.kind == KIND_SNOW) {
        for (int k = 0; k < 3; ++k) {
            const T lo = T(1) - (T)m.theta_c, hi = T(1) + (T)m.theta_s;
            s[k] = sig[k] < lo ? lo : (sig[k] > hi ? hi : sig[k]);
        }
        return;
    }
    for (int k = 0; k < 3; ++k) s[k] = sig[k];
    T e[3];
    for (int k = 0; k < 3; ++k) e[k] = log(sig[k]);
    const T e_tr = e[0] + e[1] + e[2];
    T eh[3];
    for (int k = 0; k < 3; ++k) eh[k] = e[k] - e_tr / T(3);
    const T ehn = sqrt(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]);
    if (e_tr < T(0) && ehn > T(0)) {
        // mu <= 0: the reference asserts mu > 0 (advance_particles.rs:57);
        // such particles never take the learned path
        if (!((T)m.mu > T(0))) return;
        const T dg = ehn + (T(3) * (T)m.lambda + T(2) * (T)m.mu) / T(2) / (T)m.mu * e_tr * (T)m.alpha;
        if (dg > T(0))
            for (int k = 0; k < 3; ++k) s[k] = exp(e[k] - dg / ehn * eh[k]);
    } else {
        s[0] = s[1] = s[2] = T(1);
    }
}

// The closed-form yield test: true when the return map changes the
// stretches (snow: one outside [1 - theta_c, 1 + theta_s]; sand: the
// expansion / hydrostatic branch, or a positive Drucker-Prager yield
// function on the compressive branch).  Needs mu > 0 for sand.
template <class T> __host__ __device__ inline bool yields(const Material &m, const T sig[3]) {
    if (m.kind == KIND_SNOW) {
        const T lo = T(1) - (T)m.theta_c, hi = T(1) + (T)m.theta_s;
        return sig[0] < lo || sig[0] > hi || sig[1] < lo || sig[1] > hi || sig[2] < lo || sig[2] > hi;
    }
    T e[3];
    for (int k = 0; k < 3; ++k) e[k] = log(sig[k]);
    const T e_tr = e[0] + e[1] + e[2];
    T eh[3];
    for (int k = 0; k < 3; ++k) eh[k] = e[k] - e_tr / T(3);
    const T ehn = sqrt(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]);
    if (!(e_tr < T(0) && ehn > T(0))) return !(sig[0] == T(1) && sig[1] == T(1) && sig[2] == T(1));  // s = 1
    const T dg = ehn + (T(3) * (T)m.lambda + T(2) * (T)m.mu) / T(2) / (T)m.mu * e_tr * (T)m.alpha;
    return dg > T(0);
}

// Hardening factor of the projected state and the updated plastic J (snow).
template <class T> __host__ __device__ inline T hardening(const Material &m, const T sig[3], const T s[3], T jp_in, T &jp_out) {
    if (m.kind != KIND_SNOW) {
        jp_out = jp_in;
        return T(1);
    }
    jp_out = jp_in * (sig[0] * sig[1] * sig[2]) / (s[0] * s[1] * s[2]);
    return exp((T)m.xi * (T(1) - jp_out));
}

// Principal Kirchhoff stress of the projected stretches (h folded in):
// snow = fixed-corotated 2 mu h (s^2 - s) + lambda h (J - 1) J,
// sand = Neo-Hookean mu (s^2 - 1) + lambda ln J.
template <class T> __host__ __device__ inline void kirchhoff(const Material &m, const T s[3], T h, T tau[3]) {
    const T J = s[0] * s[1] * s[2];
    if (m.kind == KIND_SNOW) {
        const T mu = (T)m.mu * h, la = (T)m.lambda * h;
        for (int k = 0; k < 3; ++k) tau[k] = T(2) * mu * (s[k] * s[k] - s[k]) + la * (J - T(1)) * J;
    } else {
        const T lj = log(J);
        for (int k = 0; k < 3; ++k) tau[k] = (T)m.mu * (s[k] * s[k] - T(1)) + (T)m.lambda * lj;
    }
}

template <class T> __host__ __device__ inline T energy(const Material &m, const T s[3], T h) {
    const T J = s[0] * s[1] * s[2];
    if (m.kind == KIND_SNOW) {
        const T d2 = (s[0] - T(1)) * (s[0] - T(1)) + (s[1] - T(1)) * (s[1] - T(1)) + (s[2] - T(1)) * (s[2] - T(1));
        return (T)m.mu * h * d2 + (T)m.lambda * h / T(2) * (J - T(1)) * (J - T(1));
    }
    const T lj = log(J);
    return (T)m.mu / T(2) * (s[0] * s[0] + s[1] * s[1] + s[2] * s[2] - T(3)) - (T)m.mu * lj + (T)m.lambda / T(2) * lj * lj;
}

// Raw training targets from the principal stretches (double precision).
__host__ __device__ inline void targets(const Material &m, const double sig[3], double jp, float y[tc::NOUT]) {
    double s[3], tau[3], jp_out;
    return_map<double>(m, sig, s);
    const double h = hardening<double>(m, sig, s, jp, jp_out);
    kirchhoff<double>(m, s, h, tau);
    for (int k = 0; k < tc::NOUT; ++k) y[k] = 0.f;
    const double muh = (double)m.mu * h;
    for (int k = 0; k < 3; ++k) {
        y[k] = (float)(log(s[k]) - log(sig[k]));
        y[3 + k] = muh > 0 ? (float)(tau[k] / muh) : 0.f;
    }
}

// Learned path, part 1: principal stretches of the trial F from the
// closed-form eigen-decomposition of F^T F, the yield test, and the
// normalised features of a yielding particle.  Returns L_PLAIN when the
// particle must take the plain path (degenerate F, mu <= 0, outside the
// hull), L_ELASTIC when the stretches stand, L_NET when the network decides.
__device__ __forceinline__ int learned_features(const Material &m, const m3f &F, const Hull &hull, float sig[3],
                                                float V[9], float x[tc::NIN]) {
    float c[6];  // F^T F: column dot products (column-major F)
    const float *a = F.a;
    c[0] = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    c[1] = a[0] * a[3] + a[1] * a[4] + a[2] * a[5];
    c[2] = a[0] * a[6] + a[1] * a[7] + a[2] * a[8];
    c[3] = a[3] * a[3] + a[4] * a[4] + a[5] * a[5];
    c[4] = a[3] * a[6] + a[4] * a[7] + a[5] * a[8];
    c[5] = a[6] * a[6] + a[7] * a[7] + a[8] * a[8];
    float lam[3];
    sym_eig3(c, lam, V);
    if (!(lam[2] > 0.f) || !(lam[0] < 1e30f) || !(m.mu > 0.f)) return L_PLAIN;
    float e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        sig[k] = sqrtf(lam[k]);
        e[k] = 0.5f * logf(lam[k]);
    }
    if (!yields<float>(m, sig)) return L_ELASTIC;
    features(m, e, x);
#pragma unroll
    for (int k = 0; k < N_FEAT; ++k) {
        if (!(x[k] >= hull.lo[k] && x[k] <= hull.hi[k])) return L_PLAIN;
        x[k] = (x[k] - hull.xm[k]) * hull.xs[k];
    }
    return L_NET;
}

// Learned path, part 2: from the network output y (normalised; NULL for
// an elastic particle: the stretches stand), the projected F, the Kirchhoff
// stress tensor P F^T (= tau), the energy and the plastic J.  Returns false
// when the residual check fails.
__device__ __forceinline__ bool learned_apply(const Material &m, const m3f &F, const float sig[3], const float V[9],
                                              const float *y, const Hull &hull, float jp_in, m3f &Fnew, m3f &tau_t,
                                              float &energy_out, float &jp_out, float &J_out) {
    float s[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) s[k] = y ? sig[k] * expf(hull.ym[k] + hull.ys[k] * y[k]) : sig[k];
    const float h = hardening<float>(m, sig, s, jp_in, jp_out);
    float tau[3];
    kirchhoff<float>(m, s, h, tau);
    if (y) {
        const float muh = m.mu * h;
        float res = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) res = fmaxf(res, fabsf(hull.ym[3 + k] + hull.ys[3 + k] * y[3 + k] - tau[k] / muh));
        if (!(res <= RES_TOL)) return false;
    }
    // G = F V; F' = G diag(s / sig) V^T; tau = G diag(tau / sig^2) G^T
    float G[9];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r)
            G[c * 3 + r] = F.a[r] * V[c * 3] + F.a[3 + r] * V[c * 3 + 1] + F.a[6 + r] * V[c * 3 + 2];
    float ps[3], pt[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) ps[k] = s[k] / sig[k], pt[k] = tau[k] / (sig[k] * sig[k]);
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            Fnew.a[c * 3 + r] = G[r] * ps[0] * V[c] + G[3 + r] * ps[1] * V[3 + c] + G[6 + r] * ps[2] * V[6 + c];
            tau_t.a[c * 3 + r] = G[r] * pt[0] * G[c] + G[3 + r] * pt[1] * G[3 + c] + G[6 + r] * pt[2] * G[6 + c];
        }
    energy_out = energy<float>(m, s, h);
    J_out = s[0] * s[1] * s[2];
    return true;
}

}  // namespace closure
}  // namespace sv
