// sv_adaptive.cuh -- adaptive time stepping of the reference
// (rust/crates/cpu/src/adaptive_time_step_state.rs:13-64 and
// rust/crates/cpu/src/phase/limit_time_step.rs:25-224): the four per-substep
// limits and the state that turns them into the time step of each phase.
// Device-side state, one thread updates it; the limits are reduced over the
// particles by the kernels in sv_substep.cu.
#pragma once
#include <float.h>
#include <stdint.h>

#include "sv_math.cuh"

namespace sv {
namespace adaptive {

constexpr float NONE = FLT_MAX;            // Option::None of a limit
constexpr int HISTORY = 11;                // the reference pops once the length exceeds 10
constexpr float SEPARATION = 1e-5f;        // util/src/consts.rs:14 SINGULAR_VALUE_SEPARATION

struct State {
    float max_dt;
    float vel, def, sound, iso;    // time_step_by_* (NONE when None)
    float hist[HISTORY];           // time_step_prior, oldest first
    int32_t hist_len;
    float dt_a, dt_b, dt_c;        // time step of external force, scatter, advance in this substep
    float pad;
    double time, target;
    // reductions of the running substep (float bits of non-negative values)
    uint32_t red_max_v, red_max_c, red_live;
    uint32_t red_sound, red_iso;
    uint32_t substeps;
    // red_sound / red_iso already hold the force limits of the current
    // particle state: the last adaptive substep's advance reduced them
    uint32_t force_ready;
    // the advance's step when the G2P's velocity and deformation limits do
    // not bind, and whether they did (the speculative advance is redone)
    float dt_spec;
    uint32_t redo;
    // the fused form: the next substep's scatter step assumed by this
    // substep's pass, the one that holds once its limits are known, and
    // whether that scatter is redone
    float dt_spec_b, dt_b_next;
    uint32_t p2g_redo;
};

// adaptive_time_step_state.rs:35-47
__host__ __device__ inline float without_prior(const State &s) {
    return fminf(fminf(fminf(s.max_dt, s.vel), fminf(s.def, s.sound)), s.iso);
}
// adaptive_time_step_state.rs:49-54
__host__ __device__ inline float allowed(const State &s) {
    float a = without_prior(s);
    for (int k = 0; k < s.hist_len; ++k) a = fminf(a, s.hist[k]);
    return a;
}
// allowed() right after the push of LimitTimeStepBeforeIntegrate, less the
// two limits that push brings (velocity and deformation): the push drops the
// oldest prior once the history is full, and the minimum over the rest does
// not depend on the new limits.  So that step is min(this, vel, def).
__host__ __device__ inline float step_without_g2p_limits(const State &s) {
    float d = fminf(fminf(s.max_dt, s.sound), s.iso);
    for (int k = s.hist_len > HISTORY - 1 ? 1 : 0; k < s.hist_len; ++k) d = fminf(d, s.hist[k]);
    return d;
}

// adaptive_time_step_state.rs:56-63
__host__ __device__ inline void push(State &s);

// The scatter step of the next substep (allowed() after its force push) if
// none of the four limits still to come binds: this substep's velocity and
// deformation limits and the next one's sound and isolated limits.  The
// pushes are played on a copy with those limits absent.
__host__ __device__ inline float next_scatter_step_without_new_limits(const State &s) {
    State c = s;
    c.vel = c.def = NONE;
    push(c);  // LimitTimeStepBeforeIntegrate of this substep
    c.sound = c.iso = NONE;
    push(c);  // LimitTimeStepBeforeForce of the next
    return allowed(c);
}

__host__ __device__ inline void push(State &s) {
    const float cur = without_prior(s);
    if (s.hist_len > HISTORY - 1) {
        for (int k = 1; k < s.hist_len; ++k) s.hist[k - 1] = s.hist[k];
        s.hist_len -= 1;
    }
    s.hist[s.hist_len++] = cur;
}

// limit_time_step.rs:36-123: dx / c with c the largest wave speed in the
// principal frame, from the first and second derivatives of the energy in
// singular-value space (Neo-Hookean for every solid, the reference's
// Solid parameters; inviscid for fluids).  s sorted descending.
template <class T>
__host__ __device__ inline T sound_limit(bool fluid, T mu, T lambda, T bulk, int32_t gamma, T mass, T volume,
                                         const T s[3], T dx) {
    const T x = s[0], y = s[1], z = s[2];
    const T J = x * y * z;
    const T g[3] = {y * z, x * z, x * y};
    const T H[3][3] = {{0, z, y}, {z, 0, x}, {y, x, 0}};
    T first[3], second[3][3];
    const T iJ = T(1) / J;
    if (!fluid) {
        // elastic.rs:314-339 with the invariant derivatives of elastic.rs:97-141, 276-295
        const T lj = log(J);
        const T d1 = (lambda * lj - mu) * iJ;
        const T d2 = (lambda * (T(1) - lj) + mu) * (iJ * iJ);
        for (int i = 0; i < 3; ++i) {
            first[i] = mu * s[i] + d1 * g[i];
            for (int j = 0; j < 3; ++j) second[i][j] = (i == j ? mu : T(0)) + d2 * g[i] * g[j] + d1 * H[i][j];
        }
    } else {
        // elastic.rs:555-570, 630-654
        T Jg = T(1);
        for (int k = 0; k < gamma; ++k) Jg *= J;
        const T iJg = T(1) / Jg;
        const T d1 = bulk * (T(1) - iJg);
        const T d2 = (T)gamma * bulk * iJg * iJ;
        for (int i = 0; i < 3; ++i) {
            first[i] = d1 * g[i];
            for (int j = 0; j < 3; ++j) second[i][j] = d2 * g[i] * g[j] + d1 * H[i][j];
        }
    }
    const bool xy = fabs(x - y) < (T)SEPARATION, yz = fabs(y - z) < (T)SEPARATION, zx = fabs(z - x) < (T)SEPARATION;
    // limit_time_step.rs:86-110 as written there (including its index choices)
    const T k3 = y * y * (xy ? (first[0] + x * second[0][0] - y * second[1][0]) / T(2) / x
                              : (x * first[0] - y * first[1]) / (x * x - y * y));
    const T k4 = y * z * (yz ? (first[1] + y * second[1][1] - z * second[2][1]) / T(2) / y
                              : (y * first[1] - z * first[2]) / (y * y - z * z));
    const T k5 = z * x * (zx ? (first[2] + x * second[2][2] - x * second[0][2]) / T(2) / z
                              : (z * first[2] - x * first[0]) / (z * z - x * x));
    T kappa = x * x * second[0][0];
    kappa = fmax(kappa, y * y * second[1][1]);
    kappa = fmax(kappa, z * z * second[2][2]);
    kappa = fmax(fmax(kappa, k3), fmax(k4, k5));
    // c^2 = (kappa / J) / rho with rho = mass / (volume J): the J cancels
    return dx / sqrt(kappa * volume / mass);
}

// limit_time_step.rs:126-178
template <class T>
__host__ __device__ inline T isolated_limit(bool fluid, T mu, T lambda, T bulk, int32_t gamma, T mass, T volume, T J,
                                            T dx) {
    if (!fluid) {
        const T xi = T(3) / dx / dx;
        return sqrt(mass / (volume * xi * (T(1) - T(1) / T(2)) * (mu + T(3) / T(2) * lambda)));
    }
    const T rho0 = mass / volume;
    T Jg = T(1);
    for (int k = 0; k < gamma; ++k) Jg *= J;
    const T first = bulk * (T(1) - T(1) / Jg);
    if (fabs(J - T(1)) > (T)SEPARATION) return dx / J * sqrt(rho0 * (J - T(1)) / (T(6) * first * T(3)));
    const T second = (T)gamma * bulk / (Jg * J);
    return dx * sqrt(rho0 / (T(6) * second * T(3)));
}

}  // namespace adaptive
}  // namespace sv
