// sv_math.cuh -- device linear algebra for the MPM substep: 3x3 matrices in
// registers, the quadratic B-spline, a one-sided Jacobi 3x3 SVD (fp32 with an
// fp64 twin for flagged particles) and the constitutive models of
// rust/crates/util/src/elastic.rs plus the fixed-corotated / snow additions.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sv {

// Column-major 3x3 like nalgebra's Matrix3: a[c * 3 + r].
template <class T> struct Mat3 {
    T a[9];
};
typedef Mat3<float> m3f;
typedef Mat3<double> m3d;

template <class T> __device__ __forceinline__ T &at(Mat3<T> &m, int r, int c) { return m.a[c * 3 + r]; }
template <class T> __device__ __forceinline__ T at(const Mat3<T> &m, int r, int c) { return m.a[c * 3 + r]; }

template <class T> __device__ __forceinline__ Mat3<T> mat_mul(const Mat3<T> &x, const Mat3<T> &y) {
    Mat3<T> r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.a[j * 3 + i] = x.a[i] * y.a[j * 3] + x.a[3 + i] * y.a[j * 3 + 1] + x.a[6 + i] * y.a[j * 3 + 2];
    return r;
}
// x * y^T
template <class T> __device__ __forceinline__ Mat3<T> mat_mul_bt(const Mat3<T> &x, const Mat3<T> &y) {
    Mat3<T> r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.a[j * 3 + i] = x.a[i] * y.a[j] + x.a[3 + i] * y.a[3 + j] + x.a[6 + i] * y.a[6 + j];
    return r;
}
template <class T> __device__ __forceinline__ T det3(const Mat3<T> &m) {
    return m.a[0] * (m.a[4] * m.a[8] - m.a[7] * m.a[5]) - m.a[3] * (m.a[1] * m.a[8] - m.a[7] * m.a[2]) +
           m.a[6] * (m.a[1] * m.a[5] - m.a[4] * m.a[2]);
}
// Cofactor matrix det(F) F^{-T}: columns c1 x c2, c2 x c0, c0 x c1
// (util/src/elastic.rs:115-120).
template <class T> __device__ __forceinline__ Mat3<T> cofactor(const Mat3<T> &m) {
    Mat3<T> r;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int p = (c + 1) % 3, q = (c + 2) % 3;
        r.a[c * 3 + 0] = m.a[p * 3 + 1] * m.a[q * 3 + 2] - m.a[p * 3 + 2] * m.a[q * 3 + 1];
        r.a[c * 3 + 1] = m.a[p * 3 + 2] * m.a[q * 3 + 0] - m.a[p * 3 + 0] * m.a[q * 3 + 2];
        r.a[c * 3 + 2] = m.a[p * 3 + 0] * m.a[q * 3 + 1] - m.a[p * 3 + 1] * m.a[q * 3 + 0];
    }
    return r;
}
// u diag(s) v^T
template <class T> __device__ __forceinline__ Mat3<T> recompose(const Mat3<T> &u, const T s[3], const Mat3<T> &v) {
    Mat3<T> r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            r.a[j * 3 + i] = u.a[i] * s[0] * v.a[j] + u.a[3 + i] * s[1] * v.a[3 + j] + u.a[6 + i] * s[2] * v.a[6 + j];
    return r;
}

template <class T> __device__ __forceinline__ T rsqrt_t(T x);
template <> __device__ __forceinline__ float rsqrt_t<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double rsqrt_t<double>(double x) { return rsqrt(x); }

// One-sided Jacobi (Hestenes) SVD: rotate the columns of A = F until they are
// mutually orthogonal; then S = column norms, U = normalised columns and V =
// the accumulated rotations.  S >= 0 (unsorted), U and V orthogonal, either
// may be a reflection -- the convention of nalgebra's SVD, so that
// U f(S) V^T and U V^T match the reference for any spectral f.  Relative
// accuracy of every singular value (Demmel & Veselic 1992) makes it safe for
// near-degenerate F in fp64.  `max_sweeps` bounds the work; each sweep stops
// early when no pair needed a rotation.
template <class T>
__device__ __forceinline__ void svd3(const Mat3<T> &F, Mat3<T> &U, T S[3], Mat3<T> &V, int max_sweeps) {
    T A[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] = F.a[i];
    T W[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    const T tol = sizeof(T) == 4 ? T(1e-7) : T(1e-15);
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        bool rotated = false;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            T alpha = A[p * 3] * A[p * 3] + A[p * 3 + 1] * A[p * 3 + 1] + A[p * 3 + 2] * A[p * 3 + 2];
            T beta = A[q * 3] * A[q * 3] + A[q * 3 + 1] * A[q * 3 + 1] + A[q * 3 + 2] * A[q * 3 + 2];
            T gamma = A[p * 3] * A[q * 3] + A[p * 3 + 1] * A[q * 3 + 1] + A[p * 3 + 2] * A[q * 3 + 2];
            if (gamma * gamma > tol * tol * alpha * beta && gamma != T(0)) {
                rotated = true;
                T zeta = (beta - alpha) / (T(2) * gamma);
                T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
                T c = rsqrt_t<T>(T(1) + t * t), s = c * t;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    T ap = A[p * 3 + r], aq = A[q * 3 + r];
                    A[p * 3 + r] = c * ap - s * aq;
                    A[q * 3 + r] = s * ap + c * aq;
                    T wp = W[p * 3 + r], wq = W[q * 3 + r];
                    W[p * 3 + r] = c * wp - s * wq;
                    W[q * 3 + r] = s * wp + c * wq;
                }
            }
        }
        if (!rotated) break;
    }
    const T tiny = sizeof(T) == 4 ? T(1e-30) : T(1e-290);
    int good[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        T n2 = A[i * 3] * A[i * 3] + A[i * 3 + 1] * A[i * 3 + 1] + A[i * 3 + 2] * A[i * 3 + 2];
        S[i] = sqrt(n2);
        good[i] = S[i] > tiny;
        T inv = good[i] ? T(1) / S[i] : T(0);
        U.a[i * 3] = A[i * 3] * inv, U.a[i * 3 + 1] = A[i * 3 + 1] * inv, U.a[i * 3 + 2] = A[i * 3 + 2] * inv;
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) V.a[i] = W[i];
    if (!(good[0] && good[1] && good[2])) {
        // Complete U to an orthonormal basis where columns vanished.
        int ng = good[0] + good[1] + good[2];
        int g0 = good[0] ? 0 : good[1] ? 1 : 2;
        if (ng == 0) {
            U.a[0] = 1, U.a[1] = 0, U.a[2] = 0;
            g0 = 0;
            good[0] = 1;
            ng = 1;
        }
        if (ng == 1) {
            int o1 = (g0 + 1) % 3;
            T ux = U.a[g0 * 3], uy = U.a[g0 * 3 + 1], uz = U.a[g0 * 3 + 2];
            T ax = fabs(ux) < T(0.9) ? T(1) : T(0), ay = fabs(ux) < T(0.9) ? T(0) : T(1);
            T wx = uy * T(0) - uz * ay, wy = uz * ax - ux * T(0), wz = ux * ay - uy * ax;
            T inv = rsqrt_t<T>(wx * wx + wy * wy + wz * wz);
            U.a[o1 * 3] = wx * inv, U.a[o1 * 3 + 1] = wy * inv, U.a[o1 * 3 + 2] = wz * inv;
            good[o1] = 1;
        }
        // exactly one column missing now: the cross product of the other two
        int m = !good[0] ? 0 : !good[1] ? 1 : 2;
        int a = (m + 1) % 3, b = (m + 2) % 3;
        U.a[m * 3 + 0] = U.a[a * 3 + 1] * U.a[b * 3 + 2] - U.a[a * 3 + 2] * U.a[b * 3 + 1];
        U.a[m * 3 + 1] = U.a[a * 3 + 2] * U.a[b * 3 + 0] - U.a[a * 3 + 0] * U.a[b * 3 + 2];
        U.a[m * 3 + 2] = U.a[a * 3 + 0] * U.a[b * 3 + 1] - U.a[a * 3 + 1] * U.a[b * 3 + 0];
    }
}

// fp32 one-sided Jacobi tuned for throughput: the column norms are updated
// in closed form after each rotation (|a_p|^2 -= t g, |a_q|^2 += t g), the
// rotation uses fast reciprocal / square-root intrinsics (any angle close to
// the optimal one still reduces the off-diagonal, and c^2 + s^2 = 1 keeps V
// orthogonal), and sweeps stop after one that started with every pair's
// cos^2 below 1e-9: in cyclic Jacobi's quadratic regime that sweep leaves
// them near 1e-18, under the rotation threshold below, and a further sweep
// would rotate nothing.  (Stopping only after a sweep that started
// below 1e-12 ran that idle sweep: 0.9 % of the 1M three-box fused pass.)
// A pair already orthogonal to fp32 epsilon is left alone (the reference
// test of one-sided Jacobi): near-identity F then gives U = V = I up to
// rounding instead of the arbitrary 45-degree rotations of a degenerate
// pair, whose fp32 rounding would put ~1e-7 noise into U V^T -- the fluid
// and sand returns rebuild F from U V^T every substep.  Returns true when a
// column vanished (degenerate F): U is then incomplete and the caller takes
// the fp64 path.
__device__ __forceinline__ bool svd3_fast_f32(const m3f &F, m3f &U, float S[3], m3f &V) {
    constexpr float EPS2 = 1.4210855e-14f;  // FLT_EPSILON^2
    float A[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) A[i] = F.a[i];
    float W[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
    float nrm[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) nrm[c] = A[c * 3] * A[c * 3] + A[c * 3 + 1] * A[c * 3 + 1] + A[c * 3 + 2] * A[c * 3 + 2];
    for (int sweep = 0; sweep < 6; ++sweep) {
        bool last = true;  // every pair's cos^2 below 1e-9 at the start of its rotation
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            const float g = A[p * 3] * A[q * 3] + A[p * 3 + 1] * A[q * 3 + 1] + A[p * 3 + 2] * A[q * 3 + 2];
            const float np = nrm[p], nq = nrm[q];
            last = last && g * g < 1e-9f * fmaxf(np * nq, 1e-30f);
            if (g * g > EPS2 * np * nq) {
                const float d = nq - np, e = 2.f * g;
                const float r2 = d * d + e * e;
                const float r = r2 * rsqrtf(r2);
                float t = __fdividef(e, fabsf(d) + r);
                t = d < 0.f ? -t : t;
                const float c = rsqrtf(1.f + t * t), s = c * t;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float ap = A[p * 3 + k], aq = A[q * 3 + k];
                    A[p * 3 + k] = c * ap - s * aq;
                    A[q * 3 + k] = s * ap + c * aq;
                    const float wp = W[p * 3 + k], wq = W[q * 3 + k];
                    W[p * 3 + k] = c * wp - s * wq;
                    W[q * 3 + k] = s * wp + c * wq;
                }
                nrm[p] = np - t * g;
                nrm[q] = nq + t * g;
            }
        }
        if (last) break;
    }
    bool good[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float n2 = A[c * 3] * A[c * 3] + A[c * 3 + 1] * A[c * 3 + 1] + A[c * 3 + 2] * A[c * 3 + 2];
        // correctly rounded, so that a unit column stays exactly unit
        S[c] = sqrtf(n2);
        const float inv = n2 > 1e-30f ? __frcp_rn(S[c]) : 0.f;
        good[c] = n2 > 1e-30f;
        U.a[c * 3] = A[c * 3] * inv, U.a[c * 3 + 1] = A[c * 3 + 1] * inv, U.a[c * 3 + 2] = A[c * 3 + 2] * inv;
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) V.a[i] = W[i];
    // a vanished column: degenerate F, whose U the fp64 path completes
    return !(good[0] && good[1] && good[2]);
}

// The fp64 SVD of an fp32 F, rounded back to fp32.
__device__ __forceinline__ void svd3_fp64(const m3f &F, m3f &U, float S[3], m3f &V) {
    m3d Fd, Ud, Vd;
    double Sd[3];
#pragma unroll
    for (int k = 0; k < 9; ++k) Fd.a[k] = (double)F.a[k];
    svd3<double>(Fd, Ud, Sd, Vd, 12);
#pragma unroll
    for (int k = 0; k < 9; ++k) U.a[k] = (float)Ud.a[k], V.a[k] = (float)Vd.a[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) S[k] = (float)Sd[k];
}

// Whether a particle's SVD is redone in fp64: a degenerate F always; policy
// 1 when det F < 0.05, policy 2 also when two singular values are closer
// than 1e-4.  SVD_ALWAYS_FP64 forces it (the deferred fp64 pass).
constexpr uint32_t SVD_ALWAYS_FP64 = 0x100u;
__device__ __forceinline__ bool svd_needs_fp64(const m3f &F, const float S[3], bool degenerate, uint32_t policy) {
    bool redo = degenerate || (policy & SVD_ALWAYS_FP64);
    if ((policy & 0xFFu) >= 1 && det3(F) < 0.05f) redo = true;
    if ((policy & 0xFFu) >= 2) {
        const float g = fminf(fabsf(S[0] - S[1]), fminf(fabsf(S[1] - S[2]), fabsf(S[0] - S[2])));
        if (g < 1e-4f) redo = true;
    }
    return redo;
}

// fp32 SVD of a particle's F with the fp64 redo for flagged particles
// (svd_needs_fp64).
__device__ __forceinline__ void particle_svd(const m3f &F, m3f &U, float S[3], m3f &V, uint32_t policy,
                                             uint32_t &fp64_count) {
    const bool degenerate = svd3_fast_f32(F, U, S, V);
    if (svd_needs_fp64(F, S, degenerate, policy)) {
        svd3_fp64(F, U, S, V);
        ++fp64_count;
    }
}

// ---------------------------------------------------------------- weights
// Quadratic B-spline weights of the three nodes base, base+1, base+2 for a
// particle at fx = x/dx - base in [0.5, 1.5) (rust/crates/cpu/src/kernels.rs:17-26
// evaluated at fx, fx - 1, fx - 2).
__device__ __forceinline__ void bspline_weights(float fx, float w[3]) {
    float a = 1.5f - fx, b = fx - 1.0f, c = fx - 0.5f;
    w[0] = 0.5f * a * a;
    w[1] = 0.75f - b * b;
    w[2] = 0.5f * c * c;
}

// ---------------------------------------------------------------- materials
// Device material record; particles point at one through the upper 24 bits of
// their packed flags word.
enum : uint32_t {
    KIND_NEO_HOOKEAN = 0,  // reference solid (util/src/elastic.rs:299-311)
    KIND_SAND = 1,         // reference solid + Drucker-Prager (advance_particles.rs:48-71)
    KIND_FLUID = 2,        // reference inviscid fluid (elastic.rs:546-592, advance_particles.rs:77-85)
    KIND_FIXED_COROTATED = 3,  // addition
    KIND_SNOW = 4,         // addition
};

struct Material {
    float mass, initial_volume;
    float mu, lambda;         // solids
    float alpha;              // sand
    float bulk_modulus;       // fluid
    int32_t exponent;         // fluid
    uint32_t kind;
    float visc_dynamic, visc_bulk;  // USE_VISCOSITY (0, 0 otherwise)
    float xi, theta_c, theta_s;     // snow
    uint32_t use_viscosity;
    uint32_t scene;  // index into the handle's scene table
    float iso_limit; // solids: the isolated-particle time step limit (set once dx is known)
};

// One independent scene of a handle: its particles are translated by `off`
// whole cells in the shared block index, and culled against its own domain
// (cell units, scene-local).
struct SceneInfo {
    double dmin[3], dmax[3];
    int32_t off[3];
    uint32_t pad;
};
static_assert(sizeof(SceneInfo) == 64, "SceneInfo is 64 bytes");
static_assert(sizeof(Material) == 64, "Material is 64 bytes");

__device__ __forceinline__ float powi_f(float x, int n) {
    float r = 1.f, b = x;
    unsigned k = n < 0 ? (unsigned)(-n) : (unsigned)n;
    while (k) {
        if (k & 1) r *= b;
        b *= b;
        k >>= 1;
    }
    return n < 0 ? 1.f / r : r;
}

// First Piola-Kirchhoff stress P(F).  `R` is the polar rotation of F and is
// only read by the corotated kinds; `hardening` scales mu and lambda (snow).
__device__ __forceinline__ m3f piola(const Material &m, const m3f &F, const m3f &R, float J, float hardening) {
    m3f cof = cofactor(F);
    m3f P;
    if (m.kind == KIND_FLUID) {
        // K (1 - J^-gamma) cof F
        float s = m.bulk_modulus * (1.f - 1.f / powi_f(J, m.exponent));
#pragma unroll
        for (int i = 0; i < 9; ++i) P.a[i] = s * cof.a[i];
    } else if (m.kind == KIND_FIXED_COROTATED || m.kind == KIND_SNOW) {
        float mu = m.mu * hardening, la = m.lambda * hardening;
        float s = la * (J - 1.f);
#pragma unroll
        for (int i = 0; i < 9; ++i) P.a[i] = 2.f * mu * (F.a[i] - R.a[i]) + s * cof.a[i];
    } else {
        // mu/2 * 2F + (lambda ln J - mu)/J cof F
        float d3 = (m.lambda * logf(J) - m.mu) / J;
        float mu = m.mu / 2.f * 2.f;
#pragma unroll
        for (int i = 0; i < 9; ++i) P.a[i] = mu * F.a[i] + d3 * cof.a[i];
    }
    return P;
}

}  // namespace sv
