// sv_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see sv_oracle.h).
//
// A CPU restatement of the reference MPM substep, Squishy Volumes
// rust/crates/cpu, templated on the scalar type: T = float follows the
// reference's f32 build, T = double is the precision twin (the reference's own
// util tests run in f64, util/src/lib.rs:27-30).  Each function cites the
// reference file:line it follows.  Parallel structure follows the reference:
// a hash-map grid keyed by (node id, collider bits) with per-node contributor
// lists, node-parallel gather P2G, particle-parallel G2P.
//
// Deliberate, documented deviations:
//  * The reference sort is unstable (sort.rs:50 par_sort_unstable_by_key); this
//    one is stable, so equal keys keep their prior order.
//  * Contributor lists are sorted by particle index, so P2G sums in a fixed
//    order (the reference pushes under a mutex from rayon threads, so its
//    summation order varies run to run, update_grid_nodes.rs:101-122).
//  * An energy error finishes the substep for every particle and then stops the
//    run; the reference short-circuits a rayon try_for_each, leaving an
//    unspecified subset of particles advanced (advance_particles.rs:28-91).
//  * The 3x3 SVD is a one-sided Jacobi (Hestenes) iteration, not nalgebra
//    0.33.3's Golub-Kahan; only convention-invariant products (U f(S) V^T,
//    U V^T) are used, so the choice of algorithm does not change results
//    beyond rounding.

#include "sv_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

namespace svo {

// ---------------------------------------------------------------- threading
class Pool {
  public:
    explicit Pool(int n) : n_(n < 1 ? 1 : n) {
        for (int i = 1; i < n_; ++i) workers_.emplace_back([this, i] { loop(i); });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto &w : workers_) w.join();
    }
    int size() const { return n_; }
    // f(begin, end, thread) over [0, n) split into contiguous chunks.
    void run(size_t n, const std::function<void(size_t, size_t, int)> &f) {
        if (n_ == 1 || n < 2048) {
            f(0, n, 0);
            return;
        }
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = &f;
            len_ = n;
            pending_ = n_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        chunk(0);
        std::unique_lock<std::mutex> l(m_);
        done_cv_.wait(l, [this] { return pending_ == 0; });
        job_ = nullptr;
    }

  private:
    void chunk(int t) {
        size_t per = (len_ + n_ - 1) / n_;
        size_t b = std::min(len_, per * (size_t)t), e = std::min(len_, b + per);
        if (b < e) (*job_)(b, e, t);
    }
    void loop(int t) {
        uint64_t seen = 0;
        for (;;) {
            std::unique_lock<std::mutex> l(m_);
            cv_.wait(l, [&] { return gen_ != seen; });
            seen = gen_;
            if (stop_) return;
            l.unlock();
            chunk(t);
            l.lock();
            if (--pending_ == 0) done_cv_.notify_one();
        }
    }
    int n_;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t, size_t, int)> *job_ = nullptr;
    size_t len_ = 0;
    int pending_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
};

// ---------------------------------------------------------------- linear algebra
template <class T> struct V3 {
    T e[3] = {0, 0, 0};
    T &operator[](int i) { return e[i]; }
    const T &operator[](int i) const { return e[i]; }
};
template <class T> V3<T> v3(T a, T b, T c) {
    V3<T> r;
    r[0] = a, r[1] = b, r[2] = c;
    return r;
}
template <class T> V3<T> operator+(V3<T> a, const V3<T> &b) {
    for (int i = 0; i < 3; ++i) a[i] += b[i];
    return a;
}
template <class T> V3<T> operator-(V3<T> a, const V3<T> &b) {
    for (int i = 0; i < 3; ++i) a[i] -= b[i];
    return a;
}
template <class T> V3<T> operator*(V3<T> a, T s) {
    for (int i = 0; i < 3; ++i) a[i] *= s;
    return a;
}
template <class T> T dot(const V3<T> &a, const V3<T> &b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <class T> V3<T> cross(const V3<T> &a, const V3<T> &b) {
    return v3<T>(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}

// Column-major like nalgebra's Matrix3: m[c * 3 + r].
template <class T> struct M3 {
    T m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    T &operator()(int r, int c) { return m[c * 3 + r]; }
    const T &operator()(int r, int c) const { return m[c * 3 + r]; }
    V3<T> col(int c) const { return v3<T>(m[c * 3], m[c * 3 + 1], m[c * 3 + 2]); }
    void set_col(int c, const V3<T> &v) {
        for (int r = 0; r < 3; ++r) m[c * 3 + r] = v[r];
    }
    static M3 identity() {
        M3 a;
        a(0, 0) = a(1, 1) = a(2, 2) = 1;
        return a;
    }
};
template <class T> M3<T> operator+(M3<T> a, const M3<T> &b) {
    for (int i = 0; i < 9; ++i) a.m[i] += b.m[i];
    return a;
}
template <class T> M3<T> operator-(M3<T> a, const M3<T> &b) {
    for (int i = 0; i < 9; ++i) a.m[i] -= b.m[i];
    return a;
}
template <class T> M3<T> operator*(M3<T> a, T s) {
    for (int i = 0; i < 9; ++i) a.m[i] *= s;
    return a;
}
template <class T> M3<T> operator*(const M3<T> &a, const M3<T> &b) {
    M3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T s = 0;
            for (int k = 0; k < 3; ++k) s += a(i, k) * b(k, j);
            r(i, j) = s;
        }
    return r;
}
template <class T> V3<T> operator*(const M3<T> &a, const V3<T> &v) {
    V3<T> r;
    for (int i = 0; i < 3; ++i) r[i] = a(i, 0) * v[0] + a(i, 1) * v[1] + a(i, 2) * v[2];
    return r;
}
template <class T> M3<T> transpose(const M3<T> &a) {
    M3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r(i, j) = a(j, i);
    return r;
}
template <class T> T det(const M3<T> &a) { return dot(a.col(0), cross(a.col(1), a.col(2))); }
template <class T> T trace(const M3<T> &a) { return a(0, 0) + a(1, 1) + a(2, 2); }
template <class T> T norm2(const M3<T> &a) {
    T s = 0;
    for (int i = 0; i < 9; ++i) s += a.m[i] * a.m[i];
    return s;
}
template <class T> M3<T> outer(const V3<T> &a, const V3<T> &b) {
    M3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r(i, j) = a[i] * b[j];
    return r;
}
template <class T> M3<T> diag_product(const M3<T> &u, const V3<T> &s, const M3<T> &v) {
    // u * diag(s) * v^T
    M3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r(i, j) = u(i, 0) * s[0] * v(j, 0) + u(i, 1) * s[1] * v(j, 1) + u(i, 2) * s[2] * v(j, 2);
    return r;
}

template <class T> T powi(T x, int n) {
    // Rust's powi for the integer exponents used by the fluid model.
    bool inv = n < 0;
    unsigned k = inv ? (unsigned)(-n) : (unsigned)n;
    T r = 1, b = x;
    while (k) {
        if (k & 1) r *= b;
        b *= b;
        k >>= 1;
    }
    return inv ? T(1) / r : r;
}

// One-sided Jacobi SVD, F = U diag(S) V^T, S >= 0 sorted descending, U and V
// orthogonal (either may be a reflection), as nalgebra's convention.
template <class T> void svd3(const M3<T> &F, M3<T> &U, V3<T> &S, M3<T> &V) {
    M3<T> A = F;
    V = M3<T>::identity();
    const T tol = std::numeric_limits<T>::epsilon();
    for (int sweep = 0; sweep < 40; ++sweep) {
        bool rotated = false;
        for (int pq = 0; pq < 3; ++pq) {
            int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            V3<T> ap = A.col(p), aq = A.col(q);
            T alpha = dot(ap, ap), beta = dot(aq, aq), gamma = dot(ap, aq);
            if (std::fabs(gamma) <= tol * std::sqrt(alpha * beta) || gamma == 0) continue;
            rotated = true;
            T zeta = (beta - alpha) / (2 * gamma);
            T t = (zeta >= 0 ? T(1) : T(-1)) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
            T c = 1 / std::sqrt(1 + t * t), s = c * t;
            A.set_col(p, ap * c - aq * s);
            A.set_col(q, ap * s + aq * c);
            V3<T> vp = V.col(p), vq = V.col(q);
            V.set_col(p, vp * c - vq * s);
            V.set_col(q, vp * s + vq * c);
        }
        if (!rotated) break;
    }
    int order[3] = {0, 1, 2};
    T nrm[3];
    for (int i = 0; i < 3; ++i) nrm[i] = std::sqrt(dot(A.col(i), A.col(i)));
    std::sort(order, order + 3, [&](int a, int b) { return nrm[a] > nrm[b]; });
    M3<T> A2, V2;
    for (int i = 0; i < 3; ++i) {
        A2.set_col(i, A.col(order[i]));
        V2.set_col(i, V.col(order[i]));
        S[i] = nrm[order[i]];
    }
    V = V2;
    // U columns: normalised A columns; complete degenerate ones orthonormally.
    const T tiny = std::numeric_limits<T>::min() * 16;
    V3<T> u[3];
    int good = 0;
    for (int i = 0; i < 3; ++i) {
        if (S[i] > tiny * (S[0] > 1 ? S[0] : 1) && S[i] > 0) {
            u[i] = A2.col(i) * (T(1) / S[i]);
            ++good;
        } else {
            good = i;
            break;
        }
    }
    if (good < 3) {
        if (good == 0) u[0] = v3<T>(1, 0, 0);
        if (good <= 1) {
            V3<T> a = std::fabs(u[0][0]) < T(0.9) ? v3<T>(1, 0, 0) : v3<T>(0, 1, 0);
            V3<T> w = cross(u[0], a);
            u[1] = w * (T(1) / std::sqrt(dot(w, w)));
        }
        u[2] = cross(u[0], u[1]);
    }
    for (int i = 0; i < 3; ++i) U.set_col(i, u[i]);
}

// ---------------------------------------------------------------- elastic.rs
// util/src/elastic.rs:52-64 (Lamé parameters from E and nu).
template <class T> T lame_mu(T E, T nu) { return E / T(2) / (T(1) + nu); }
template <class T> T lame_lambda(T E, T nu) { return E * nu / (T(1) + nu) / (T(1) - T(2) * nu); }

// util/src/elastic.rs:115-120 partial_invariant_3_by_position_gradient:
// columns c1 x c2, c2 x c0, c0 x c1 (the cofactor matrix).
template <class T> M3<T> cofactor(const M3<T> &F) {
    M3<T> r;
    r.set_col(0, cross(F.col(1), F.col(2)));
    r.set_col(1, cross(F.col(2), F.col(0)));
    r.set_col(2, cross(F.col(0), F.col(1)));
    return r;
}

// util/src/elastic.rs:299-311 first_piola_stress_neo_hookean with the partials
// of :282-291 (mu/2 * 2F + (lambda ln J - mu)/J * cof F).
template <class T> M3<T> piola_neo_hookean(T mu, T lambda, const M3<T> &F) {
    T J = det(F);
    T d3 = (lambda * std::log(J) - mu) / J;
    return F * (mu / T(2) * T(2)) + cofactor(F) * d3;
}

// util/src/elastic.rs:233-272 (NH energy by invariants; J <= 0 is an error).
template <class T> T energy_neo_hookean(T mu, T lambda, const M3<T> &F) {
    T I2 = norm2(F), J = det(F);
    T lj = std::log(J);
    return mu / T(2) * (I2 - T(3)) - mu * lj + lambda / T(2) * lj * lj;
}

// util/src/elastic.rs:546-592 inviscid fluid.
template <class T> T energy_inviscid(T K, int gamma, T J) {
    T at_rest = K * (T(1) - T(1) / (T(1) - T(gamma)));
    return K * (J - powi(J, 1 - gamma) / (T(1) - T(gamma))) - at_rest;
}
template <class T> M3<T> piola_inviscid(T K, int gamma, const M3<T> &F) {
    T J = det(F);
    return cofactor(F) * (K * (T(1) - T(1) / powi(J, gamma)));
}

// util/src/elastic.rs:659-677 Newtonian viscous Cauchy stress.
template <class T> M3<T> cauchy_viscosity(T dyn, T bulk, const M3<T> &C) {
    M3<T> r = (C + transpose(C)) * (T(0.5) * T(2) * dyn);
    T tr = trace(C) * bulk;
    r(0, 0) += tr, r(1, 1) += tr, r(2, 2) += tr;
    return r;
}

// Not in the reference: fixed-corotated elasticity (Stomakhin et al. 2012),
// psi = mu |F - R|^2 + lambda/2 (J - 1)^2, P = 2 mu (F - R) + lambda (J - 1) cof F.
template <class T> M3<T> polar_rotation(const M3<T> &F) {
    M3<T> U, V;
    V3<T> S;
    svd3(F, U, S, V);
    return U * transpose(V);
}
template <class T> M3<T> piola_fixed_corotated(T mu, T lambda, const M3<T> &F) {
    M3<T> R = polar_rotation(F);
    T J = det(F);
    return (F - R) * (T(2) * mu) + cofactor(F) * (lambda * (J - T(1)));
}
template <class T> T energy_fixed_corotated(T mu, T lambda, const M3<T> &F) {
    M3<T> R = polar_rotation(F);
    T J = det(F);
    return mu * norm2(F - R) + lambda / T(2) * (J - T(1)) * (J - T(1));
}

// rust/crates/cpu/src/phase/advance_particles.rs:48-71 sand (Drucker-Prager
// return map in Hencky strain).  In expansion (or pure volume change) F
// becomes U V^T whatever mu is.  Returns false, leaving F as it is, on the
// compressive branch with mu <= 0, where the reference asserts mu > 0
// (advance_particles.rs:57).
template <class T> bool project_sand(T mu, T lambda, T alpha, M3<T> &F) {
    M3<T> U, V;
    V3<T> s;
    svd3(F, U, s, V);
    V3<T> e = v3<T>(std::log(s[0]), std::log(s[1]), std::log(s[2]));
    T e_tr = e[0] + e[1] + e[2];
    V3<T> e_hat = e - v3<T>(e_tr / T(3), e_tr / T(3), e_tr / T(3));
    T e_hat_norm = std::sqrt(dot(e_hat, e_hat));
    if (e_tr < T(0) && e_hat_norm > T(0)) {
        if (!(mu > T(0))) return false;
        T delta_gamma = e_hat_norm + (T(3) * lambda + T(2) * mu) / T(2) / mu * e_tr * alpha;
        if (delta_gamma > T(0)) {
            V3<T> H = e - e_hat * (delta_gamma / e_hat_norm);
            F = diag_product(U, v3<T>(std::exp(H[0]), std::exp(H[1]), std::exp(H[2])), V);
        }
    } else {
        F = U * transpose(V);
    }
    return true;
}

// rust/crates/cpu/src/phase/advance_particles.rs:77-85 fluid: all singular
// values replaced by their geometric mean.
template <class T> void project_fluid(M3<T> &F) {
    M3<T> U, V;
    V3<T> s;
    svd3(F, U, s, V);
    T g = std::pow(s[0] * s[1] * s[2], T(1) / T(3));
    F = diag_product(U, v3<T>(g, g, g), V);
}

// Not in the reference: snow plasticity (Stomakhin et al. 2013): clamp the
// singular values of the elastic F to [1 - theta_c, 1 + theta_s] and move the
// removed volume into J_p.
template <class T> void project_snow(T theta_c, T theta_s, M3<T> &F, T &plastic_j) {
    M3<T> U, V;
    V3<T> s;
    svd3(F, U, s, V);
    V3<T> c;
    for (int i = 0; i < 3; ++i) c[i] = std::min(std::max(s[i], T(1) - theta_c), T(1) + theta_s);
    plastic_j = plastic_j * (s[0] * s[1] * s[2]) / (c[0] * c[1] * c[2]);
    F = diag_product(U, c, V);
}

// rust/crates/cpu/src/kernels.rs:17-26.
template <class T> T kernel_quadratic(T x) {
    x = std::fabs(x);
    if (x < T(0.5)) return T(0.75) - x * x;
    if (x < T(1.5)) return T(0.5) * (T(1.5) - x) * (T(1.5) - x);
    return T(0);
}

// ---------------------------------------------------------------- particle state
enum : uint32_t {
    IS_SOLID = 1u << 0,
    IS_FLUID = 1u << 1,
    USE_VISCOSITY = 1u << 2,
    USE_SAND_ALPHA = 1u << 3,
    HAS_GOAL = 1u << 4,
    TOMBSTONED = 1u << 5,
    FAILED = 1u << 6,
};

struct Params {
    float mass, initial_volume;
    float vdyn, vbulk;
    float mu, lambda, alpha;
    int32_t exponent;
    float bulk_modulus;
    uint32_t model;
    float xi, theta_c, theta_s;
};

struct GridKey {
    int32_t i, j, k;
    uint32_t bits;
    bool operator==(const GridKey &o) const { return i == o.i && j == o.j && k == o.k && bits == o.bits; }
    bool operator<(const GridKey &o) const {
        if (i != o.i) return i < o.i;
        if (j != o.j) return j < o.j;
        if (k != o.k) return k < o.k;
        return bits < o.bits;
    }
};

// Open-addressing map GridKey -> u32 with an FxHash-style mix, standing in for
// the reference's FxHashMap<GridKey, u32> (cpu/src/grid_nodes.rs:15-33).
// Concurrent readers are allowed while no writer runs.
class NodeMap {
  public:
    void clear() {
        slots_.assign(slots_.size(), Slot{});
        size_ = 0;
    }
    size_t size() const { return size_; }
    void reserve(size_t n) {
        size_t want = 16;
        while (want < 2 * n) want <<= 1;
        if (want > slots_.size()) rehash(want);
    }
    const uint32_t *get(const GridKey &k) const {
        if (slots_.empty()) return nullptr;
        size_t mask = slots_.size() - 1, h = hash(k) & mask;
        for (;;) {
            const Slot &s = slots_[h];
            if (!s.used) return nullptr;
            if (s.key == k) return &s.value;
            h = (h + 1) & mask;
        }
    }
    // Inserts when absent; returns the stored value.
    uint32_t insert(const GridKey &k, uint32_t value) {
        if (2 * (size_ + 1) > slots_.size()) rehash(slots_.empty() ? 16 : slots_.size() * 2);
        size_t mask = slots_.size() - 1, h = hash(k) & mask;
        for (;;) {
            Slot &s = slots_[h];
            if (!s.used) {
                s.used = true, s.key = k, s.value = value;
                ++size_;
                return value;
            }
            if (s.key == k) return s.value;
            h = (h + 1) & mask;
        }
    }
    template <class F> void for_each(F f) const {
        for (auto &s : slots_)
            if (s.used) f(s.key, s.value);
    }

  private:
    struct Slot {
        GridKey key{0, 0, 0, 0};
        uint32_t value = 0;
        bool used = false;
    };
    static size_t hash(const GridKey &k) {
        uint64_t h = 0;
        const uint64_t K = 0x517cc1b727220a95ull;
        for (uint32_t w : {(uint32_t)k.i, (uint32_t)k.j, (uint32_t)k.k, k.bits}) h = ((h << 5 | h >> 59) ^ w) * K;
        return (size_t)(h ^ (h >> 29));
    }
    void rehash(size_t n) {
        std::vector<Slot> old;
        old.swap(slots_);
        slots_.assign(n, Slot{});
        size_ = 0;
        for (auto &s : old)
            if (s.used) insert(s.key, s.value);
    }
    std::vector<Slot> slots_;
    size_t size_ = 0;
};

// util/src/collider_bits.rs:34-38.
inline bool compatible(uint32_t a, uint32_t b) {
    uint32_t mask = (a & b) >> 16;
    uint32_t diff = a ^ b;
    return (mask & diff) == 0;
}

struct Base {
    virtual ~Base() {}
    virtual int set_frame_input(const svo_frame_input *in) = 0;
    virtual void set_time(double t) = 0;
    virtual double get_time() const = 0;
    virtual int step(uint32_t n, float dt, const float g[3]) = 0;
    virtual int step_adaptive(double *time, double target, float max_dt, const float g[3], uint32_t *substeps,
                              float limits[8]) = 0;
    virtual void download(svo_particles *out) = 0;
    virtual uint64_t grid(int32_t *ids, float *m, float *v, uint64_t cap) = 0;
    virtual void p2g_only(float dt, const float g[3]) = 0;
};

template <class T> struct State : Base {
    Pool pool;
    size_t n = 0;
    // cpu/src/particles.rs:13-31
    std::vector<uint32_t> sort_map, reverse_sort_map, flags, collider_bits;
    std::vector<Params> params;
    std::vector<V3<T>> x, v;
    std::vector<M3<T>> F, C;
    std::vector<T> energy, plastic_j;
    bool has_plastic_j = false;
    T dx;
    T dmin[3], dmax[3];
    int ground_mode = 0, ground_axis = 2;
    T ground_height = 0;
    // cpu/src/grid_nodes.rs:21-33
    NodeMap map;
    std::vector<GridKey> keys;
    std::vector<uint32_t> contrib_count, contrib_offset, contrib;
    std::vector<T> masses;
    std::vector<V3<T>> velocities;
    std::vector<uint32_t> node_of;  // [n * 27] node index of each (particle, stencil entry)

    State(const svo_particles *p, const svo_consts *c, int threads) : pool(threads) {
        n = (size_t)p->n;
        sort_map.resize(n), reverse_sort_map.resize(n);
        for (size_t i = 0; i < n; ++i) sort_map[i] = reverse_sort_map[i] = (uint32_t)i;
        flags.assign(p->flags, p->flags + n);
        collider_bits.resize(n, 0);
        if (p->collider_bits) collider_bits.assign(p->collider_bits, p->collider_bits + n);
        params.resize(n);
        x.resize(n), v.resize(n), F.resize(n), C.resize(n), energy.resize(n, 0), plastic_j.resize(n, T(1));
        has_plastic_j = p->plastic_j != nullptr;
        for (size_t i = 0; i < n; ++i) {
            Params &q = params[i];
            q.mass = p->mass[i], q.initial_volume = p->initial_volume[i];
            q.vdyn = p->viscosity_dynamic ? p->viscosity_dynamic[i] : 0.f;
            q.vbulk = p->viscosity_bulk ? p->viscosity_bulk[i] : 0.f;
            q.mu = p->mu ? p->mu[i] : 0.f;
            q.lambda = p->lambda ? p->lambda[i] : 0.f;
            q.alpha = p->sand_alpha ? p->sand_alpha[i] : 0.f;
            q.exponent = p->exponent ? p->exponent[i] : 0;
            q.bulk_modulus = p->bulk_modulus ? p->bulk_modulus[i] : 0.f;
            q.model = p->model ? p->model[i] : 0u;
            q.xi = p->hardening ? p->hardening[i] : 0.f;
            q.theta_c = p->crit_compression ? p->crit_compression[i] : 0.f;
            q.theta_s = p->crit_stretch ? p->crit_stretch[i] : 0.f;
            for (int a = 0; a < 3; ++a) x[i][a] = (T)p->positions[3 * i + a], v[i][a] = (T)p->velocities[3 * i + a];
            for (int a = 0; a < 9; ++a) F[i].m[a] = (T)p->position_gradients[9 * i + a], C[i].m[a] = (T)p->velocity_gradients[9 * i + a];
            if (p->elastic_energies) energy[i] = (T)p->elastic_energies[i];
            if (p->plastic_j) plastic_j[i] = (T)p->plastic_j[i];
        }
        dx = (T)c->grid_node_size;
        for (int a = 0; a < 3; ++a) dmin[a] = (T)c->domain_min[a], dmax[a] = (T)c->domain_max[a];
        ground_mode = c->ground_mode, ground_axis = c->ground_axis, ground_height = (T)c->ground_height;
    }

    // cpu/src/phase/sort.rs:17-114 (stable here, see header).
    void sort() {
        struct Key {
            int32_t i, j, k;
        };
        std::vector<Key> key(n);
        pool.run(n, [&](size_t b, size_t e, int) {
            for (size_t p = b; p < e; ++p)
                for (int a = 0; a < 3; ++a) (&key[p].i)[a] = (int32_t)std::floor(x[p][a] / dx - T(0.5));
        });
        std::vector<uint32_t> perm(n);
        for (size_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
        std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) {
            const Key &ka = key[a], &kb = key[b];
            if (ka.i != kb.i) return ka.i < kb.i;
            if (ka.j != kb.j) return ka.j < kb.j;
            return ka.k < kb.k;
        });
        auto apply = [&](auto &vec) {
            auto old = vec;
            pool.run(n, [&](size_t b, size_t e, int) {
                for (size_t i = b; i < e; ++i) vec[i] = old[perm[i]];
            });
        };
        // elastic_energies and reverse_sort_map are not moved (sort.rs:78-81):
        // live particles get a fresh energy in advance_particles, tombstoned
        // ones keep whatever value sits at their new index.
        apply(flags), apply(x), apply(sort_map), apply(params), apply(F), apply(v), apply(C),
            apply(collider_bits), apply(plastic_j);
        for (size_t cur = 0; cur < n; ++cur) reverse_sort_map[sort_map[cur]] = (uint32_t)cur;
    }

    // cpu/src/phase/external_force.rs:17-50: gravity, or the velocity that
    // reaches the interpolated goal in one step when both frames give the
    // particle a goal.
    void external_force(T dt, const V3<T> &g) {
        pool.run(n, [&](size_t b, size_t e, int) {
            for (size_t p = b; p < e; ++p) {
                if (flags[p] & TOMBSTONED) continue;
                const uint32_t o = sort_map[p];
                if (fin.goals && (fin.gflag_a[o] & HAS_GOAL) && (fin.gflag_b[o] & HAS_GOAL)) {
                    for (int a = 0; a < 3; ++a) v[p][a] = ((T)igoal[3 * o + a] - x[p][a]) / dt;
                } else {
                    v[p] = v[p] + g * dt;
                }
            }
        });
    }

    // gravity of the substep: the interpolated input's, else the argument
    V3<T> substep_gravity(const float g_f[3]) const {
        if (fin.set) return v3<T>((T)ig[0], (T)ig[1], (T)ig[2]);
        return v3<T>((T)g_f[0], (T)g_f[1], (T)g_f[2]);
    }

    // cpu/src/kernels.rs:46-49 position_to_shift_quadratic.
    V3<int> shift_of(const V3<T> &pos) const {
        V3<int> s;
        for (int a = 0; a < 3; ++a) s[a] = (int)std::floor(pos[a] / dx - T(0.5));
        return s;
    }

    // cpu/src/phase/update_grid_nodes.rs:31-156: keep the previous map, prune
    // nodes that had no contributors, look existing nodes up in parallel,
    // insert new nodes serially, then build per-node contributor lists.
    void update_grid_nodes() {
        {
            NodeMap pruned;
            pruned.reserve(map.size());
            uint32_t next = 0;
            std::vector<std::pair<GridKey, uint32_t>> kept;
            map.for_each([&](const GridKey &k, uint32_t idx) {
                if (idx < contrib_count.size() && contrib_count[idx] > 0) kept.push_back({k, idx});
            });
            std::sort(kept.begin(), kept.end(), [](auto &a, auto &b) { return a.second < b.second; });
            for (auto &kv : kept) pruned.insert(kv.first, next++);
            map = std::move(pruned);
        }
        node_of.assign(n * 27, UINT32_MAX);
        int nt = pool.size();
        std::vector<std::vector<std::pair<GridKey, uint32_t>>> missing(nt);
        pool.run(n, [&](size_t b, size_t e, int t) {
            for (size_t p = b; p < e; ++p) {
                if (flags[p] & TOMBSTONED) continue;
                V3<int> s = shift_of(x[p]);
                int q = 0;
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j)
                        for (int k = 0; k < 3; ++k, ++q) {
                            GridKey key{s[0] + i, s[1] + j, s[2] + k, collider_bits[p]};
                            const uint32_t *idx = map.get(key);
                            if (idx) node_of[p * 27 + q] = *idx;
                            else missing[t].push_back({key, (uint32_t)(p * 27 + q)});
                        }
            }
        });
        // serial collector (update_grid_nodes.rs:75-91)
        for (auto &list : missing)
            for (auto &kv : list) node_of[kv.second] = map.insert(kv.first, (uint32_t)map.size());
        size_t m = map.size();
        keys.assign(m, GridKey{0, 0, 0, 0});
        map.for_each([&](const GridKey &k, uint32_t idx) { keys[idx] = k; });
        contrib_count.assign(m, 0);
        for (size_t p = 0; p < n; ++p) {
            if (flags[p] & TOMBSTONED) continue;
            for (int q = 0; q < 27; ++q) contrib_count[node_of[p * 27 + q]]++;
        }
        contrib_offset.assign(m + 1, 0);
        for (size_t i = 0; i < m; ++i) contrib_offset[i + 1] = contrib_offset[i] + contrib_count[i];
        contrib.resize(contrib_offset[m]);
        std::vector<uint32_t> cursor(contrib_offset.begin(), contrib_offset.end() - 1);
        for (size_t p = 0; p < n; ++p) {
            if (flags[p] & TOMBSTONED) continue;
            for (int q = 0; q < 27; ++q) contrib[cursor[node_of[p * 27 + q]]++] = (uint32_t)p;
        }
    }

    // util/src/elastic.rs stresses as selected by scatter_momentum.rs:46-61,
    // plus the additions (model 1 fixed-corotated, model 2 snow).
    M3<T> stress(size_t p) const {
        const Params &q = params[p];
        if (flags[p] & IS_FLUID) return piola_inviscid<T>((T)q.bulk_modulus, q.exponent, F[p]);
        if (q.model == 1) return piola_fixed_corotated<T>((T)q.mu, (T)q.lambda, F[p]);
        if (q.model == 2) {
            T h = std::exp((T)q.xi * (T(1) - plastic_j[p]));
            return piola_fixed_corotated<T>((T)q.mu * h, (T)q.lambda * h, F[p]);
        }
        return piola_neo_hookean<T>((T)q.mu, (T)q.lambda, F[p]);
    }

    // cpu/src/phase/scatter_momentum.rs:22-93: P2G gathered per node over its
    // contributor list.
    void scatter_momentum(T dt) {
        size_t m = keys.size();
        T scaling = dt * T(4) / (dx * dx);
        masses.assign(m, T(0));
        velocities.assign(m, V3<T>{});
        // P(F) is recomputed per (node, particle) pair by the reference; it is
        // a pure function of the particle, so it is cached here.
        std::vector<M3<T>> stress_c(n);
        std::vector<T> detF(n);
        pool.run(n, [&](size_t b, size_t e, int) {
            for (size_t p = b; p < e; ++p)
                if (!(flags[p] & TOMBSTONED)) stress_c[p] = stress(p), detF[p] = det(F[p]);
        });
        pool.run(m, [&](size_t b, size_t e, int) {
            for (size_t node = b; node < e; ++node) {
                const GridKey &key = keys[node];
                V3<T> nid = v3<T>((T)key.i, (T)key.j, (T)key.k);
                T mass = 0;
                V3<T> mom;
                for (uint32_t c = contrib_offset[node]; c < contrib_offset[node + 1]; ++c) {
                    uint32_t p = contrib[c];
                    V3<T> normalized;
                    for (int a = 0; a < 3; ++a) normalized[a] = x[p][a] / dx;
                    V3<T> to_norm = nid - normalized;
                    T w = kernel_quadratic(to_norm[0]) * kernel_quadratic(to_norm[1]) * kernel_quadratic(to_norm[2]);
                    V3<T> to_node = to_norm * dx;
                    const Params &q = params[p];
                    V3<T> imparted = (v[p] + C[p] * to_node) * (T)q.mass;
                    if (flags[p] & USE_VISCOSITY) {
                        M3<T> cs = cauchy_viscosity<T>((T)q.vdyn, (T)q.vbulk, C[p]);
                        imparted = imparted - cs * (to_node * (scaling * detF[p] * (T)q.initial_volume));
                    }
                    imparted = imparted - stress_c[p] * (transpose(F[p]) * (to_node * (scaling * (T)q.initial_volume)));
                    imparted = imparted * w;
                    mass += w * (T)q.mass;
                    mom = mom + imparted;
                }
                masses[node] = mass;
                velocities[node] = mom;
            }
        });
    }

    // cpu/src/phase/meld_grid.rs:16-69, plus the grid boundary plane addition.
    void meld_grid() {
        size_t m = keys.size();
        std::vector<T> m0 = masses;
        std::vector<V3<T>> v0 = velocities;
        // multi map node id -> variants (update_grid_nodes.rs:145-155)
        bool any_bits = false;
        for (auto &k : keys) any_bits |= k.bits != 0;
        NodeMap first;  // node id -> first variant index (only used when bits exist)
        std::vector<std::vector<uint32_t>> variants;
        if (any_bits) {
            for (size_t i = 0; i < m; ++i) {
                GridKey id{keys[i].i, keys[i].j, keys[i].k, 0};
                uint32_t slot = first.insert(id, (uint32_t)variants.size());
                if (slot == variants.size()) variants.emplace_back();
                variants[slot].push_back((uint32_t)i);
            }
        }
        pool.run(m, [&](size_t b, size_t e, int) {
            for (size_t i = b; i < e; ++i) {
                T mass = masses[i];
                V3<T> vel = velocities[i];
                if (any_bits) {
                    GridKey id{keys[i].i, keys[i].j, keys[i].k, 0};
                    for (uint32_t o : variants[*first.get(id)]) {
                        if (o == i || !compatible(keys[i].bits, keys[o].bits)) continue;
                        mass += m0[o];
                        vel = vel + v0[o];
                    }
                }
                if (mass > T(0)) vel = vel * (T(1) / mass);
                else vel = V3<T>{};
                if (ground_mode != 0) {
                    int node_c = ground_axis == 0 ? keys[i].i : ground_axis == 1 ? keys[i].j : keys[i].k;
                    if ((T)node_c * dx <= ground_height) {
                        if (ground_mode == 1) vel = V3<T>{};
                        else if (vel[ground_axis] < T(0)) vel[ground_axis] = T(0);
                    }
                }
                masses[i] = mass;
                velocities[i] = vel;
            }
        });
    }

    // cpu/src/phase/collect_velocity.rs:19-75: G2P with 27 map lookups.
    void collect_velocity() {
        pool.run(n, [&](size_t b, size_t e, int) {
            for (size_t p = b; p < e; ++p) {
                if (flags[p] & TOMBSTONED) continue;
                V3<T> vel;
                M3<T> grad;
                V3<T> normalized;
                for (int a = 0; a < 3; ++a) normalized[a] = x[p][a] / dx;
                V3<T> shift, shifted;
                for (int a = 0; a < 3; ++a) shift[a] = std::floor(normalized[a] - T(0.5)), shifted[a] = normalized[a] - shift[a];
                T w[3][3];
                for (int a = 0; a < 3; ++a)
                    for (int i = 0; i < 3; ++i) w[a][i] = kernel_quadratic(shifted[a] - (T)i);
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j)
                        for (int k = 0; k < 3; ++k) {
                            T weight = w[0][i] * w[1][j] * w[2][k];
                            GridKey key{(int)shift[0] + i, (int)shift[1] + j, (int)shift[2] + k, collider_bits[p]};
                            V3<T> gnp = v3<T>((T)key.i * dx, (T)key.j * dx, (T)key.k * dx);
                            V3<T> to_grid_node = gnp - x[p];
                            const uint32_t *idx = map.get(key);
                            V3<T> gv = velocities[*idx];
                            vel = vel + gv * weight;
                            grad = grad + outer(gv * weight, to_grid_node);
                        }
                v[p] = vel;
                C[p] = grad * (T(4) / dx / dx);
            }
        });
    }

    // cpu/src/phase/advance_particles.rs:17-93 (+ snow / fixed-corotated
    // additions).  Returns the number of particles whose energy failed.
    size_t advance_particles(T dt) {
        std::atomic<size_t> failed{0};
        pool.run(n, [&](size_t b, size_t e, int) {
            size_t local = 0;
            for (size_t p = b; p < e; ++p) {
                if (flags[p] & TOMBSTONED) continue;
                x[p] = x[p] + v[p] * dt;
                F[p] = F[p] + (C[p] * F[p]) * dt;
                const Params &q = params[p];
                if (flags[p] & IS_FLUID) {
                    project_fluid(F[p]);
                    energy[p] = energy_inviscid<T>((T)q.bulk_modulus, q.exponent, det(F[p]));
                    continue;
                }
                T mu = (T)q.mu, lambda = (T)q.lambda;
                if (q.model == 2) {
                    project_snow<T>((T)q.theta_c, (T)q.theta_s, F[p], plastic_j[p]);
                } else if (flags[p] & USE_SAND_ALPHA) {
                    if (!project_sand<T>(mu, lambda, (T)q.alpha, F[p])) sand_mu_error = true;
                }
                T J = det(F[p]);
                if (!(J > T(0))) {
                    flags[p] |= FAILED;
                    ++local;
                    continue;
                }
                if (q.model == 1) energy[p] = energy_fixed_corotated(mu, lambda, F[p]);
                else if (q.model == 2) {
                    T h = std::exp((T)q.xi * (T(1) - plastic_j[p]));
                    energy[p] = energy_fixed_corotated(mu * h, lambda * h, F[p]);
                } else energy[p] = energy_neo_hookean(mu, lambda, F[p]);
            }
            failed += local;
        });
        return failed.load();
    }

    // cpu/src/phase/cull_particles.rs:17-41 (strict bounds).
    void cull_particles() {
        pool.run(n, [&](size_t b, size_t e, int) {
            for (size_t p = b; p < e; ++p) {
                if (flags[p] & TOMBSTONED) continue;
                bool inside = true;
                for (int a = 0; a < 3; ++a) inside = inside && x[p][a] > dmin[a] && x[p][a] < dmax[a];
                if (!inside) flags[p] |= TOMBSTONED;
            }
        });
    }

    // cpu/src/cpu_state.rs:146-197 with adaptive_time_steps = false and the
    // phase order of cpu/src/phase/mod.rs:27-41 (InterpolateInput and Collide
    // have no inputs here: gravity is passed in, there are no colliders).
    // Returns 1 on an energy error, 3 on a sand particle compressed with
    // mu <= 0 (where the reference asserts mu > 0).
    int step(uint32_t nsub, float dt_f, const float g_f[3]) override {
        T dt = (T)dt_f;
        for (uint32_t s = 0; s < nsub; ++s) {
            if (fin.set && interpolate_input()) return -2;
            const V3<T> g = substep_gravity(g_f);
            sort();
            collide(dt);
            external_force(dt, g);
            update_grid_nodes();
            scatter_momentum(dt);
            meld_grid();
            collect_velocity();
            if (advance_particles(dt) > 0) return 1;
            if (sand_mu_error) return 3;
            cull_particles();
            time += (double)dt_f;
        }
        return 0;
    }

    // ---- frame input (xpu/src/frame_input.rs:33-65) and its interpolation
    struct FrameIn {
        bool set = false;
        uint32_t fps = 24, frame = 0;
        bool has_b = false;
        float g_a[3] = {0, 0, 0}, g_b[3] = {0, 0, 0};
        bool goals = false;
        std::vector<uint32_t> gflag_a, gflag_b;
        std::vector<float> goal_a, goal_b;
        uint32_t nv = 0, nt = 0;
        std::vector<uint32_t> tri, tri_col;
        std::vector<float> va, vb, fr_a, fr_b, dm_a, dm_b;
        float leaf = 1.f;
        std::vector<uint32_t> opp;                 // mesh_util/src/mesh.rs:71-94: ab, bc, ca neighbours
        std::vector<std::vector<uint32_t>> vtris;  // mesh.rs:106-135: emptied where the mesh is not closed
        std::vector<float> vvel;                   // frame_input.rs:329-343 linear_vertex_velocities
        std::vector<int32_t> lmin, lmax;           // frame_input.rs:345-390 padded leaf boxes
    } fin;
    double time = 0;
    // a sand particle met the compressive branch with mu <= 0, where the
    // reference asserts mu > 0 (advance_particles.rs:57); the step reports 3
    std::atomic<bool> sand_mu_error{false};
    // InterpolatedInput (cpu/src/interpolated_input.rs:12-23)
    float ig[3] = {0, 0, 0};
    std::vector<float> igoal, ivpos, ivnorm, itnorm, ifric, idamp;

    float forget_distance() const { return (float)dx * 2.2f; }  // file_input/src/header.rs:60-66
    float accept_distance() const { return (float)dx * 2.f; }

    void set_time(double t) override { time = t; }
    double get_time() const override { return time; }

    int set_frame_input(const svo_frame_input *in) override {
        FrameIn f;
        f.set = true;
        f.fps = in->frames_per_second, f.frame = in->frame, f.has_b = in->has_b != 0;
        for (int a = 0; a < 3; ++a) f.g_a[a] = in->gravity_a[a], f.g_b[a] = f.has_b ? in->gravity_b[a] : in->gravity_a[a];
        f.goals = in->goal_flags_a && in->goal_positions_a;
        if (f.goals) {
            f.gflag_a.assign(in->goal_flags_a, in->goal_flags_a + n);
            f.goal_a.assign(in->goal_positions_a, in->goal_positions_a + 3 * n);
            const bool hb = f.has_b && in->goal_flags_b && in->goal_positions_b;
            f.gflag_b = hb ? std::vector<uint32_t>(in->goal_flags_b, in->goal_flags_b + n) : f.gflag_a;
            f.goal_b = hb ? std::vector<float>(in->goal_positions_b, in->goal_positions_b + 3 * n) : f.goal_a;
        }
        f.nv = in->n_vertices, f.nt = in->n_triangles, f.leaf = in->leaf_size;
        if (f.nt) {
            f.tri.assign(in->triangles, in->triangles + 3 * f.nt);
            f.tri_col.assign(in->triangle_collider, in->triangle_collider + f.nt);
            f.va.assign(in->vertex_positions_a, in->vertex_positions_a + 3 * f.nv);
            f.vb = f.has_b ? std::vector<float>(in->vertex_positions_b, in->vertex_positions_b + 3 * f.nv) : f.va;
            f.fr_a.assign(in->friction_a, in->friction_a + f.nt);
            f.dm_a.assign(in->damping_a, in->damping_a + f.nt);
            f.fr_b = f.has_b ? std::vector<float>(in->friction_b, in->friction_b + f.nt) : f.fr_a;
            f.dm_b = f.has_b ? std::vector<float>(in->damping_b, in->damping_b + f.nt) : f.dm_a;
            for (uint32_t t = 0; t < f.nt; ++t) {
                if (f.tri_col[t] >= 16) return -1;
                for (int k = 0; k < 3; ++k)
                    if (f.tri[3 * t + k] >= f.nv) return -1;  // mesh.rs:37-47
            }
            // edge -> triangles (mesh.rs:49-68), opposites (mesh.rs:71-94)
            std::map<std::pair<uint32_t, uint32_t>, std::vector<uint32_t>> edges;
            auto edge = [](uint32_t a, uint32_t b) { return a < b ? std::make_pair(a, b) : std::make_pair(b, a); };
            for (uint32_t t = 0; t < f.nt; ++t)
                for (int k = 0; k < 3; ++k) edges[edge(f.tri[3 * t + k], f.tri[3 * t + (k + 1) % 3])].push_back(t);
            for (auto &e : edges)
                if (e.second.size() > 2) return -1;  // NonManifoldEdge
            f.opp.assign(3 * f.nt, 0xFFFFFFFFu);
            for (uint32_t t = 0; t < f.nt; ++t)
                for (int k = 0; k < 3; ++k)
                    for (uint32_t o : edges[edge(f.tri[3 * t + k], f.tri[3 * t + (k + 1) % 3])])
                        if (o != t) f.opp[3 * t + k] = o;
            // vertex -> triangles, emptied at vertices whose neighbour counts are not all 2
            f.vtris.assign(f.nv, {});
            for (uint32_t t = 0; t < f.nt; ++t)
                for (int k = 0; k < 3; ++k) f.vtris[f.tri[3 * t + k]].push_back(t);
            for (uint32_t v = 0; v < f.nv; ++v) {
                std::map<uint32_t, int> count;
                for (uint32_t t : f.vtris[v])
                    for (int k = 0; k < 3; ++k)
                        if (f.tri[3 * t + k] != v) ++count[f.tri[3 * t + k]];
                for (auto &c : count)
                    if (c.second != 2) {
                        f.vtris[v].clear();
                        break;
                    }
            }
            f.vvel.assign(3 * f.nv, 0.f);
            if (f.has_b)
                for (uint32_t k = 0; k < 3 * f.nv; ++k) f.vvel[k] = (f.vb[k] - f.va[k]) * (float)f.fps;
            const float margin = forget_distance();
            f.lmin.resize(3 * f.nt), f.lmax.resize(3 * f.nt);
            for (uint32_t t = 0; t < f.nt; ++t)
                for (int a = 0; a < 3; ++a) {
                    float lo = std::numeric_limits<float>::max(), hi = -lo;
                    for (int k = 0; k < 3; ++k) {
                        const uint32_t v = f.tri[3 * t + k];
                        lo = std::min(lo, f.va[3 * v + a]), hi = std::max(hi, f.va[3 * v + a]);
                        if (f.has_b) lo = std::min(lo, f.vb[3 * v + a]), hi = std::max(hi, f.vb[3 * v + a]);
                    }
                    f.lmin[3 * t + a] = (int32_t)std::floor((lo - margin) / f.leaf);
                    f.lmax[3 * t + a] = (int32_t)std::ceil((hi + margin) / f.leaf);
                }
        }
        fin = std::move(f);
        return 0;
    }

    static void f3_cross(const float a[3], const float b[3], float o[3]) {
        o[0] = a[1] * b[2] - a[2] * b[1], o[1] = a[2] * b[0] - a[0] * b[2], o[2] = a[0] * b[1] - a[1] * b[0];
    }
    static float f3_dot(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
    static float f3_norm(const float a[3]) { return std::sqrt(f3_dot(a, a)); }
    // nalgebra try_normalize(1e-5) (util/src/consts.rs:11 NORMALIZATION_EPS), zero on failure
    static void f3_normalize_or_zero(float a[3]) {
        const float nn = f3_norm(a);
        if (nn <= 1e-5f) a[0] = a[1] = a[2] = 0.f;
        else a[0] /= nn, a[1] /= nn, a[2] /= nn;
    }

    // cpu/src/phase/interpolate_input.rs:18-106 at the state's time
    int interpolate_input() {
        const double ft = time * (double)fin.fps;
        const double low = std::floor(ft);
        if ((int64_t)low != (int64_t)fin.frame) return -2;  // xpu frame_input.rs:266-278 WrongFrameLoaded
        const float fb = (float)std::fmod(ft, 1.0), fa = 1.f - fb;
        for (int a = 0; a < 3; ++a) ig[a] = fa * fin.g_a[a] + fb * fin.g_b[a];
        if (fin.goals) {
            igoal.resize(3 * n);
            for (size_t k = 0; k < 3 * n; ++k) igoal[k] = fa * fin.goal_a[k] + fb * fin.goal_b[k];
        }
        if (!fin.nt) return 0;
        ivpos.resize(3 * fin.nv);
        for (size_t k = 0; k < 3 * fin.nv; ++k) ivpos[k] = fa * fin.va[k] + fb * fin.vb[k];
        itnorm.assign(3 * fin.nt, 0.f);
        for (uint32_t t = 0; t < fin.nt; ++t) {
            const float *A = &ivpos[3 * fin.tri[3 * t]], *B = &ivpos[3 * fin.tri[3 * t + 1]], *C = &ivpos[3 * fin.tri[3 * t + 2]];
            const float ab[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]}, ac[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
            f3_cross(ab, ac, &itnorm[3 * t]);
            f3_normalize_or_zero(&itnorm[3 * t]);
        }
        ivnorm.assign(3 * fin.nv, 0.f);
        for (uint32_t v = 0; v < fin.nv; ++v) {
            float s[3] = {0, 0, 0};
            for (uint32_t t : fin.vtris[v]) {
                uint32_t others[2], m = 0;
                for (int k = 0; k < 3; ++k)
                    if (fin.tri[3 * t + k] != v && m < 2) others[m++] = fin.tri[3 * t + k];
                const float *P = &ivpos[3 * v], *A = &ivpos[3 * others[0]], *B = &ivpos[3 * others[1]];
                const float pa[3] = {A[0] - P[0], A[1] - P[1], A[2] - P[2]}, pb[3] = {B[0] - P[0], B[1] - P[1], B[2] - P[2]};
                // nalgebra angle: acos of the clamped cosine, 0 for a zero vector
                const float na = f3_norm(pa), nb = f3_norm(pb);
                float ang = 0.f;
                if (na != 0.f && nb != 0.f) {
                    const float c = f3_dot(pa, pb) / (na * nb);
                    ang = c > 1.f ? 0.f : (c < -1.f ? 3.14159265358979f : std::acos(c));
                }
                for (int a = 0; a < 3; ++a) s[a] += ang * itnorm[3 * t + a];
            }
            f3_normalize_or_zero(s);
            for (int a = 0; a < 3; ++a) ivnorm[3 * v + a] = s[a];
        }
        ifric.resize(fin.nt), idamp.resize(fin.nt);
        for (uint32_t t = 0; t < fin.nt; ++t)
            ifric[t] = fa * fin.fr_a[t] + fb * fin.fr_b[t], idamp[t] = fa * fin.dm_a[t] + fb * fin.dm_b[t];
        return 0;
    }

    // mesh_util/src/mesh.rs:247-308
    struct DistanceResult {
        float distance, to_p[3], normal[3];
    };
    static DistanceResult segment_result(const float p[3], const float s[3], const float e[3], const float sn[3],
                                         const float segn[3], const float en[3]) {
        const float seg[3] = {e[0] - s[0], e[1] - s[1], e[2] - s[2]};
        const float ps[3] = {p[0] - s[0], p[1] - s[1], p[2] - s[2]};
        const float along = f3_dot(ps, seg) / f3_dot(seg, seg);
        DistanceResult r;
        const float *nn;
        if (along < 0.f) {
            for (int a = 0; a < 3; ++a) r.to_p[a] = ps[a];
            nn = sn;
        } else if (along < 1.f) {
            for (int a = 0; a < 3; ++a) r.to_p[a] = p[a] - s[a] - seg[a] * along;
            nn = segn;
        } else {
            for (int a = 0; a < 3; ++a) r.to_p[a] = p[a] - e[a];
            nn = en;
        }
        r.distance = f3_norm(r.to_p);
        for (int a = 0; a < 3; ++a) r.normal[a] = nn[a];
        return r;
    }
    static float segment_distance(const float p[3], const float s[3], const float e[3]) {
        const float z[3] = {0, 0, 0};
        return segment_result(p, s, e, z, z, z).distance;
    }
    static float triangle_distance(const float p[3], const float A[3], const float B[3], const float C[3],
                                   const float nrm[3]) {
        const float ab[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
        const float bc[3] = {B[0] - C[0], B[1] - C[1], B[2] - C[2]};
        const float ca[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
        const float cp[3] = {C[0] - p[0], C[1] - p[1], C[2] - p[2]};
        const float ap[3] = {A[0] - p[0], A[1] - p[1], A[2] - p[2]};
        const float bp[3] = {B[0] - p[0], B[1] - p[1], B[2] - p[2]};
        float x[3];
        f3_cross(bc, cp, x);
        const bool sa = f3_dot(nrm, x) > 0.f;
        f3_cross(ca, ap, x);
        const bool sb = f3_dot(nrm, x) > 0.f;
        f3_cross(ab, bp, x);
        const bool sc = f3_dot(nrm, x) > 0.f;
        if (sa && sb && sc) {
            const float pa[3] = {p[0] - A[0], p[1] - A[1], p[2] - A[2]};
            return std::fabs(f3_dot(pa, nrm));
        }
        float d = std::numeric_limits<float>::max();
        if (!sa) d = std::min(d, segment_distance(p, B, C));
        if (!sb) d = std::min(d, segment_distance(p, C, A));
        if (!sc) d = std::min(d, segment_distance(p, A, B));
        return d;
    }

    // util/src/collider_bits.rs:9-38
    static bool cb_near(uint32_t b, int c) { return (b & (0x00010000u << c)) != 0; }
    static bool cb_side(uint32_t b, int c) { return (b & (0x00000001u << c)) != 0; }
    static void cb_set(uint32_t &b, int c, int side) {  // side: -1 None, 0 false, 1 true
        b &= ~(0x00010001u << c);
        if (side == 1) b |= 0x00010001u << c;
        else if (side == 0) b |= 0x00010000u << c;
    }

    // cpu/src/phase/collide.rs:21-206.  The BVH query of the reference
    // returns a superset of the triangles whose padded leaf box holds the
    // particle's leaf cell; here that set itself is scanned, in index order.
    void collide(T dt_t) {
        if (!fin.nt) return;
        const float dt = (float)dt_t, forget = forget_distance(), accept = accept_distance();
        pool.run(n, [&](size_t b, size_t e, int) {
            for (size_t p = b; e > p; ++p) {
                if (flags[p] & TOMBSTONED) continue;
                const float P[3] = {(float)x[p][0], (float)x[p][1], (float)x[p][2]};
                int32_t leaf[3];
                for (int a = 0; a < 3; ++a) leaf[a] = (int32_t)std::floor(P[a] / fin.leaf);
                uint32_t closest[16];
                float mind[16];
                bool any = false;
                for (int c = 0; c < 16; ++c) closest[c] = 0xFFFFFFFFu, mind[c] = std::numeric_limits<float>::max();
                for (uint32_t t = 0; t < fin.nt; ++t) {
                    bool in = true;
                    for (int a = 0; a < 3; ++a) in = in && fin.lmin[3 * t + a] <= leaf[a] && leaf[a] <= fin.lmax[3 * t + a];
                    if (!in) continue;
                    any = true;
                    const float *nrm = &itnorm[3 * t];
                    if (nrm[0] == 0.f && nrm[1] == 0.f && nrm[2] == 0.f) continue;
                    const float *A = &ivpos[3 * fin.tri[3 * t]], *B = &ivpos[3 * fin.tri[3 * t + 1]], *C = &ivpos[3 * fin.tri[3 * t + 2]];
                    const float d = triangle_distance(P, A, B, C, nrm);
                    if (d >= forget) continue;
                    const uint32_t c = fin.tri_col[t];
                    if (d < mind[c]) mind[c] = d, closest[c] = t;
                }
                if (!any) {
                    collider_bits[p] = 0;
                    continue;
                }
                float vel[3] = {(float)v[p][0], (float)v[p][1], (float)v[p][2]};
                uint32_t bits = collider_bits[p];
                for (int c = 0; c < 16; ++c) {
                    if (closest[c] == 0xFFFFFFFFu) {
                        cb_set(bits, c, -1);
                        continue;
                    }
                    const uint32_t t = closest[c];
                    const uint32_t ia = fin.tri[3 * t], ib = fin.tri[3 * t + 1], ic = fin.tri[3 * t + 2];
                    const float *nrm = &itnorm[3 * t];
                    const float *A = &ivpos[3 * ia], *B = &ivpos[3 * ib], *C = &ivpos[3 * ic];
                    float abn[3] = {0, 0, 0}, bcn[3] = {0, 0, 0}, can[3] = {0, 0, 0};
                    const uint32_t *o = &fin.opp[3 * t];
                    if (o[0] != 0xFFFFFFFFu)
                        for (int a = 0; a < 3; ++a) abn[a] = nrm[a] + itnorm[3 * o[0] + a];
                    if (o[1] != 0xFFFFFFFFu)
                        for (int a = 0; a < 3; ++a) bcn[a] = nrm[a] + itnorm[3 * o[1] + a];
                    if (o[2] != 0xFFFFFFFFu)
                        for (int a = 0; a < 3; ++a) can[a] = nrm[a] + itnorm[3 * o[2] + a];
                    const float ab[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
                    const float bc[3] = {B[0] - C[0], B[1] - C[1], B[2] - C[2]};
                    const float ca[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
                    float x1[3];
                    f3_cross(ca, ab, x1);
                    const float area2 = f3_dot(nrm, x1);
                    const float cp[3] = {C[0] - P[0], C[1] - P[1], C[2] - P[2]};
                    const float ap[3] = {A[0] - P[0], A[1] - P[1], A[2] - P[2]};
                    const float bp[3] = {B[0] - P[0], B[1] - P[1], B[2] - P[2]};
                    f3_cross(bc, cp, x1);
                    const float ba = f3_dot(nrm, x1) / area2;
                    f3_cross(ca, ap, x1);
                    const float bb = f3_dot(nrm, x1) / area2;
                    f3_cross(ab, bp, x1);
                    const float bcb = f3_dot(nrm, x1) / area2;
                    DistanceResult r;
                    if (ba > 0.f && bb > 0.f && bcb > 0.f) {
                        const float pa[3] = {P[0] - A[0], P[1] - A[1], P[2] - A[2]};
                        const float h = f3_dot(pa, nrm);
                        r.distance = std::fabs(h);
                        for (int a = 0; a < 3; ++a) r.to_p[a] = nrm[a] * h, r.normal[a] = nrm[a];
                    } else {
                        const float *na = &ivnorm[3 * ia], *nb = &ivnorm[3 * ib], *nc = &ivnorm[3 * ic];
                        const DistanceResult r1 = segment_result(P, A, B, na, abn, nb);
                        const DistanceResult r2 = segment_result(P, B, C, nb, bcn, nc);
                        const DistanceResult r3 = segment_result(P, C, A, nc, can, na);
                        r = r1;  // min_by(total_cmp): the first of equal distances
                        if (r2.distance < r.distance) r = r2;
                        if (r3.distance < r.distance) r = r3;
                    }
                    if (r.normal[0] == 0.f && r.normal[1] == 0.f && r.normal[2] == 0.f) {
                        cb_set(bits, c, -1);
                        continue;
                    }
                    const bool new_side = 0.f <= f3_dot(r.to_p, r.normal);
                    if (!cb_near(bits, c)) {
                        if (r.distance < accept) cb_set(bits, c, new_side ? 1 : 0);
                        continue;
                    }
                    if (cb_side(bits, c) == new_side) continue;
                    if (r.distance > 1e-5f) {
                        float cv[3], rel[3], cn[3], nv[3], tv[3];
                        for (int a = 0; a < 3; ++a) {
                            cv[a] = fin.vvel[3 * ia + a] * ba + fin.vvel[3 * ib + a] * bb + fin.vvel[3 * ic + a] * bcb;
                            rel[a] = vel[a] - cv[a];
                            cn[a] = r.to_p[a] / r.distance;
                        }
                        const float rn = f3_dot(rel, cn);
                        for (int a = 0; a < 3; ++a) nv[a] = cn[a] * rn, tv[a] = rel[a] - nv[a];
                        const float tvn = f3_norm(tv);
                        if (tvn > 1e-5f) {
                            const float mag = std::min(ifric[t] * r.distance / dt, tvn);
                            for (int a = 0; a < 3; ++a) vel[a] -= tv[a] / tvn * mag;
                        }
                        const float dmp = std::min(idamp[t], 1.f);
                        for (int a = 0; a < 3; ++a) vel[a] -= dmp * nv[a];
                    }
                    for (int a = 0; a < 3; ++a) vel[a] -= r.to_p[a] / dt;
                }
                collider_bits[p] = bits;
                for (int a = 0; a < 3; ++a) v[p][a] = (T)vel[a];
            }
        });
    }

    // ---- adaptive time steps
    // cpu/src/adaptive_time_step_state.rs:13-64: each limit is an Option<f32>
    // (has_* false = None), the prior limits a deque of at most 11.
    struct Adaptive {
        float max_dt = std::numeric_limits<float>::max();
        bool has_vel = false, has_def = false, has_sound = false, has_iso = false;
        float vel = 0, def = 0, sound = 0, iso = 0;
        std::deque<float> prior;
        float without_prior() const {
            const float big = std::numeric_limits<float>::max();
            float r = max_dt;
            r = std::min(r, has_vel ? vel : big);
            r = std::min(r, has_def ? def : big);
            r = std::min(r, has_sound ? sound : big);
            r = std::min(r, has_iso ? iso : big);
            return r;
        }
        float allowed() const {
            float r = without_prior();
            for (float p : prior) r = std::min(r, p);
            return r;
        }
        void push() {
            if (prior.size() > 10) prior.pop_front();
            prior.push_back(without_prior());
        }
    } ad;

    // singular values of F, descending
    V3<T> singular_values(const M3<T> &f) const {
        M3<T> U, V;
        V3<T> s;
        svd3(f, U, s, V);
        return s;
    }

    // cpu/src/phase/limit_time_step.rs:36-123, in f32 like the reference
    // (T = f32 there): dx / c, c from the largest of six stiffness terms.
    static float sound_speed_limit(const Params &q, bool fluid, const float s[3], float dx) {
        const float x = s[0], y = s[1], z = s[2];
        const float j = x * y * z;
        // partial_invariant_3_by_svd and double_partial_invariant_3_by_svd (elastic.rs:123-141)
        const float g3[3] = {y * z, x * z, x * y};
        const float h3[3][3] = {{0, z, y}, {z, 0, x}, {y, x, 0}};
        float first[3], second[3][3];
        if (!fluid) {
            // elastic.rs:314-339: dPsi/dI2 = mu / 2, dPsi/dI3 and d2Psi/dI3^2 of 276-295
            const float e3 = (q.lambda * std::log(j) - q.mu) / j;
            const float ee3 = (q.lambda * (1.f - std::log(j)) + q.mu) / (j * j);
            for (int a = 0; a < 3; ++a) {
                first[a] = q.mu / 2.f * 2.f * s[a] + e3 * g3[a];
                for (int b = 0; b < 3; ++b) second[a][b] = (a == b ? q.mu / 2.f * 2.f : 0.f) + ee3 * g3[a] * g3[b] + e3 * h3[a][b];
            }
        } else {
            // elastic.rs:555-570 and 630-654
            const float e3 = q.bulk_modulus * (1.f - 1.f / powi<float>(j, q.exponent));
            const float ee3 = (float)q.exponent * q.bulk_modulus / powi<float>(j, q.exponent + 1);
            for (int a = 0; a < 3; ++a) {
                first[a] = e3 * g3[a];
                for (int b = 0; b < 3; ++b) second[a][b] = ee3 * g3[a] * g3[b] + e3 * h3[a][b];
            }
        }
        const float sep = 1e-5f;  // util/src/consts.rs:14
        const bool xy = std::fabs(x - y) < sep, yz = std::fabs(y - z) < sep, zx = std::fabs(z - x) < sep;
        const float terms[6] = {
            x * x * second[0][0],
            y * y * second[1][1],
            z * z * second[2][2],
            y * y * (xy ? (first[0] + x * second[0][0] - y * second[1][0]) / 2.f / x : (x * first[0] - y * first[1]) / (x * x - y * y)),
            y * z * (yz ? (first[1] + y * second[1][1] - z * second[2][1]) / 2.f / y : (y * first[1] - z * first[2]) / (y * y - z * z)),
            z * x * (zx ? (first[2] + x * second[2][2] - x * second[0][2]) / 2.f / z : (z * first[2] - x * first[0]) / (z * z - x * x)),
        };
        float kappa = terms[0];
        for (int k = 1; k < 6; ++k) kappa = std::max(kappa, terms[k]);
        kappa /= j;
        const float density = q.mass / q.initial_volume / j;
        return dx / std::sqrt(kappa / density);
    }

    // limit_time_step.rs:126-178
    static float isolated_limit(const Params &q, bool fluid, float det, float dx) {
        if (!fluid) {
            const float xi = 3.f / dx / dx;
            return std::sqrt(q.mass / (q.initial_volume * xi * (1.f - 1.f / 2.f) * (q.mu + 3.f / 2.f * q.lambda)));
        }
        const float rho0 = q.mass / q.initial_volume;
        const float first = q.bulk_modulus * (1.f - 1.f / powi<float>(det, q.exponent));
        if (std::fabs(det - 1.f) > 1e-5f) return dx / det * std::sqrt(rho0 * (det - 1.f) / (6.f * first * 3.f));
        const float second = (float)q.exponent * q.bulk_modulus / powi<float>(det, q.exponent + 1);
        return dx * std::sqrt(rho0 / (6.f * second * 3.f));
    }

    // limit_time_step.rs:25-33.  Non-finite candidates are skipped (the
    // reference's total_cmp would order a NaN first).
    void limit_time_step_before_force() {
        const float dxf = (float)dx;
        float sound = std::numeric_limits<float>::max(), iso = sound;
        bool any = false;
        for (size_t p = 0; p < n; ++p) {
            if (flags[p] & TOMBSTONED) continue;
            any = true;
            const bool fluid = (flags[p] & IS_FLUID) != 0;
            const V3<T> sv = singular_values(F[p]);
            const float s[3] = {(float)sv[0], (float)sv[1], (float)sv[2]};
            const float a = sound_speed_limit(params[p], fluid, s, dxf);
            const float b = isolated_limit(params[p], fluid, (float)det(F[p]), dxf);
            if (std::isfinite(a) && a > 0) sound = std::min(sound, a);
            if (std::isfinite(b) && b > 0) iso = std::min(iso, b);
        }
        ad.has_sound = any && sound < std::numeric_limits<float>::max(), ad.sound = sound;
        ad.has_iso = any && iso < std::numeric_limits<float>::max(), ad.iso = iso;
        ad.push();
    }

    // limit_time_step.rs:181-222
    void limit_time_step_before_integrate() {
        float max_vel = 0, max_c = 0;
        bool any = false;
        for (size_t p = 0; p < n; ++p) {
            if (flags[p] & TOMBSTONED) continue;
            any = true;
            const float vx = (float)v[p][0], vy = (float)v[p][1], vz = (float)v[p][2];
            max_vel = std::max(max_vel, std::sqrt(vx * vx + vy * vy + vz * vz));
            for (int k = 0; k < 9; ++k) max_c = std::max(max_c, std::fabs((float)C[p].m[k]));
        }
        ad.has_vel = any && max_vel != 0.f, ad.vel = ad.has_vel ? 0.5f * (float)dx / max_vel : 0.f;
        ad.has_def = any, ad.def = 0.2f / std::max(max_c, 1e-8f);
        ad.push();
    }

    // cpu/src/cpu_state.rs:146-197 with adaptive_time_steps = true and the
    // phase order of cpu/src/phase/mod.rs:27-41.  Returns 1 on an energy
    // error (time not advanced for that substep), 2 on a zero time step, 3 on
    // a sand particle compressed with mu <= 0 (the reference's assert).
    int step_adaptive(double *time, double target, float max_dt, const float g_f[3], uint32_t *substeps,
                      float limits[8]) override {
        ad.max_dt = max_dt;
        uint32_t done = 0;
        int rc = 0;
        float dt_a = 0, dt_b = 0, dt_c = 0;
        this->time = *time;
        while (*time < target) {
            if (ad.allowed() == 0.f) {
                rc = 2;
                break;
            }
            this->time = *time;
            if (fin.set && interpolate_input()) {
                rc = -2;
                break;
            }
            const V3<T> g = substep_gravity(g_f);
            sort();
            dt_a = ad.allowed();
            collide((T)dt_a);
            external_force((T)dt_a, g);
            update_grid_nodes();
            limit_time_step_before_force();
            dt_b = ad.allowed();
            scatter_momentum((T)dt_b);
            meld_grid();
            collect_velocity();
            limit_time_step_before_integrate();
            dt_c = ad.allowed();
            if (advance_particles((T)dt_c) > 0) {
                rc = 1;
                ++done;
                break;
            }
            if (sand_mu_error) {
                rc = 3;
                ++done;
                break;
            }
            cull_particles();
            *time += (double)ad.allowed();
            this->time = *time;
            ++done;
        }
        if (substeps) *substeps = done;
        if (limits) {
            const float big = std::numeric_limits<float>::max();
            limits[0] = dt_a, limits[1] = dt_b, limits[2] = dt_c;
            limits[3] = ad.has_vel ? ad.vel : big, limits[4] = ad.has_def ? ad.def : big;
            limits[5] = ad.has_sound ? ad.sound : big, limits[6] = ad.has_iso ? ad.iso : big;
            limits[7] = ad.allowed();
        }
        return rc;
    }

    void p2g_only(float dt_f, const float g_f[3]) override {
        T dt = (T)dt_f;
        V3<T> g = v3<T>((T)g_f[0], (T)g_f[1], (T)g_f[2]);
        sort();
        auto v_saved = v;
        external_force(dt, g);
        update_grid_nodes();
        scatter_momentum(dt);
        meld_grid();
        v = v_saved;
    }

    void download(svo_particles *o) override {
        for (size_t cur = 0; cur < n; ++cur) {
            size_t i = sort_map[cur];
            o->flags[i] = flags[cur];
            for (int a = 0; a < 3; ++a) o->positions[3 * i + a] = (float)x[cur][a], o->velocities[3 * i + a] = (float)v[cur][a];
            for (int a = 0; a < 9; ++a)
                o->position_gradients[9 * i + a] = (float)F[cur].m[a], o->velocity_gradients[9 * i + a] = (float)C[cur].m[a];
            if (o->elastic_energies) o->elastic_energies[i] = (float)energy[cur];
            if (o->collider_bits) o->collider_bits[i] = collider_bits[cur];
            if (o->plastic_j) o->plastic_j[i] = (float)plastic_j[cur];
        }
    }

    uint64_t grid(int32_t *ids, float *mo, float *vo, uint64_t cap) override {
        std::vector<uint32_t> idx;
        for (size_t i = 0; i < keys.size(); ++i)
            if (masses.size() == keys.size() && masses[i] > T(0)) idx.push_back((uint32_t)i);
        std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
        for (size_t c = 0; c < idx.size() && c < cap; ++c) {
            const GridKey &k = keys[idx[c]];
            ids[3 * c] = k.i, ids[3 * c + 1] = k.j, ids[3 * c + 2] = k.k;
            mo[c] = (float)masses[idx[c]];
            for (int a = 0; a < 3; ++a) vo[3 * c + a] = (float)velocities[idx[c]][a];
        }
        return idx.size();
    }
};

template <class T> M3<T> load9(const double *a) {
    M3<T> m;
    for (int i = 0; i < 9; ++i) m.m[i] = (T)a[i];
    return m;
}
template <class T> void store9(const M3<T> &m, double *a) {
    for (int i = 0; i < 9; ++i) a[i] = (double)m.m[i];
}

}  // namespace svo

using namespace svo;

extern "C" {

double svo_mu(double E, double nu) { return lame_mu(E, nu); }
double svo_lambda(double E, double nu) { return lame_lambda(E, nu); }
double svo_kernel_quadratic(double x) { return kernel_quadratic(x); }
double svo_energy_neo_hookean(double mu, double lambda, const double F[9]) {
    return energy_neo_hookean(mu, lambda, load9<double>(F));
}
void svo_piola_neo_hookean(double mu, double lambda, const double F[9], double P[9]) {
    store9(piola_neo_hookean(mu, lambda, load9<double>(F)), P);
}
double svo_energy_inviscid(double K, int32_t gamma, const double F[9]) {
    return energy_inviscid(K, gamma, det(load9<double>(F)));
}
void svo_piola_inviscid(double K, int32_t gamma, const double F[9], double P[9]) {
    store9(piola_inviscid(K, gamma, load9<double>(F)), P);
}
double svo_energy_fixed_corotated(double mu, double lambda, const double F[9]) {
    return energy_fixed_corotated(mu, lambda, load9<double>(F));
}
void svo_piola_fixed_corotated(double mu, double lambda, const double F[9], double P[9]) {
    store9(piola_fixed_corotated(mu, lambda, load9<double>(F)), P);
}
void svo_cauchy_viscosity(double dyn, double bulk, const double C[9], double S[9]) {
    store9(cauchy_viscosity(dyn, bulk, load9<double>(C)), S);
}
void svo_svd3(const double F[9], double U[9], double S[3], double V[9]) {
    M3<double> u, v;
    V3<double> s;
    svd3(load9<double>(F), u, s, v);
    store9(u, U), store9(v, V);
    for (int i = 0; i < 3; ++i) S[i] = s[i];
}
int svo_project_sand(double mu, double lambda, double alpha, double F[9]) {
    M3<double> f = load9<double>(F);
    if (!project_sand(mu, lambda, alpha, f)) return -1;
    store9(f, F);
    return 0;
}
void svo_project_fluid(double F[9]) {
    M3<double> f = load9<double>(F);
    project_fluid(f);
    store9(f, F);
}
void svo_project_snow(double theta_c, double theta_s, double F[9], double *plastic_j) {
    M3<double> f = load9<double>(F);
    project_snow(theta_c, theta_s, f, *plastic_j);
    store9(f, F);
}
// Not in the reference (whose "Sand Alpha" is a raw input): Drucker-Prager
// cone coefficient from a friction angle, alpha = sqrt(2/3) 2 sin(phi) /
// (3 - sin(phi)) (Klar et al. 2016).
double svo_friction_angle_to_alpha(double phi) {
    double s = std::sin(phi);
    return std::sqrt(2.0 / 3.0) * 2.0 * s / (3.0 - s);
}

void *svo_create(const svo_particles *p, const svo_consts *c, int fp64, int threads) {
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    if (fp64) return static_cast<Base *>(new State<double>(p, c, threads));
    return static_cast<Base *>(new State<float>(p, c, threads));
}
void svo_destroy(void *s) { delete static_cast<Base *>(s); }
int svo_step(void *s, uint32_t n, float dt, const float g[3]) { return static_cast<Base *>(s)->step(n, dt, g); }
int svo_step_adaptive(void *s, double *time, double target, float max_dt, const float g[3], uint32_t *substeps,
                      float limits[8]) {
    return static_cast<Base *>(s)->step_adaptive(time, target, max_dt, g, substeps, limits);
}
int svo_set_frame_input(void *s, const svo_frame_input *in) { return static_cast<Base *>(s)->set_frame_input(in); }
void svo_set_time(void *s, double time) { static_cast<Base *>(s)->set_time(time); }
double svo_get_time(void *s) { return static_cast<Base *>(s)->get_time(); }
void svo_download(void *s, svo_particles *out) { static_cast<Base *>(s)->download(out); }
uint64_t svo_grid(void *s, int32_t *ids, float *m, float *v, uint64_t cap) {
    return static_cast<Base *>(s)->grid(ids, m, v, cap);
}
void svo_p2g_only(void *s, float dt, const float g[3]) { static_cast<Base *>(s)->p2g_only(dt, g); }

void svo_binning_keys(uint64_t n, const float *pos, const uint32_t *flags, float dx, const int32_t origin[3],
                      const int32_t nb[3], uint32_t *keys) {
    for (uint64_t p = 0; p < n; ++p) {
        if (flags && (flags[p] & TOMBSTONED)) {
            keys[p] = 0xFFFFFFFFu;
            continue;
        }
        int32_t lc[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
            float q = pos[3 * p + a] / dx - 0.5f;
            lc[a] = (int32_t)std::floor(q) - origin[a];
            ok = ok && lc[a] >= 0 && (lc[a] >> 2) < nb[a];
        }
        if (!ok) {
            keys[p] = 0xFFFFFFFFu;
            continue;
        }
        uint32_t block = ((uint32_t)(lc[0] >> 2) * (uint32_t)nb[1] + (uint32_t)(lc[1] >> 2)) * (uint32_t)nb[2] +
                         (uint32_t)(lc[2] >> 2);
        keys[p] = block << 6 | (uint32_t)((lc[0] & 3) << 4 | (lc[1] & 3) << 2 | (lc[2] & 3));
    }
}

void svo_stable_sort_perm(uint64_t n, const uint32_t *keys, uint32_t *perm) {
    for (uint64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    std::stable_sort(perm, perm + n, [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
}

// The reference's P2G mass (rust/crates/cpu/src/phase/scatter_momentum.rs:
// 22-93: w = kernel(n - x/dx) per axis, kernels.rs:17-26, times the mass)
// with each node's sum taken in one canonical order, in fp32, left to right:
// over the 27 base cells c = n - (i, j, k), (i, j, k) in lexicographic order
// (i outermost), and within a cell over its particles in ascending index.
// The base cell is kernels.rs:46-49's floor(x/dx - 1/2).  Tombstoned
// particles take no part.  Writes the nodes with mass > 0 in ascending
// (i, j, k) order, at most `cap`; returns their count.
uint64_t svo_deterministic_grid_mass(const float *pos, const float *mass, const uint32_t *flags, uint64_t n, float dx,
                                     int32_t *ids, float *masses, uint64_t cap) {
    std::map<std::array<int32_t, 3>, std::vector<uint32_t>> cells;  // base cell -> particles, ascending
    for (uint64_t p = 0; p < n; ++p) {
        if (flags[p] & TOMBSTONED) continue;
        std::array<int32_t, 3> c;
        for (int a = 0; a < 3; ++a) c[a] = (int32_t)std::floor(pos[3 * p + a] / dx - 0.5f);
        cells[c].push_back((uint32_t)p);
    }
    std::vector<std::array<int32_t, 3>> nodes;
    for (auto &kv : cells)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) nodes.push_back({kv.first[0] + i, kv.first[1] + j, kv.first[2] + k});
    std::sort(nodes.begin(), nodes.end());
    nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
    uint64_t count = 0;
    for (auto &nd : nodes) {
        float sum = 0.f;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    auto it = cells.find({nd[0] - i, nd[1] - j, nd[2] - k});
                    if (it == cells.end()) continue;
                    for (uint32_t p : it->second) {
                        float w = 1.f;
                        for (int a = 0; a < 3; ++a) {
                            const float r = (float)nd[a] - pos[3 * p + a] / dx;
                            w = a == 0 ? kernel_quadratic<float>(r) : w * kernel_quadratic<float>(r);
                        }
                        sum = sum + w * mass[p];
                    }
                }
        if (!(sum > 0.f)) continue;
        if (count < cap && ids && masses) {
            for (int a = 0; a < 3; ++a) ids[3 * count + a] = nd[a];
            masses[count] = sum;
        }
        ++count;
    }
    return count;
}

}  // extern "C"
