// sv_eig.cuh -- closed-form eigen-decomposition of a symmetric 3x3 matrix
// (host and device): the learned closure's principal stretches.
#pragma once
#include <math.h>

namespace sv {

// ------------------------------------------------------------------ eigen
// Eigen-decomposition of a symmetric 3x3 matrix in closed form, after
// D. Eberly, "A Robust Eigensolver for 3x3 Symmetric Matrices" (Geometric
// Tools, 2014): eigenvalues from the trigonometric solution of the
// characteristic cubic of the scaled, shifted matrix; the eigenvector of the
// best-separated eigenvalue from the longest cross product of two rows of
// A - lambda I; the next one from the 2x2 problem in that vector's orthogonal
// complement; the last by a cross product.  a = (a00, a01, a02, a11, a12,
// a22).  Eigenvalues come out descending, V's columns (column-major a[c*3+r])
// are the matching unit eigenvectors.
__host__ __device__ inline void sym_eig3(const float a_in[6], float lam[3], float V[9]) {
    float m = fmaxf(fmaxf(fmaxf(fabsf(a_in[0]), fabsf(a_in[1])), fmaxf(fabsf(a_in[2]), fabsf(a_in[3]))),
                    fmaxf(fabsf(a_in[4]), fabsf(a_in[5])));
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.f : 0.f;
    if (!(m > 0.f)) {
        lam[0] = lam[1] = lam[2] = 0.f;
        return;
    }
    const float s = 1.f / m;
    const float a00 = a_in[0] * s, a01 = a_in[1] * s, a02 = a_in[2] * s, a11 = a_in[3] * s, a12 = a_in[4] * s,
                a22 = a_in[5] * s;
    const float norm = a01 * a01 + a02 * a02 + a12 * a12;
    const float q = (a00 + a11 + a22) / 3.f;
    const float b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
    const float p = sqrtf((b00 * b00 + b11 * b11 + b22 * b22 + 2.f * norm) / 6.f);
    if (!(p > 0.f)) {
        lam[0] = lam[1] = lam[2] = q * m;
        return;
    }
    // det((A - qI) / p), formed from the divided entries so that a tiny p
    // (A close to a multiple of I) cannot underflow
    const float ip = 1.f / p;
    const float d00 = b00 * ip, d11 = b11 * ip, d22 = b22 * ip, d01 = a01 * ip, d02 = a02 * ip, d12 = a12 * ip;
    const float det = d00 * (d11 * d22 - d12 * d12) - d01 * (d01 * d22 - d12 * d02) + d02 * (d01 * d12 - d11 * d02);
    const float half = fminf(fmaxf(0.5f * det, -1.f), 1.f);
    const float ang = acosf(half) / 3.f;
    const float two_thirds_pi = 2.09439510239319549f;
    const float beta2 = 2.f * cosf(ang), beta0 = 2.f * cosf(ang + two_thirds_pi);
    const float beta1 = -(beta0 + beta2);
    // ascending eigenvalues of the scaled matrix
    const float al[3] = {q + p * beta0, q + p * beta1, q + p * beta2};
    const float A[3][3] = {{a00, a01, a02}, {a01, a11, a12}, {a02, a12, a22}};
    auto cross = [](const float u[3], const float v[3], float w[3]) {
        w[0] = u[1] * v[2] - u[2] * v[1];
        w[1] = u[2] * v[0] - u[0] * v[2];
        w[2] = u[0] * v[1] - u[1] * v[0];
    };
    // eigenvector of the eigenvalue `e` that is well separated from the others
    auto vec0 = [&](float e, float out[3]) {
        // rows of A - e I, scaled to a largest entry of 1 so that their cross
        // products cannot underflow when A is close to a multiple of I
        float r0[3] = {A[0][0] - e, A[0][1], A[0][2]};
        float r1[3] = {A[1][0], A[1][1] - e, A[1][2]};
        float r2[3] = {A[2][0], A[2][1], A[2][2] - e};
        float rm = 0.f;
        for (int k = 0; k < 3; ++k) rm = fmaxf(rm, fmaxf(fabsf(r0[k]), fmaxf(fabsf(r1[k]), fabsf(r2[k]))));
        if (!(rm > 0.f)) {
            out[0] = 1.f, out[1] = 0.f, out[2] = 0.f;
            return;
        }
        const float irm = 1.f / rm;
        for (int k = 0; k < 3; ++k) r0[k] *= irm, r1[k] *= irm, r2[k] *= irm;
        float x0[3], x1[3], x2[3];
        cross(r0, r1, x0);
        cross(r0, r2, x1);
        cross(r1, r2, x2);
        const float d0 = x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2];
        const float d1 = x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2];
        const float d2 = x2[0] * x2[0] + x2[1] * x2[1] + x2[2] * x2[2];
        const float *best = x0;
        float dm = d0;
        if (d1 > dm) best = x1, dm = d1;
        if (d2 > dm) best = x2, dm = d2;
        if (!(dm > 0.f)) {
            out[0] = 1.f, out[1] = 0.f, out[2] = 0.f;
            return;
        }
        const float inv = 1.f / sqrtf(dm);
        out[0] = best[0] * inv, out[1] = best[1] * inv, out[2] = best[2] * inv;
    };
    // eigenvector of `e` orthogonal to the unit vector w
    auto vec1 = [&](const float w[3], float e, float out[3]) {
        float u[3], v[3];
        if (fabsf(w[0]) > fabsf(w[1])) {
            const float inv = 1.f / sqrtf(w[0] * w[0] + w[2] * w[2]);
            u[0] = -w[2] * inv, u[1] = 0.f, u[2] = w[0] * inv;
        } else {
            const float inv = 1.f / sqrtf(w[1] * w[1] + w[2] * w[2]);
            u[0] = 0.f, u[1] = w[2] * inv, u[2] = -w[1] * inv;
        }
        cross(w, u, v);
        float au[3], av[3];
        for (int r = 0; r < 3; ++r) {
            au[r] = A[r][0] * u[0] + A[r][1] * u[1] + A[r][2] * u[2];
            av[r] = A[r][0] * v[0] + A[r][1] * v[1] + A[r][2] * v[2];
        }
        float m00 = u[0] * au[0] + u[1] * au[1] + u[2] * au[2] - e;
        float m01 = u[0] * av[0] + u[1] * av[1] + u[2] * av[2];
        float m11 = v[0] * av[0] + v[1] * av[1] + v[2] * av[2] - e;
        const float x00 = fabsf(m00), x01 = fabsf(m01), x11 = fabsf(m11);
        float cu = 1.f, cv = 0.f;  // out = cu u + cv v
        if (x00 >= x11) {
            if (fmaxf(x00, x01) > 0.f) {
                if (x00 >= x01) {
                    m01 /= m00;
                    m00 = 1.f / sqrtf(1.f + m01 * m01);
                    m01 *= m00;
                } else {
                    m00 /= m01;
                    m01 = 1.f / sqrtf(1.f + m00 * m00);
                    m00 *= m01;
                }
                cu = m01, cv = -m00;
            }
        } else {
            if (fmaxf(x11, x01) > 0.f) {
                if (x11 >= x01) {
                    m01 /= m11;
                    m11 = 1.f / sqrtf(1.f + m01 * m01);
                    m01 *= m11;
                } else {
                    m11 /= m01;
                    m01 = 1.f / sqrtf(1.f + m11 * m11);
                    m11 *= m01;
                }
                cu = m11, cv = -m01;
            }
        }
        out[0] = cu * u[0] + cv * v[0], out[1] = cu * u[1] + cv * v[1], out[2] = cu * u[2] + cv * v[2];
    };
    float e0[3], e1[3], e2[3];  // eigenvectors of al[0], al[1], al[2]
    if (half >= 0.f) {
        vec0(al[2], e2);
        vec1(e2, al[1], e1);
        cross(e1, e2, e0);
    } else {
        vec0(al[0], e0);
        vec1(e0, al[1], e1);
        cross(e0, e1, e2);
    }
    // eigenvalues as Rayleigh quotients of the eigenvectors: the cubic's
    // trigonometric roots lose accuracy at a double root, the vectors do not
    auto rq = [&](const float v[3]) {
        float s = 0.f;
        for (int r = 0; r < 3; ++r) s += v[r] * (A[r][0] * v[0] + A[r][1] * v[1] + A[r][2] * v[2]);
        return s;
    };
    lam[0] = rq(e2) * m, lam[1] = rq(e1) * m, lam[2] = rq(e0) * m;
    for (int r = 0; r < 3; ++r) V[r] = e2[r], V[3 + r] = e1[r], V[6 + r] = e0[r];
}

}  // namespace sv
