// Per-tet mixed-FEM math of the global step, fp32, one tet per thread.
//
// Everything here is written for registers: fixed-size arrays indexed by
// compile-time constants after unrolling.  The functions are host+device so
// the same arithmetic can be exercised off the GPU.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define MFEM_HD __host__ __device__ __forceinline__
#else
#define MFEM_HD inline
#endif

namespace mfem {
namespace em {

// SYM = diag(1,1,1,2,2,2), INV_SYM = diag(1,1,1,.5,.5,.5)
// (src/mfem/refinement/utils.py:4-5); sym6 order (xx, yy, zz, xy, xz, yz).
MFEM_HD float sym_w(int i) { return i < 3 ? 1.0f : 2.0f; }
MFEM_HD float inv_sym_w(int i) { return i < 3 ? 1.0f : 0.5f; }

MFEM_HD constexpr int p21(int i, int j) {
    return (i <= j) ? (i * 6 - (i * (i - 1)) / 2 + (j - i)) : (j * 6 - (j * (j - 1)) / 2 + (i - j));
}

// Scalar helpers that pick the float or double function, so the polar
// decomposition below serves both precisions from one source.
MFEM_HD float sqrt_r(float v) { return sqrtf(v); }
MFEM_HD double sqrt_r(double v) { return sqrt(v); }
MFEM_HD float abs_r(float v) { return fabsf(v); }
MFEM_HD double abs_r(double v) { return fabs(v); }
MFEM_HD float max_r(float a, float b) { return fmaxf(a, b); }
MFEM_HD double max_r(double a, double b) { return fmax(a, b); }
MFEM_HD float sign_r(float v) { return copysignf(1.0f, v); }
MFEM_HD double sign_r(double v) { return copysign(1.0, v); }

// Below this ratio of the second to the first column norm the QR step of the
// SVD takes any unit vector orthogonal to u0 (a tet collapsed onto a line).
template <class Real>
struct QrTiny;
template <>
struct QrTiny<float> {
    static constexpr float value = 1.0e-7f;
};
template <>
struct QrTiny<double> {
    static constexpr double value = 1.0e-14;
};

template <class Real>
MFEM_HD Real det3(const Real a[3][3]) {
    return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
           a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
           a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
}

// One Jacobi rotation zeroing A[p][q] of a symmetric 3x3 (Golub & Van Loan,
// "Matrix Computations", sec. 8.5.2: the symmetric Schur decomposition),
// accumulated into V.
template <int p, int q, class Real>
MFEM_HD void jacobi_rotate(Real A[3][3], Real V[3][3]) {
    constexpr int r = 3 - p - q;
    const Real apq = A[p][q];
    if (apq == Real(0)) return;
    const Real theta = (A[q][q] - A[p][p]) / (Real(2) * apq);
    Real t;
    if (abs_r(theta) > Real(1.0e18)) {
        t = Real(0.5) / theta;
    } else {
        t = sign_r(theta) / (abs_r(theta) + sqrt_r(theta * theta + Real(1)));
    }
    const Real c = Real(1) / sqrt_r(t * t + Real(1));
    const Real s = t * c;
    A[p][p] -= t * apq;
    A[q][q] += t * apq;
    A[p][q] = Real(0);
    A[q][p] = Real(0);
    const Real arp = A[r][p], arq = A[r][q];
    A[r][p] = A[p][r] = c * arp - s * arq;
    A[r][q] = A[q][r] = s * arp + c * arq;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const Real vkp = V[k][p], vkq = V[k][q];
        V[k][p] = c * vkp - s * vkq;
        V[k][q] = s * vkp + c * vkq;
    }
}

template <int i, int j, class Real>
MFEM_HD void sort_pair(Real d[3], Real V[3][3]) {
    if (d[i] < d[j]) {
        Real t = d[i];
        d[i] = d[j];
        d[j] = t;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            Real v = V[k][i];
            V[k][i] = V[k][j];
            V[k][j] = v;
        }
    }
}

// Rotation-variant SVD F = U diag(sig) V^T with U, V proper rotations,
// |sig| descending and the sign of det F carried by sig[2] -- the convention
// of the reference's rotational_svd (src/mfem/refinement/utils.py:46-67).
// Method (McAdams et al. 2011, "Computing the singular value decomposition of
// 3x3 matrices with minimal branching and elementary floating point
// operations"): Jacobi eigen-analysis of F^T F gives V; a QR factorisation of
// F V that keeps U a rotation gives U and the signed singular values.
// ROLLED keeps the five sweeps as a loop (same operations in the same
// order): the element kernel, whose fully unrolled body overflows the
// instruction cache, takes it; the line-search trial, which unrolled needs
// fewer registers, does not.
template <class Real, bool ROLLED = false>
MFEM_HD void polar_svd(const Real F[3][3], Real U[3][3], Real sig[3], Real V[3][3]) {
    Real A[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            A[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? Real(1) : Real(0);
    if (ROLLED) {
#pragma unroll 1
        for (int sweep = 0; sweep < 5; ++sweep) {
            jacobi_rotate<0, 1, Real>(A, V);
            jacobi_rotate<0, 2, Real>(A, V);
            jacobi_rotate<1, 2, Real>(A, V);
        }
    } else {
#pragma unroll
        for (int sweep = 0; sweep < 5; ++sweep) {
            jacobi_rotate<0, 1, Real>(A, V);
            jacobi_rotate<0, 2, Real>(A, V);
            jacobi_rotate<1, 2, Real>(A, V);
        }
    }
    Real d[3] = {A[0][0], A[1][1], A[2][2]};
    sort_pair<0, 1, Real>(d, V);
    sort_pair<0, 2, Real>(d, V);
    sort_pair<1, 2, Real>(d, V);
    // make V a rotation (flip the column of the smallest eigenvalue)
    Real vdet = det3(V);
    if (vdet < Real(0)) {
        V[0][2] = -V[0][2];
        V[1][2] = -V[1][2];
        V[2][2] = -V[2][2];
    }
    // B = F V
    Real B[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) B[i][j] = F[i][0] * V[0][j] + F[i][1] * V[1][j] + F[i][2] * V[2][j];
    // u0 = b0 / |b0|
    Real n0 = sqrt_r(B[0][0] * B[0][0] + B[1][0] * B[1][0] + B[2][0] * B[2][0]);
    Real u0[3];
    if (n0 > Real(1.0e-30)) {
        Real inv = Real(1) / n0;
        u0[0] = B[0][0] * inv;
        u0[1] = B[1][0] * inv;
        u0[2] = B[2][0] * inv;
    } else {
        u0[0] = Real(1);
        u0[1] = Real(0);
        u0[2] = Real(0);
    }
    // u1 = normalise(b1 - (u0.b1) u0), or any unit vector orthogonal to u0
    Real proj = u0[0] * B[0][1] + u0[1] * B[1][1] + u0[2] * B[2][1];
    Real w[3] = {B[0][1] - proj * u0[0], B[1][1] - proj * u0[1], B[2][1] - proj * u0[2]};
    Real n1 = sqrt_r(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    Real u1[3];
    if (n1 > Real(1.0e-30) && n1 > QrTiny<Real>::value * n0) {
        Real inv = Real(1) / n1;
        u1[0] = w[0] * inv;
        u1[1] = w[1] * inv;
        u1[2] = w[2] * inv;
    } else {
        // cross u0 with the axis it is least aligned with
        Real ax = abs_r(u0[0]), ay = abs_r(u0[1]), az = abs_r(u0[2]);
        Real e[3] = {Real(0), Real(0), Real(0)};
        if (ax <= ay && ax <= az) e[0] = Real(1);
        else if (ay <= az) e[1] = Real(1);
        else e[2] = Real(1);
        Real cx = u0[1] * e[2] - u0[2] * e[1];
        Real cy = u0[2] * e[0] - u0[0] * e[2];
        Real cz = u0[0] * e[1] - u0[1] * e[0];
        Real inv = Real(1) / sqrt_r(cx * cx + cy * cy + cz * cz);
        u1[0] = cx * inv;
        u1[1] = cy * inv;
        u1[2] = cz * inv;
    }
    Real u2[3] = {u0[1] * u1[2] - u0[2] * u1[1], u0[2] * u1[0] - u0[0] * u1[2], u0[0] * u1[1] - u0[1] * u1[0]};
    sig[0] = u0[0] * B[0][0] + u0[1] * B[1][0] + u0[2] * B[2][0];
    sig[1] = u1[0] * B[0][1] + u1[1] * B[1][1] + u1[2] * B[2][1];
    sig[2] = u2[0] * B[0][2] + u2[1] * B[1][2] + u2[2] * B[2][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        U[i][0] = u0[i];
        U[i][1] = u1[i];
        U[i][2] = u2[i];
    }
}

// sym6 of the polar stretch S = V diag(sig) V^T (src/mfem/refinement/utils.py:70-72).
template <class Real>
MFEM_HD void stretch_sym6(const Real sig[3], const Real V[3][3], Real sF[6]) {
    Real VS[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) VS[i][k] = V[i][k] * sig[k];
    auto Sij = [&](int i, int j) { return VS[i][0] * V[j][0] + VS[i][1] * V[j][1] + VS[i][2] * V[j][2]; };
    sF[0] = Sij(0, 0);
    sF[1] = Sij(1, 1);
    sF[2] = Sij(2, 2);
    sF[3] = Sij(0, 1);
    sF[4] = Sij(0, 2);
    sF[5] = Sij(1, 2);
}

// Three columns of dS/dF (the reference's 6x9 stretch_gradient,
// src/mfem/refinement/utils.py:75-121): columns a*3+b for b = 0..2, i.e.
// the derivatives by F[a][0..2].  Written in the SVD basis: with
// E^ = U^T E_ab V, the rotation derivative is U Omega V^T where
// Omega_ij = (E^_ij - E^_ji) / max(sig_i + sig_j, 1e-8) (the reference's
// dR/dF, same clamp), and dS = dR^T F + R^T dF = V (E^ - Omega diag(sig)) V^T.
// The reference stores sym6 of dS^T, i.e. the lower triangle of dS.
template <class Real>
MFEM_HD void stretch_gradient_row(int a, const Real U[3][3], const Real sig[3], const Real V[3][3],
                                  Real Jc[3][6]) {
    const Real s01 = max_r(sig[0] + sig[1], Real(1.0e-8));
    const Real s12 = max_r(sig[1] + sig[2], Real(1.0e-8));
    const Real s02 = max_r(sig[0] + sig[2], Real(1.0e-8));
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        Real N[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) N[i][j] = U[a][i] * V[b][j];
        const Real o01 = (N[0][1] - N[1][0]) / s01;
        const Real o12 = (N[1][2] - N[2][1]) / s12;
        const Real o02 = (N[0][2] - N[2][0]) / s02;
        N[0][1] -= o01 * sig[1];
        N[1][0] += o01 * sig[0];
        N[1][2] -= o12 * sig[2];
        N[2][1] += o12 * sig[1];
        N[0][2] -= o02 * sig[2];
        N[2][0] += o02 * sig[0];
        Real W[3][3];  // V N
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int j = 0; j < 3; ++j) W[p][j] = V[p][0] * N[0][j] + V[p][1] * N[1][j] + V[p][2] * N[2][j];
        auto dS = [&](int p, int q) { return W[p][0] * V[q][0] + W[p][1] * V[q][1] + W[p][2] * V[q][2]; };
        Jc[b][0] = dS(0, 0);
        Jc[b][1] = dS(1, 1);
        Jc[b][2] = dS(2, 2);
        Jc[b][3] = dS(1, 0);
        Jc[b][4] = dS(2, 0);
        Jc[b][5] = dS(2, 1);
    }
}

// det / gradient / Hessian of det on sym6 (src/mfem/utils.py:66-97).
MFEM_HD float det_sym6(const float s[6]) {
    return (s[0] * s[1] * s[2] + 2.0f * s[3] * s[4] * s[5]) -
           (s[1] * s[4] * s[4] + s[0] * s[5] * s[5] + s[2] * s[3] * s[3]);
}

MFEM_HD void grad_det_sym6(const float s[6], float g[6]) {
    g[0] = s[1] * s[2] - s[5] * s[5];
    g[1] = s[0] * s[2] - s[4] * s[4];
    g[2] = s[0] * s[1] - s[3] * s[3];
    g[3] = 2.0f * (s[4] * s[5] - s[2] * s[3]);
    g[4] = 2.0f * (s[3] * s[5] - s[1] * s[4]);
    g[5] = 2.0f * (s[3] * s[4] - s[0] * s[5]);
}

MFEM_HD void hess_det_sym6(const float s[6], float h[6][6]) {
    const float z = 0.0f;
    const float rows[6][6] = {
        {z, s[2], s[1], z, z, -2.0f * s[5]},
        {s[2], z, s[0], z, -2.0f * s[4], z},
        {s[1], s[0], z, -2.0f * s[3], z, z},
        {z, z, -2.0f * s[3], -2.0f * s[2], 2.0f * s[5], 2.0f * s[4]},
        {z, -2.0f * s[4], z, 2.0f * s[5], -2.0f * s[1], 2.0f * s[3]},
        {-2.0f * s[5], z, z, 2.0f * s[4], 2.0f * s[3], -2.0f * s[0]},
    };
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) h[i][j] = rows[i][j];
}

// Gill-Murray-Wright (1981) modified Cholesky of a symmetric 6x6 and the PSD
// fix built on it: returns A + E = L L^T and its inverse, both packed upper
// (src/mfem/numerical/gmw81.py:18-86, src/mfem/numerical/psd_fix.py:157-191;
// same constants eps = 1.19e-7, delta = sqrt(eps)).
MFEM_HD void psd_fix6(float A[6][6], float fixed[21], float inv[21]) {
    const float eps = 1.19e-7f;
    const float delta = sqrtf(eps);
    float gamma = 0.0f, xi = 0.0f;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        gamma = fmaxf(gamma, fabsf(A[i][i]));
#pragma unroll
        for (int j = i + 1; j < 6; ++j) xi = fmaxf(xi, fabsf(A[i][j]));
    }
    const float beta2 = fmaxf(gamma, fmaxf(xi / sqrtf(35.0f), eps));
#pragma unroll
    for (int j = 0; j < 6; ++j) {
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            float c_ij = A[j][i];
#pragma unroll
            for (int k = 0; k < j; ++k) c_ij -= A[k][k] * A[k][k] * A[i][k] * A[j][k];
            A[i][j] = c_ij;
        }
        float theta = 0.0f;
#pragma unroll
        for (int i = j + 1; i < 6; ++i) theta = fmaxf(theta, fabsf(A[i][j]));
        const float d_j = fmaxf(delta, fmaxf(fabsf(A[j][j]), theta * theta / beta2));
        A[j][j] = sqrtf(d_j);
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            const float c_ij = A[i][j];
            A[i][j] = c_ij / d_j;
            A[i][i] -= c_ij * c_ij / d_j;
        }
    }
    // L~[i][j] = l_ij sqrt(d_j)
    float L[6][6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const float sq = A[j][j];
#pragma unroll
        for (int i = 0; i < 6; ++i) L[i][j] = (i > j) ? A[i][j] * sq : ((i == j) ? sq : 0.0f);
    }
    // A + E = L L^T
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k <= j; ++k) acc += L[i][k] * L[j][k];
            fixed[p21(j, i)] = acc;
        }
    // Z = L^-1 in place (forward substitution, column by column)
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        L[k][k] = 1.0f / L[k][k];
#pragma unroll
        for (int i = k + 1; i < 6; ++i) {
            float acc = 0.0f;
#pragma unroll
            for (int j = k; j < i; ++j) acc += L[i][j] * L[j][k];
            L[i][k] = -acc / L[i][i];
        }
    }
    // (A + E)^-1 = Z^T Z
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j <= i; ++j) {
            float acc = 0.0f;
#pragma unroll
            for (int k = i; k < 6; ++k) acc += L[k][i] * L[k][j];
            inv[p21(j, i)] = acc;
        }
}

// Energy terms in s: gradient g_s, H_lambda = INV_SYM H_s INV_SYM and H_s^-1
// (src/mfem/refinement/elastic_energy.py:127-197 ARAP, 255-346 Neo-Hookean;
// src/mfem/refinement/kernels.py:207-217).
MFEM_HD void energy_terms(int energy, const float s[6], float mu, float lam, float vol, float g_s[6],
                          float H_l[21], float H_si[21]) {
    if (energy == 0) {
        const float muvol = mu * vol;
        const float inv_muvol = 1.0f / muvol;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float e = i < 3 ? 1.0f : 0.0f;
            g_s[i] = vol * (mu * (2.0f * sym_w(i) * s[i] - 2.0f * e) / 2.0f);
        }
#pragma unroll
        for (int k = 0; k < 21; ++k) {
            H_l[k] = 0.0f;
            H_si[k] = 0.0f;
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float hs = muvol * sym_w(i);
            H_l[p21(i, i)] = hs * inv_sym_w(i) * inv_sym_w(i);
            H_si[p21(i, i)] = inv_muvol * inv_sym_w(i);
        }
    } else {
        const float J = det_sym6(s);
        float gJ[6];
        grad_det_sym6(s, gJ);
        float hJ[6][6];
        hess_det_sym6(s, hJ);
        const float coef = lam * (J - 1.0f) - mu;
#pragma unroll
        for (int i = 0; i < 6; ++i) g_s[i] = vol * (mu * sym_w(i) * s[i] + coef * gJ[i]);
        float A[6][6];
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = 0; j < 6; ++j)
                A[i][j] = vol * (((i == j) ? mu * sym_w(i) : 0.0f) + lam * gJ[i] * gJ[j] + coef * hJ[i][j]);
        float Hs[21];
        psd_fix6(A, Hs, H_si);
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = i; j < 6; ++j) H_l[p21(i, j)] = Hs[p21(i, j)] * inv_sym_w(i) * inv_sym_w(j);
    }
}

// Elastic energy value in s (the *_energy_only kernels,
// src/mfem/refinement/elastic_energy.py:155-176 ARAP, 287-311 Neo-Hookean),
// written in E = s - I so that no O(1) terms cancel near rest:
//   ARAP  vol mu (I2 + 3 - 2 I1) / 2 with the reference's
//         I2 = s0 s1 + s1 s2 + s2 s0 + 2 (s3^2 + s4^2 + s5^2)
//         = vol mu (e0 e1 + e1 e2 + e2 e0 + 2 (s3^2 + s4^2 + s5^2)) / 2;
//   NH    vol (mu (|s|_F^2 - 3) / 2 - mu (J - 1) + lam (J - 1)^2 / 2)
//         = vol (mu (|E|_F^2 / 2 - m2(E) - det E) + lam (J - 1)^2 / 2),
//         J - 1 = tr E + m2(E) + det E, m2 = sum of the principal 2x2 minors.
MFEM_HD float elastic_energy(int energy, const float s[6], float mu, float lam, float vol) {
    const float e0 = s[0] - 1.0f, e1 = s[1] - 1.0f, e2 = s[2] - 1.0f;
    const float oo = s[3] * s[3] + s[4] * s[4] + s[5] * s[5];
    if (energy == 0) return vol * (mu * (e0 * e1 + e1 * e2 + e2 * e0 + 2.0f * oo) / 2.0f);
    const float m2 = e0 * e1 + e1 * e2 + e2 * e0 - oo;
    const float dE = e0 * e1 * e2 + 2.0f * s[3] * s[4] * s[5] - e0 * s[5] * s[5] - e1 * s[4] * s[4] -
                     e2 * s[3] * s[3];
    const float jm1 = (e0 + e1 + e2) + m2 + dE;
    const float fro = e0 * e0 + e1 * e1 + e2 * e2 + 2.0f * oo;
    return vol * (mu * (0.5f * fro - m2 - dE) + 0.5f * lam * jm1 * jm1);
}

// F = [x1-x0, x2-x0, x3-x0] DmInv (src/mfem/refinement/kernels.py:145-156),
// evaluated in Real from the float32 positions and DmInv.
template <class Real>
MFEM_HD void deformation_gradient(const float x[4][3], const float Dm[3][3], Real F[3][3]) {
    Real e[3][3];  // e[c] = x_{c+1} - x0
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int i = 0; i < 3; ++i) e[c][i] = Real(x[c + 1][i]) - Real(x[0][i]);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            F[i][j] = e[0][i] * Real(Dm[0][j]) + e[1][i] * Real(Dm[1][j]) + e[2][i] * Real(Dm[2][j]);
}

// Tets with det F below this take the polar decomposition and its
// derivative in float64 (near-degenerate, flattened or inverted tets, where
// dS/dF carries 1 / (sig_i + sig_j) and float32 loses the small singular
// values of F^T F).
constexpr float kPolarFp64Det = 1.0e-3f;

// Constraint c = SYM (sym6(S(F)) - s) and its Jacobian G = -SYM dS/dF dF/dx
// (the reference's compute_constraints, src/mfem/refinement/kernels.py:
// 131-169), the polar decomposition and dS/dF evaluated in Real, c and G
// rounded to float.
template <class Real, bool ROLLED = false>
MFEM_HD void element_geometry_t(const float x[4][3], const float Dm[3][3], const float s[6], float c[6],
                                float G[6][12]) {
    Real F[3][3];
    deformation_gradient<Real>(x, Dm, F);
    Real U[3][3], sig[3], V[3][3];
    polar_svd<Real, ROLLED>(F, U, sig, V);
    Real sF[6];
    stretch_sym6<Real>(sig, V, sF);
#pragma unroll
    for (int i = 0; i < 6; ++i) c[i] = (float)(Real(sym_w(i)) * (sF[i] - Real(s[i])));
    // dF/dx rows: B[0] = -(sum of DmInv rows), B[k] = DmInv[k-1] (utils.py:123-177)
    Real B[4][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        B[0][j] = -Real(Dm[0][j]) - Real(Dm[1][j]) - Real(Dm[2][j]);
        B[1][j] = Real(Dm[0][j]);
        B[2][j] = Real(Dm[1][j]);
        B[3][j] = Real(Dm[2][j]);
    }
    // G[:, 3k+a] = -(SYM sum_b J[:, a*3+b] B[k][b])  (kernels.py:161-169)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        Real Jc[3][6];
        stretch_gradient_row<Real>(a, U, sig, V, Jc);
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                const Real sr = Real(sym_w(r));
                G[r][3 * k + a] =
                    (float)(-((sr * Jc[0][r]) * B[k][0] + (sr * Jc[1][r]) * B[k][1] + (sr * Jc[2][r]) * B[k][2]));
            }
    }
}

// det F in float32: the test that sends a tet to the float64 polar path.
MFEM_HD float deformation_det(const float x[4][3], const float Dm[3][3]) {
    float F[3][3];
    deformation_gradient<float>(x, Dm, F);
    return det3(F);
}

MFEM_HD void element_geometry(const float x[4][3], const float Dm[3][3], const float s[6], float c[6],
                              float G[6][12]) {
    element_geometry_t<float>(x, Dm, s, c, G);
}

}  // namespace em
}  // namespace mfem
