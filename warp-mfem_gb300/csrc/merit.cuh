// Terms of the line-search merit function (lambda held fixed), shared by the
// local-solve kernel (which sums them at the current x, s) and the line-search
// kernel (which sums them at each trial x + alpha dx, s + alpha ds).
// Reference: the objective of src/mfem/refinement/solver.py:803-869.
#pragma once

#include "contact_terms.cuh"
#include "element_math.cuh"
#include "internal.h"

namespace mfem {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

// Psi_t(s + alpha ds) - lambda_t . c_t(x + alpha dx, s + alpha ds) of tet t
// (*_energy_only kernels, elastic_energy.py:155-176, 287-311;
// add_constraint_objective, kernels.py:301-334).  ds is component-major [6][T].
__device__ __forceinline__ double tet_merit(const TetViews &tv, const float *x, const float *dx,
                                            const float *ds, int energy, int t, float alpha) {
    const int T = tv.n_tets;
    const int4 tt = tv.tets[t];
    const int vid[4] = {tt.x, tt.y, tt.z, tt.w};
    float xv[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) xv[k][c] = fmaf(alpha, dx[3 * vid[k] + c], x[3 * vid[k] + c]);
    float Dm[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Dm[i][j] = tv.dminv[(size_t)t * 9 + i * 3 + j];
    // The merit needs S(F) only, which the float32 polar decomposition gives
    // to about eps |F| even for near-degenerate tets (the QR step recovers
    // the small singular value from F v); the float64 path of the element
    // stage is for dS/dF, whose 1 / (sig_i + sig_j) float32 cannot carry.
    float F[3][3], U[3][3], sig[3], V[3][3], sF[6];
    em::deformation_gradient(xv, Dm, F);
    em::polar_svd(F, U, sig, V);
    em::stretch_sym6(sig, V, sF);
    float st[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) st[i] = fmaf(alpha, ds[(size_t)i * T + t], tv.stretch[(size_t)t * 6 + i]);
    const float mu = tv.materials[(size_t)t * 3 + 0];
    const float lm = tv.materials[(size_t)t * 3 + 1];
    const float vol = 1.0f / (6.0f * em::det3(Dm));
    float lc = 0.0f;
#pragma unroll
    for (int i = 0; i < 6; ++i) lc += tv.lambda[(size_t)t * 6 + i] * (em::sym_w(i) * (sF[i] - st[i]));
    return (double)em::elastic_energy(energy, st, mu, lm, vol) - (double)lc;
}

// [m |x - x~|^2 / 2 + k |x - p|^2 / 2] / dt^2 of vertex v at x + alpha dx
// (kinetic_objective_kernel, kernels.py:286-298; the attachment energy
// x.(Q x / 2 + b) + c of boundary_condition.py:62-71 as k |x - p|^2 / 2).
__device__ __forceinline__ double vertex_merit(const VertexViews &vv, const float *x, int v, float alpha,
                                               double inv_dt2) {
    float kin = 0.0f, att = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float xc = fmaf(alpha, vv.dx[3 * v + c], x[3 * v + c]);
        const float d = xc - vv.x_tilde[3 * v + c];
        const float e = xc - vv.pin_target[3 * v + c];
        kin += d * d;
        att += e * e;
    }
    return (double)(0.5f * vv.mass[v] * kin + 0.5f * vv.pin_k[v] * att) * inv_dt2;
}

}  // namespace mfem
