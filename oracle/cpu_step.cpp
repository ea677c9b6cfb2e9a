// CPU restatement of the mixed-FEM global step with OpenMP on all host cores.
//
// Test and measurement infrastructure, not the product: it is the timed CPU
// baseline of bench.py (the reference's own Warp path cannot run here), and
// tests/test_cpu_step.py checks it against the float64 numpy oracle.  It
// restates RefinementSolver.step (src/mfem/refinement/solver.py:429-579)
// with refinement, contact and the line search off:
//   predictor x~ = x + v dt + g dt^2 / 2          (kernels.py:77-91)
//   K Newton iterations of
//     per-tet c, G, g_s, H_lambda, element blocks  (kernels.py:131-249,
//                                                    elastic_energy.py:127-407)
//     assembly H = sum G^T H_l G + (M + Q)/dt^2,
//              g = sum G^T (H_l c + INV_SYM g_s) - g_x   (solver.py:682-743)
//     block-Jacobi PCG from x~ - x to ||r|| <= tol ||g||  (solver.py:581-609)
//     local solve lambda, ds; x += dx, s += ds      (kernels.py:252-283)
//   velocity (x - x_in) / dt                        (kernels.py:351-363)
// The per-tet arithmetic is the library's own element math header
// (float32, host-compiled), so this baseline times the same operations the
// GPU performs; the numpy oracle stays the independent checker.  PCG
// vectors are float32 like the reference's CG; dot products are summed in
// float64 per thread and combined in thread order.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "element_math.cuh"

namespace {

using namespace mfem::em;

constexpr int kKe = 90;  // 10 upper 3x3 blocks of G^T H_l G per tet

inline int ke_block(int k, int l) { return k * 4 - (k * (k - 1)) / 2 + (l - k); }

struct CpuStep {
    int n = 0, T = 0, iterations = 8, energy = 0, maxiter = 1000;
    float tol = 1e-6f, k_attach = 10.0f, singular = 1e-20f;
    float gravity[3] = {0, 0, 0};
    std::vector<int32_t> tets, row_ptr, col_idx;
    std::vector<int32_t> cptr, ccode;      // contributions per slot: code = tet*16 + k*4 + l
    std::vector<int32_t> vptr, vcode;      // incident (tet, corner) per vertex: tet*4 + corner
    std::vector<float> Dm, mat, mass, hess_diag, pin_k, pin_target;
    std::vector<float> s, lam, c, G, g_s, H_l, Ke, fe, H, g, Minv, dx, r, z, p, Ap, x_tilde;
};

double dot(const std::vector<float> &a, const std::vector<float> &b) {
    const int m = (int)a.size();
    const int nt = omp_get_max_threads();
    std::vector<double> part(nt, 0.0);
#pragma omp parallel
    {
        double acc = 0.0;
#pragma omp for schedule(static)
        for (int i = 0; i < m; ++i) acc += (double)a[i] * (double)b[i];
        part[omp_get_thread_num()] = acc;
    }
    double t = 0.0;
    for (double v : part) t += v;
    return t;
}

void spmv(const CpuStep &S, const std::vector<float> &v, std::vector<float> &out) {
#pragma omp parallel for schedule(static)
    for (int row = 0; row < S.n; ++row) {
        float acc[3] = {0, 0, 0};
        for (int k = S.row_ptr[row]; k < S.row_ptr[row + 1]; ++k) {
            const float *h = &S.H[(size_t)9 * k];
            const float *x = &v[(size_t)3 * S.col_idx[k]];
            for (int a = 0; a < 3; ++a) acc[a] += h[3 * a] * x[0] + h[3 * a + 1] * x[1] + h[3 * a + 2] * x[2];
        }
        for (int a = 0; a < 3; ++a) out[(size_t)3 * row + a] = acc[a];
    }
}

void precond(const CpuStep &S, const std::vector<float> &rr, std::vector<float> &zz) {
#pragma omp parallel for schedule(static)
    for (int v = 0; v < S.n; ++v) {
        const float *M = &S.Minv[(size_t)9 * v];
        const float *x = &rr[(size_t)3 * v];
        for (int a = 0; a < 3; ++a) zz[(size_t)3 * v + a] = M[3 * a] * x[0] + M[3 * a + 1] * x[1] + M[3 * a + 2] * x[2];
    }
}

void element_stage(CpuStep &S, const float *xpos) {
    const int T = S.T;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; ++t) {
        float xv[4][3], Dm[3][3], s[6];
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) xv[k][a] = xpos[3 * S.tets[4 * t + k] + a];
        for (int i = 0; i < 9; ++i) Dm[i / 3][i % 3] = S.Dm[(size_t)9 * t + i];
        for (int i = 0; i < 6; ++i) s[i] = S.s[(size_t)6 * t + i];
        const float mu = S.mat[(size_t)3 * t], lm = S.mat[(size_t)3 * t + 1];
        const float vol = 1.0f / (6.0f * det3(Dm));
        float gs[6], Hl[21], Hsi[21], c[6], G[6][12];
        energy_terms(S.energy, s, mu, lm, vol, gs, Hl, Hsi);
        element_geometry(xv, Dm, s, c, G);
        for (int i = 0; i < 6; ++i) {
            S.c[(size_t)6 * t + i] = c[i];
            S.g_s[(size_t)6 * t + i] = gs[i];
        }
        for (int k = 0; k < 21; ++k) S.H_l[(size_t)21 * t + k] = Hl[k];
        std::memcpy(&S.G[(size_t)72 * t], G, sizeof(G));
        float w[6];
        for (int i = 0; i < 6; ++i) {
            float acc = inv_sym_w(i) * gs[i];
            for (int j = 0; j < 6; ++j) acc += Hl[p21(i, j)] * c[j];
            w[i] = acc;
        }
        float *ke = &S.Ke[(size_t)kKe * t];
        float *fe = &S.fe[(size_t)12 * t];
        for (int l = 0; l < 4; ++l) {
            float P[6][3];
            for (int i = 0; i < 6; ++i)
                for (int b = 0; b < 3; ++b) {
                    float acc = 0.0f;
                    for (int j = 0; j < 6; ++j) acc += Hl[p21(i, j)] * G[j][3 * l + b];
                    P[i][b] = acc;
                }
            for (int b = 0; b < 3; ++b) {
                float acc = 0.0f;
                for (int i = 0; i < 6; ++i) acc += G[i][3 * l + b] * w[i];
                fe[3 * l + b] = acc;
            }
            for (int k = 0; k <= l; ++k) {
                float *blk = ke + 9 * ke_block(k, l);
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        float acc = 0.0f;
                        for (int i = 0; i < 6; ++i) acc += G[i][3 * k + a] * P[i][b];
                        blk[3 * a + b] = acc;
                    }
            }
        }
    }
}

void assemble(CpuStep &S, const float *x, float dt) {
    const float alpha = (float)(1.0 / ((double)dt * (double)dt));
    const float dt2 = dt * dt;
#pragma omp parallel for schedule(static)
    for (int row = 0; row < S.n; ++row) {
        for (int slot = S.row_ptr[row]; slot < S.row_ptr[row + 1]; ++slot) {
            float v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int q = S.cptr[slot]; q < S.cptr[slot + 1]; ++q) {
                const int code = S.ccode[q];
                const int e = code >> 4, k = (code >> 2) & 3, l = code & 3;
                const float *blk = &S.Ke[(size_t)kKe * e + 9 * ke_block(std::min(k, l), std::max(k, l))];
                if (k <= l)
                    for (int i = 0; i < 9; ++i) v[i] += blk[i];
                else
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) v[3 * a + b] += blk[3 * b + a];
            }
            if (S.col_idx[slot] == row) {
                const float hd = alpha * S.hess_diag[row];
                v[0] += hd;
                v[4] += hd;
                v[8] += hd;
                const float c00 = v[4] * v[8] - v[5] * v[7], c01 = v[5] * v[6] - v[3] * v[8],
                            c02 = v[3] * v[7] - v[4] * v[6];
                const float det = v[0] * c00 + v[1] * c01 + v[2] * c02;
                float *M = &S.Minv[(size_t)9 * row];
                if (!(std::fabs(det) >= S.singular)) {
                    for (int i = 0; i < 9; ++i) M[i] = (i % 4 == 0) ? 1.0f : 0.0f;
                } else {
                    const float id = 1.0f / det;
                    M[0] = c00 * id;
                    M[1] = (v[2] * v[7] - v[1] * v[8]) * id;
                    M[2] = (v[1] * v[5] - v[2] * v[4]) * id;
                    M[3] = c01 * id;
                    M[4] = (v[0] * v[8] - v[2] * v[6]) * id;
                    M[5] = (v[2] * v[3] - v[0] * v[5]) * id;
                    M[6] = c02 * id;
                    M[7] = (v[1] * v[6] - v[0] * v[7]) * id;
                    M[8] = (v[0] * v[4] - v[1] * v[3]) * id;
                }
            }
            std::memcpy(&S.H[(size_t)9 * slot], v, sizeof(v));
        }
        // g = sum of the incident element rhs - g_x; warm start x~ - x
        float gg[3] = {0, 0, 0};
        for (int q = S.vptr[row]; q < S.vptr[row + 1]; ++q) {
            const int e = S.vcode[q] >> 2, k = S.vcode[q] & 3;
            for (int a = 0; a < 3; ++a) gg[a] += S.fe[(size_t)12 * e + 3 * k + a];
        }
        const float m = S.mass[row], kp = S.pin_k[row];
        for (int a = 0; a < 3; ++a) {
            const float xa = x[3 * row + a];
            const float gx = m * (xa - S.x_tilde[3 * row + a]) / dt2 + (kp * xa + (-(kp * S.pin_target[3 * row + a]))) / dt2;
            S.g[(size_t)3 * row + a] = gg[a] - gx;
            S.dx[(size_t)3 * row + a] = S.x_tilde[3 * row + a] - xa;
        }
    }
}

int pcg(CpuStep &S) {
    spmv(S, S.dx, S.Ap);
    const int m = 3 * S.n;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) S.r[i] = S.g[i] - S.Ap[i];
    const double bb = dot(S.g, S.g);
    const double thr = (double)S.tol * (double)S.tol * bb;
    double rr = dot(S.r, S.r);
    if (rr <= thr) return 0;
    precond(S, S.r, S.z);
    S.p = S.z;
    double rz = dot(S.r, S.z);
    int it = 0;
    while (it < S.maxiter) {
        spmv(S, S.p, S.Ap);
        const float alpha = (float)(rz / dot(S.p, S.Ap));
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; ++i) {
            S.dx[i] += alpha * S.p[i];
            S.r[i] -= alpha * S.Ap[i];
        }
        ++it;
        rr = dot(S.r, S.r);
        if (rr <= thr) break;
        precond(S, S.r, S.z);
        const double rz_new = dot(S.r, S.z);
        const float beta = (float)(rz_new / rz);
        rz = rz_new;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; ++i) S.p[i] = S.z[i] + beta * S.p[i];
    }
    return it;
}

void local_solve(CpuStep &S, float *x) {
#pragma omp parallel for schedule(static)
    for (int t = 0; t < S.T; ++t) {
        float u[6];
        for (int i = 0; i < 6; ++i) u[i] = S.c[(size_t)6 * t + i];
        const float *G = &S.G[(size_t)72 * t];
        for (int k = 0; k < 4; ++k) {
            const float *d = &S.dx[(size_t)3 * S.tets[4 * t + k]];
            for (int i = 0; i < 6; ++i) u[i] -= G[12 * i + 3 * k] * d[0] + G[12 * i + 3 * k + 1] * d[1] + G[12 * i + 3 * k + 2] * d[2];
        }
        const float *Hl = &S.H_l[(size_t)21 * t];
        for (int i = 0; i < 6; ++i) {
            float acc = inv_sym_w(i) * S.g_s[(size_t)6 * t + i];
            for (int j = 0; j < 6; ++j) acc += Hl[p21(i, j)] * u[j];
            S.lam[(size_t)6 * t + i] = -acc;
            S.s[(size_t)6 * t + i] += inv_sym_w(i) * u[i];
        }
    }
    const int m = 3 * S.n;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) x[i] += S.dx[i];
}

}  // namespace

extern "C" {

// Builds the baseline for one mesh (host arrays as for mfem_plan_create);
// s starts at S(F_rest), lambda at 0.  Returns NULL on a bad mesh.
void *cpu_step_create(int n, int T, const int32_t *tets, const float *poses, const float *materials,
                      const float *rest, const float *mass, const float *inv_mass, const float *gravity,
                      int iterations, int energy, float tol, int maxiter, float attachment_stiffness) {
    if (n <= 0 || T < 0) return nullptr;
    for (int64_t i = 0; i < (int64_t)4 * T; ++i)
        if (tets[i] < 0 || tets[i] >= n) return nullptr;
    auto *S = new CpuStep();
    S->n = n;
    S->T = T;
    S->iterations = iterations;
    S->energy = energy;
    S->tol = tol;
    S->maxiter = maxiter;
    S->k_attach = attachment_stiffness;
    for (int a = 0; a < 3; ++a) S->gravity[a] = gravity[a];
    S->tets.assign(tets, tets + (size_t)4 * T);
    S->Dm.assign(poses, poses + (size_t)9 * T);
    S->mat.assign(materials, materials + (size_t)3 * T);
    S->mass.assign(mass, mass + n);
    S->hess_diag.resize(n);
    S->pin_k.resize(n);
    S->pin_target.assign(rest, rest + (size_t)3 * n);
    for (int v = 0; v < n; ++v) {
        const bool pinned = inv_mass[v] == 0.0f;
        S->pin_k[v] = pinned ? attachment_stiffness : 0.0f;
        // Hessian mass: identity on attached vertices (kernels.py:21-27)
        S->hess_diag[v] = (pinned ? 1.0f : 1.0f / inv_mass[v]) + S->pin_k[v];
    }
    // sparsity: vertex adjacency, ascending columns
    std::vector<std::vector<int32_t>> adj(n);
    for (int v = 0; v < n; ++v) adj[v].push_back(v);
    for (int e = 0; e < T; ++e)
        for (int k = 0; k < 4; ++k)
            for (int l = 0; l < 4; ++l) adj[tets[4 * e + k]].push_back(tets[4 * e + l]);
    S->row_ptr.assign(n + 1, 0);
    for (int v = 0; v < n; ++v) {
        std::sort(adj[v].begin(), adj[v].end());
        adj[v].erase(std::unique(adj[v].begin(), adj[v].end()), adj[v].end());
        S->row_ptr[v + 1] = S->row_ptr[v] + (int)adj[v].size();
        S->col_idx.insert(S->col_idx.end(), adj[v].begin(), adj[v].end());
    }
    const int nnzb = S->row_ptr[n];
    // contributions per slot, in tet order
    std::vector<int32_t> cnt(nnzb + 1, 0);
    std::vector<int32_t> slot((size_t)16 * T);
    for (int e = 0; e < T; ++e)
        for (int k = 0; k < 4; ++k) {
            const int row = tets[4 * e + k];
            const int32_t *b = &S->col_idx[S->row_ptr[row]], *en = &S->col_idx[S->row_ptr[row + 1]];
            for (int l = 0; l < 4; ++l) {
                const int sl = (int)(std::lower_bound(b, en, tets[4 * e + l]) - S->col_idx.data());
                slot[(size_t)16 * e + 4 * k + l] = sl;
                ++cnt[sl + 1];
            }
        }
    S->cptr.assign(nnzb + 1, 0);
    for (int i = 0; i < nnzb; ++i) S->cptr[i + 1] = S->cptr[i] + cnt[i + 1];
    S->ccode.resize((size_t)16 * T);
    std::vector<int32_t> fill(S->cptr.begin(), S->cptr.end() - 1);
    for (int e = 0; e < T; ++e)
        for (int q = 0; q < 16; ++q) S->ccode[fill[slot[(size_t)16 * e + q]]++] = 16 * e + q;
    // incident (tet, corner) per vertex
    S->vptr.assign(n + 1, 0);
    for (int64_t i = 0; i < (int64_t)4 * T; ++i) ++S->vptr[tets[i] + 1];
    for (int v = 0; v < n; ++v) S->vptr[v + 1] += S->vptr[v];
    S->vcode.resize((size_t)4 * T);
    std::vector<int32_t> vf(S->vptr.begin(), S->vptr.end() - 1);
    for (int e = 0; e < T; ++e)
        for (int k = 0; k < 4; ++k) S->vcode[vf[tets[4 * e + k]]++] = 4 * e + k;
    // work arrays
    S->s.resize((size_t)6 * T);
    S->lam.assign((size_t)6 * T, 0.0f);
    S->c.resize((size_t)6 * T);
    S->G.resize((size_t)72 * T);
    S->g_s.resize((size_t)6 * T);
    S->H_l.resize((size_t)21 * T);
    S->Ke.resize((size_t)kKe * T);
    S->fe.resize((size_t)12 * T);
    S->H.resize((size_t)9 * nnzb);
    S->Minv.resize((size_t)9 * n);
    for (auto *v : {&S->g, &S->dx, &S->r, &S->z, &S->p, &S->Ap, &S->x_tilde}) v->resize((size_t)3 * n);
    // s = S(F) at rest (additional_state.py:146-189)
#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; ++t) {
        float xv[4][3], Dm[3][3], F[3][3], U[3][3], sig[3], V[3][3], sF[6];
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) xv[k][a] = rest[3 * tets[4 * t + k] + a];
        for (int i = 0; i < 9; ++i) Dm[i / 3][i % 3] = poses[(size_t)9 * t + i];
        deformation_gradient(xv, Dm, F);
        polar_svd(F, U, sig, V);
        stretch_sym6(sig, V, sF);
        for (int i = 0; i < 6; ++i) S->s[(size_t)6 * t + i] = sF[i];
    }
    return S;
}

void cpu_step_destroy(void *h) { delete static_cast<CpuStep *>(h); }

int cpu_step_threads(void) { return omp_get_max_threads(); }

// Threads of the following steps (<= 0: leave OpenMP's default, all cores).
void cpu_step_set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}

// One step: q_out, qd_out from q_in, qd_in (host arrays [n][3]).  PCG
// iterations of the step's solves go to iters[iterations] if non-NULL.
int cpu_step_run(void *h, const float *q_in, const float *qd_in, float *q_out, float *qd_out, float dt,
                 int32_t *iters) {
    auto &S = *static_cast<CpuStep *>(h);
    const int m = 3 * S.n;
    for (int i = 0; i < m; ++i) {
        S.x_tilde[i] = q_in[i] + qd_in[i] * dt + S.gravity[i % 3] * dt * dt / 2.0f;
        q_out[i] = q_in[i];
    }
    for (int it = 0; it < S.iterations; ++it) {
        element_stage(S, q_out);
        assemble(S, q_out, dt);
        const int k = pcg(S);
        if (iters) iters[it] = k;
        local_solve(S, q_out);
    }
    for (int i = 0; i < m; ++i) qd_out[i] = (q_out[i] - q_in[i]) / dt;
    return 0;
}

}  // extern "C"
