// Adaptive refinement: one edge-bisection pass over a plan's mesh.
//
// The reference's refine() (src/mfem/refinement/refinement.py:914-1322)
// scores every edge, lets each tet pick one edge above a threshold, resolves
// the picks over a few sweeps so that no tet holds two, and splits every tet
// around a picked edge in two at a new vertex on the edge.  It keys edges in
// a hash table and settles conflicts with unordered flag writes, so the
// outcome can change with thread scheduling.  Here:
//
//  * the edges are the upper off-diagonal slots of H's sparsity (exact
//    vertex adjacency, built on the host with the plan), with per-edge and
//    per-vertex tet lists in ascending tet order: no hashing, and every sum
//    is taken in a fixed order;
//  * selection is deterministic: edges rank by score, ties by the smaller
//    (min, max) vertex key; each sweep every tet picks its best available
//    candidate (keeping an edge it already holds), a candidate that every
//    tet containing it picked is selected, and the other edges of those tets
//    leave the race.  Every write of a sweep writes the same value whoever
//    writes it, so the kernels' order does not matter, no tet ever holds two
//    selected edges and every tet around a selected edge splits;
//  * new vertices are numbered in ascending edge order, new tets and tris
//    keep the reference's layout (exclusive scans of 1 + split, the two
//    children of a split element side by side);
//  * on a pass that splits, each vertex's lumped mass is the sum of
//    density * volume / 4 over its tets in (old tet, child) order, and
//    non-kinematic vertices get inv_mass = 1 / mass;
//  * a pass over capacity is dropped whole (refinement.py:578-604), and a
//    pass that splits nothing leaves the mesh as it is.  The output arrays
//    always receive the resulting mesh.
//
// Floating-point work uses round-to-nearest intrinsics so that no multiply-
// add is contracted: scores, new vertices, DmInv and masses follow a fixed
// operation order.
#include <algorithm>

#include "contact_terms.cuh"
#include "element_math.cuh"

namespace mfem {
namespace {

constexpr int kRefineThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kRefineThreads * kScanItems;
constexpr unsigned char kAvailable = 1, kSelected = 2, kUnavailable = 3;
constexpr int kCtrlRefining = 0, kCtrlApply = 1;

inline int blocks_for(int64_t n, int threads) { return (int)std::max<int64_t>(1, (n + threads - 1) / threads); }

__device__ __forceinline__ float len3(const float *a, const float *b) {
    const float dx = __fsub_rn(b[0], a[0]), dy = __fsub_rn(b[1], a[1]), dz = __fsub_rn(b[2], a[2]);
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}

// cofactor expansion along the first row
__device__ __forceinline__ float det3_rn(const float M[9]) {
    const float c0 = __fsub_rn(__fmul_rn(M[4], M[8]), __fmul_rn(M[5], M[7]));
    const float c1 = __fsub_rn(__fmul_rn(M[5], M[6]), __fmul_rn(M[3], M[8]));
    const float c2 = __fsub_rn(__fmul_rn(M[3], M[7]), __fmul_rn(M[4], M[6]));
    return __fadd_rn(__fadd_rn(__fmul_rn(M[0], c0), __fmul_rn(M[1], c1)), __fmul_rn(M[2], c2));
}

// adjugate over determinant; returns the determinant
__device__ __forceinline__ float inverse3_rn(const float M[9], float out[9]) {
    const float a = M[0], b = M[1], c = M[2], d = M[3], e = M[4], f = M[5], g = M[6], h = M[7], i = M[8];
    const float A = __fsub_rn(__fmul_rn(e, i), __fmul_rn(f, h));
    const float B = __fsub_rn(__fmul_rn(f, g), __fmul_rn(d, i));
    const float C = __fsub_rn(__fmul_rn(d, h), __fmul_rn(e, g));
    const float det = __fadd_rn(__fadd_rn(__fmul_rn(a, A), __fmul_rn(b, B)), __fmul_rn(c, C));
    const float r = __fdiv_rn(1.0f, det);
    out[0] = __fmul_rn(A, r);
    out[1] = __fmul_rn(__fsub_rn(__fmul_rn(c, h), __fmul_rn(b, i)), r);
    out[2] = __fmul_rn(__fsub_rn(__fmul_rn(b, f), __fmul_rn(c, e)), r);
    out[3] = __fmul_rn(B, r);
    out[4] = __fmul_rn(__fsub_rn(__fmul_rn(a, i), __fmul_rn(c, g)), r);
    out[5] = __fmul_rn(__fsub_rn(__fmul_rn(c, d), __fmul_rn(a, f)), r);
    out[6] = __fmul_rn(C, r);
    out[7] = __fmul_rn(__fsub_rn(__fmul_rn(b, g), __fmul_rn(a, h)), r);
    out[8] = __fmul_rn(__fsub_rn(__fmul_rn(a, e), __fmul_rn(b, d)), r);
    return det;
}

__device__ __forceinline__ float lerp_rn(float a, float b, float t) { return __fadd_rn(a, __fmul_rn(__fsub_rn(b, a), t)); }

__device__ __forceinline__ bool kinematic_edge(const RefineViews &rv, int a, int b) {
    return rv.inv_mass[a] == 0.0f && rv.inv_mass[b] == 0.0f;
}

// local vertex pairs (i, j), j < i, in the reference's loop order
__constant__ int kTetPairI[6] = {1, 2, 2, 3, 3, 3};
__constant__ int kTetPairJ[6] = {0, 0, 1, 0, 1, 2};
__constant__ int kTriPairI[3] = {1, 2, 2};
__constant__ int kTriPairJ[3] = {0, 0, 1};

__global__ void refine_begin_kernel(int *ctrl, int *pass_counter, int refine_every) {
    int refining = 1;
    if (pass_counter) {
        const int c = *pass_counter;
        refining = (refine_every <= 1 || c % refine_every == 0) ? 1 : 0;
        *pass_counter = c + 1;
    }
    ctrl[kCtrlRefining] = refining;
    ctrl[kCtrlApply] = 0;
}

// Per surface tri: distance to the nearest capsule, closest-point weights
// and barrier energy at q (compute_tri_distance, contact.py:626-656).
__global__ void refine_tri_inputs_kernel(RefineViews rv, ContactViews cv, const float *__restrict__ q) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rv.m) return;
    float p[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) p[k][c] = q[3 * rv.tris[3 * t + k] + c];
    float w[3], nrm[3];
    int sid;
    const float d = tri_contact_geometry(cv, p[0], p[1], p[2], w, nrm, sid);
    float e = 0.0f;
    if (d < cv.d1) {
        float de, d2e;
        ct::barrier(d, cv.d0, cv.d1, cv.q, e, de, d2e);
        e *= cv.k;
    }
    rv.tdist[t] = d;
#pragma unroll
    for (int k = 0; k < 3; ++k) rv.tbary[3 * t + k] = w[k];
    rv.tenergy[t] = e;
}

// Per vertex: nearest shape and its signed distance at q (compute_distance,
// contact.py:98-164) and the legacy vertex score, the barrier energy k b(d)
// plus the tris' energies weighted by the vertex's closest-point weight
// (evaluate_barrier_energy, evaluate_tri_barrier_energy: contact.py:191-233,
// 685-741), tris taken in ascending order.
__global__ void refine_vertex_inputs_kernel(RefineViews rv, ContactViews cv, const float *__restrict__ q) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= rv.n) return;
    float d = 1.0e8f;
    int sid = -1;
    float e = 0.0f;
    if (cv.on && cv.n_shapes > 0) {
        const float x[3] = {q[3 * v], q[3 * v + 1], q[3 * v + 2]};
        float nrm[3];
        d = vertex_distance(cv, x, nrm, sid);
        if (d < cv.d1) {
            float de, d2e;
            ct::barrier(d, cv.d0, cv.d1, cv.q, e, de, d2e);
            e *= cv.k;
        }
        if (rv.m > 0) {
            for (int i = cv.vt_ptr[v]; i < cv.vt_ptr[v + 1]; ++i) {
                const int code = cv.vt_code[i];
                const int t = code / 3, corner = code - 3 * t;
                e = __fadd_rn(e, __fmul_rn(rv.tbary[3 * t + corner], rv.tenergy[t]));
            }
        }
    }
    rv.vdist[v] = d;
    rv.vsid[v] = sid;
    rv.vscore[v] = e;
}

// Per tet: elastic energy in s (unless given), strain-energy density over mu
// and longest edge for the geometric score (refinement.py:163-176, 219-223);
// per-block float64 sums of the density in a fixed order.
__global__ void refine_tet_kernel(RefineViews rv, const float *__restrict__ q, int geometric) {
    __shared__ double s_sum[kRefineThreads];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double dens_d = 0.0;
    if (t < rv.T) {
        float Dm[3][3], M[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            M[i] = rv.dminv[(size_t)t * 9 + i];
            Dm[i / 3][i % 3] = M[i];
        }
        float E;
        if (rv.tet_scores) {
            E = rv.tet_scores[t];
        } else {
            float s[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) s[i] = rv.stretch[(size_t)t * 6 + i];
            const float vol = 1.0f / (6.0f * em::det3(Dm));
            E = em::elastic_energy(rv.energy, s, rv.materials[(size_t)t * 3 + 0], rv.materials[(size_t)t * 3 + 1],
                                   vol);
        }
        rv.e_tet[t] = E;
        if (geometric) {
            const float vol = fabsf(__fdiv_rn(1.0f, __fmul_rn(6.0f, det3_rn(M))));
            const float mu = rv.materials[(size_t)t * 3 + 0];
            float dens = 0.0f;
            if (mu > 0.0f && vol > 0.0f) dens = __fdiv_rn(fmaxf(E, 0.0f), __fmul_rn(vol, mu));
            rv.dens[t] = dens;
            dens_d = (double)dens;
            const int4 tt = rv.tets[t];
            const int vid[4] = {tt.x, tt.y, tt.z, tt.w};
            float lmax = 0.0f;
#pragma unroll
            for (int p = 0; p < 6; ++p)
                lmax = fmaxf(lmax, len3(q + 3 * vid[kTetPairI[p]], q + 3 * vid[kTetPairJ[p]]));
            rv.lmax[t] = fmaxf(lmax, 1.0e-20f);
        }
    }
    if (!geometric) return;
    s_sum[threadIdx.x] = dens_d;
    __syncthreads();
    for (int w = kRefineThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s_sum[threadIdx.x] += s_sum[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) rv.partials[blockIdx.x] = s_sum[0];
}

// Mean density over the tets (elastic_density_stats, refinement.py:179-192):
// the block sums added in block order; 0 when there is nothing to be
// relative to.
__global__ void refine_stats_kernel(RefineViews rv, int blocks) {
    if (threadIdx.x != 0) return;
    double total = 0.0;
    for (int b = 0; b < blocks; ++b) total += rv.partials[b];
    const double count = (double)rv.T;
    *rv.mean_density = (count > 0.0 && total > 0.0) ? (float)(total / count) : 0.0f;
}

__device__ __forceinline__ float capsule_proximity(const RefineViews &rv, const ContactViews &cv, int v, float d1) {
    const int sid = rv.particle_shape_id ? rv.particle_shape_id[v] : rv.vsid[v];
    if (sid < 0) return 0.0f;
    if (cv.type == nullptr || sid >= cv.n_shapes || cv.type[sid] != ct::kShapeCapsule) return 0.0f;
    const float d = rv.particle_distance ? rv.particle_distance[v] : rv.vdist[v];
    return fmaxf(__fdiv_rn(__fsub_rn(d1, d), d1), 0.0f);
}

// Per edge: the legacy score, the sum over its tets in ascending order of
// (E_t w_t + min(vs_a, vs_b) w_v) L, or the penetration score when the
// midpoint lies inside a shape (populate_candidates, refinement.py:74-121);
// or the geometric score, the max over its tets of (L/h)(L/L_max)(w_e s_el +
// w_c s_c) for L >= 2h (populate_candidates_geometric, :195-256).
__global__ void refine_score_kernel(RefineViews rv, ContactViews cv, RefineParams rp, const float *__restrict__ q) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= rv.nnzb) return;
    const int a = rv.slot_row[s], b = rv.col_idx[s];
    float score = 0.0f;
    if (a < b && !kinematic_edge(rv, a, b)) {
        const float L = len3(q + 3 * a, q + 3 * b);
        if (rp.scoring == 0) {
            const float *vs = rv.vertex_scores ? rv.vertex_scores : rv.vscore;
            const float vterm = __fmul_rn(fminf(vs[a], vs[b]), rp.vert_w);
            for (int i = rv.edge_start[s]; i < rv.edge_start[s + 1]; ++i) {
                const int t = rv.edge_tet[i];
                score = __fadd_rn(score, __fmul_rn(__fadd_rn(__fmul_rn(rv.e_tet[t], rp.tet_w), vterm), L));
            }
            if (cv.on && cv.n_shapes > 0) {
                const float mid[3] = {__fmul_rn(0.5f, __fadd_rn(q[3 * a], q[3 * b])),
                                      __fmul_rn(0.5f, __fadd_rn(q[3 * a + 1], q[3 * b + 1])),
                                      __fmul_rn(0.5f, __fadd_rn(q[3 * a + 2], q[3 * b + 2]))};
                float nrm[3];
                int sid;
                if (vertex_distance(cv, mid, nrm, sid) < 0.0f) score = fmaxf(0.0f, rp.pen_score);
            }
        } else {
            const float h = rp.min_edge;
            if (L >= __fmul_rn(2.0f, h)) {
                const float sc = fmaxf(capsule_proximity(rv, cv, a, rp.d1), capsule_proximity(rv, cv, b, rp.d1));
                const float cterm = __fmul_rn(rp.vc_w, sc);
                const float mean = *rv.mean_density;
                const float lh = __fdiv_rn(L, h);
                for (int i = rv.edge_start[s]; i < rv.edge_start[s + 1]; ++i) {
                    const int t = rv.edge_tet[i];
                    float sel = rv.dens[t];
                    if (mean > 0.0f) sel = fmaxf(__fsub_rn(__fdiv_rn(sel, mean), 1.0f), 0.0f);
                    const float v = __fmul_rn(__fmul_rn(lh, __fdiv_rn(L, rv.lmax[t])),
                                              __fadd_rn(__fmul_rn(rp.el_w, sel), cterm));
                    score = fmaxf(score, fmaxf(v, 0.0f));
                }
            }
        }
    }
    rv.score[s] = score;
}

// Per surface tri inside the barrier range: raises the scores of its edges,
// the edge nearest the closest point most (populate_tri_candidates_geometric,
// refinement.py:259-316).  Scores are non-negative, so a max over their bit
// patterns is the max over the values, in any order.
__global__ void refine_tri_score_kernel(RefineViews rv, RefineParams rp, const float *__restrict__ q) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rv.m) return;
    const float d = rv.tri_distance ? rv.tri_distance[t] : rv.tdist[t];
    if (!(d < rp.d1)) return;
    const float *bary = rv.tri_bary ? rv.tri_bary + 3 * t : rv.tbary + 3 * t;
    const float prox = fmaxf(__fdiv_rn(__fsub_rn(rp.d1, d), rp.d1), 0.0f);
    const int v[3] = {rv.tris[3 * t], rv.tris[3 * t + 1], rv.tris[3 * t + 2]};
    float lmax = 1.0e-20f;
#pragma unroll
    for (int k = 0; k < 3; ++k) lmax = fmaxf(lmax, len3(q + 3 * v[(k + 1) % 3], q + 3 * v[k]));
    const float h = rp.min_edge;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        // the edge opposite vertex k is local pair 2 - k of (1,0) (2,0) (2,1)
        const int i = v[(k + 1) % 3], j = v[(k + 2) % 3];
        if (kinematic_edge(rv, i, j)) continue;
        const float L = len3(q + 3 * i, q + 3 * j);
        if (!(L >= __fmul_rn(2.0f, h))) continue;
        const float w = __fsub_rn(1.0f, bary[k]);
        float val = __fmul_rn(__fdiv_rn(L, h), __fdiv_rn(L, lmax));
        val = __fmul_rn(__fmul_rn(__fmul_rn(val, rp.tri_w), prox), w);
        val = fmaxf(val, 0.0f);
        const int s = rv.tri_edge[3 * t + (2 - k)];
        atomicMax(reinterpret_cast<int *>(rv.score + s), __float_as_int(val));
    }
}

__global__ void refine_state_kernel(RefineViews rv, float threshold) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= rv.nnzb) return;
    const int a = rv.slot_row[s], b = rv.col_idx[s];
    const bool cand = rv.ctrl[kCtrlRefining] && a < b && !kinematic_edge(rv, a, b) && rv.score[s] > threshold;
    rv.state[s] = cand ? kAvailable : 0;
    rv.blocked[s] = 0;
}

// Each tet picks the edge it holds, or its best available candidate (score,
// then the smaller slot); the other available candidates of the tet are
// blocked for this sweep.
__global__ void refine_candidate_kernel(RefineViews rv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rv.T) return;
    int e[6];
#pragma unroll
    for (int p = 0; p < 6; ++p) e[p] = rv.tet_edge[(size_t)t * 6 + p];
    int held = -1;
#pragma unroll
    for (int p = 0; p < 6; ++p)
        if (rv.state[e[p]] == kSelected) held = e[p];
    if (held >= 0) {
        rv.cand[t] = held;
        return;
    }
    int best = -1;
    float best_sc = 0.0f;
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        if (rv.state[e[p]] != kAvailable) continue;
        const float sc = rv.score[e[p]];
        if (best < 0 || sc > best_sc || (sc == best_sc && e[p] < best)) {
            best = e[p];
            best_sc = sc;
        }
    }
    rv.cand[t] = best;
#pragma unroll
    for (int p = 0; p < 6; ++p)
        if (e[p] != best && rv.state[e[p]] == kAvailable) rv.blocked[e[p]] = 1;
}

__global__ void refine_select_kernel(RefineViews rv) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= rv.nnzb) return;
    if (rv.state[s] == kAvailable && !rv.blocked[s]) rv.state[s] = kSelected;
    rv.blocked[s] = 0;
}

// A tet whose pick was selected takes its other edges out of the race.
__global__ void refine_lock_kernel(RefineViews rv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rv.T) return;
    const int c = rv.cand[t];
    if (c < 0 || rv.state[c] != kSelected) return;
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        const int e = rv.tet_edge[(size_t)t * 6 + p];
        if (e != c && rv.state[e] != kSelected) rv.state[e] = kUnavailable;
    }
}

// Split flags: per tet its selected edge, per edge whether it was selected,
// per tri its selected edge; the counts the scans turn into offsets.
__global__ void refine_count_kernel(RefineViews rv) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rv.T) {
        int ss = -1;
#pragma unroll
        for (int p = 0; p < 6; ++p) {
            const int e = rv.tet_edge[(size_t)i * 6 + p];
            if (rv.state[e] == kSelected) ss = e;
        }
        rv.split_slot[i] = ss;
        rv.tet_cnt[i] = ss >= 0 ? 2 : 1;
    }
    if (i < rv.nnzb) rv.edge_cnt[i] = rv.state[i] == kSelected ? 1 : 0;
    if (i < rv.m) {
        int ss = -1;
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            const int e = rv.tri_edge[3 * i + p];
            if (rv.state[e] == kSelected) ss = e;
        }
        rv.tri_slot[i] = ss;
        rv.tri_cnt[i] = ss >= 0 ? 2 : 1;
    }
}

// ---- exclusive scan in place: x[0..n) -> offsets, x[n] = total ----------

__device__ __forceinline__ int block_exclusive_scan(int v, int *s_warp, int &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kRefineThreads / 32 ? s_warp[lane] : 0;
        int wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= off) wi += o;
        }
        if (lane < kRefineThreads / 32) s_warp[lane] = wi - w;
        if (lane == kRefineThreads / 32 - 1) s_warp[kRefineThreads / 32] = wi;
    }
    __syncthreads();
    const int out = s_warp[warp] + incl - v;
    total = s_warp[kRefineThreads / 32];
    __syncthreads();
    return out;
}

__global__ void scan_block_sums_kernel(const int *__restrict__ x, int64_t n, int *__restrict__ sums) {
    __shared__ int s_warp[kRefineThreads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    int v = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) v += x[base + k];
    int total;
    block_exclusive_scan(v, s_warp, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_sums_kernel(int *__restrict__ sums, int64_t nb) {
    __shared__ int s_warp[kRefineThreads / 32 + 1];
    int carry = 0;
    for (int64_t base = 0; base < nb; base += kRefineThreads) {
        const int64_t i = base + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, s_warp, total);
        if (i < nb) sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void scan_apply_kernel(int *__restrict__ x, int64_t n, const int *__restrict__ sums, int64_t nb) {
    __shared__ int s_warp[kRefineThreads / 32 + 1];
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    int local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? x[base + k] : 0;
        local += v[k];
    }
    int total;
    int off = block_exclusive_scan(local, s_warp, total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) x[base + k] = off;
        off += v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) x[n] = sums[nb];
}

cudaError_t scan_in_place(int *x, int64_t n, int *tmp, cudaStream_t s) {
    const int64_t nb = std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock);
    scan_block_sums_kernel<<<(unsigned)nb, kRefineThreads, 0, s>>>(x, n, tmp);
    scan_sums_kernel<<<1, kRefineThreads, 0, s>>>(tmp, nb);
    scan_apply_kernel<<<(unsigned)nb, kRefineThreads, 0, s>>>(x, n, tmp, nb);
    count_launches(3);
    return cudaGetLastError();
}

// Totals, the capacity guard (check_split_capacity / drop_candidates_on_
// overflow, refinement.py:578-604) and the counts the caller reads.
__global__ void refine_finalize_kernel(RefineViews rv, RefineParams rp, int *counts) {
    const int added = rv.edge_cnt[rv.nnzb];
    const int T_new = rv.tet_cnt[rv.T];
    const int m_new = rv.tri_cnt[rv.m];
    const bool over = added > 0 && ((int64_t)T_new > rp.max_tets || (int64_t)rv.n + added > rp.max_particles ||
                                    (int64_t)m_new > rp.max_tris);
    const bool apply = added > 0 && !over;
    rv.ctrl[kCtrlApply] = apply ? 1 : 0;
    counts[0] = apply ? rv.n + added : rv.n;
    counts[1] = apply ? T_new : rv.T;
    counts[2] = apply ? m_new : rv.m;
    counts[3] = apply ? added : 0;
    counts[4] = over ? 1 : 0;
    counts[5] = rv.ctrl[kCtrlRefining];
    counts[6] = 0;
    counts[7] = 0;
}

// Old vertices' rest positions; each new vertex at split_position along its
// edge from the lower to the higher vertex (claim_new_vertices,
// refinement.py:697-730).
__global__ void refine_vertex_out_kernel(RefineViews rv, RefineParams rp, RefineOut out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rv.n) {
#pragma unroll
        for (int c = 0; c < 3; ++c) out.rest[3 * i + c] = rv.rest[3 * i + c];
        return;
    }
    const int64_t s = i - rv.n;
    if (s >= rv.nnzb || !rv.ctrl[kCtrlApply]) return;
    if (rv.edge_cnt[s + 1] == rv.edge_cnt[s]) return;
    const int a = rv.slot_row[s], b = rv.col_idx[s];
    const int64_t v = rv.n + rv.edge_cnt[s];
    const float t = rp.split_t;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        out.q[3 * v + c] = lerp_rn(out.q[3 * a + c], out.q[3 * b + c], t);
        out.qd[3 * v + c] = lerp_rn(out.qd[3 * a + c], out.qd[3 * b + c], t);
        out.rest[3 * v + c] = lerp_rn(rv.rest[3 * a + c], rv.rest[3 * b + c], t);
    }
}

// Tets (scatter_tets, refinement.py:733-824): an unsplit tet is copied with
// lumped mass density / (6 det DmInv); a split one becomes two children,
// child 0 with local vertex i of its split pair (i, j) replaced by the new
// vertex, child 1 with j, each with DmInv from its rest edges, mass
// det(Dm) / 6 * density and the parent's s, lambda and materials.
__global__ void refine_tet_out_kernel(RefineViews rv, RefineParams rp, RefineOut out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rv.T) return;
    const bool apply = rv.ctrl[kCtrlApply] != 0;
    const int dst = apply ? rv.tet_cnt[t] : t;
    const int ss = apply ? rv.split_slot[t] : -1;
    const int4 tt = rv.tets[t];
    const int vid[4] = {tt.x, tt.y, tt.z, tt.w};
    float M[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) M[i] = rv.dminv[(size_t)t * 9 + i];
    float sv[6], lv[6], mat[3];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        sv[i] = rv.stretch[(size_t)t * 6 + i];
        lv[i] = rv.lambda[(size_t)t * 6 + i];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) mat[i] = rv.materials[(size_t)t * 3 + i];
    const int children = ss >= 0 ? 2 : 1;
    int pi = 0, pj = 0;
    if (ss >= 0) {
        const int lo = rv.slot_row[ss], hi = rv.col_idx[ss];
#pragma unroll
        for (int p = 0; p < 6; ++p) {
            const int a = vid[kTetPairI[p]], b = vid[kTetPairJ[p]];
            if ((a == lo && b == hi) || (a == hi && b == lo)) {
                pi = kTetPairI[p];
                pj = kTetPairJ[p];
            }
        }
        rv.split_pair[t] = pi * 4 + pj;
    }
    const int nv = ss >= 0 ? rv.n + rv.edge_cnt[ss] : -1;
    for (int c = 0; c < children; ++c) {
        const int64_t o = (int64_t)dst + c;
        int cv[4] = {vid[0], vid[1], vid[2], vid[3]};
        float P[9];
        float tm;
        if (ss >= 0) {
            cv[c == 0 ? pi : pj] = nv;
            float x[4][3];
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
                for (int d = 0; d < 3; ++d) x[k][d] = out.rest[3 * (int64_t)cv[k] + d];
            float Dm[9];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int k = 0; k < 3; ++k) Dm[3 * r + k] = __fsub_rn(x[k + 1][r], x[0][r]);
            const float det = inverse3_rn(Dm, P);
            tm = __fmul_rn(__fdiv_rn(det, 6.0f), rp.density);
        } else {
#pragma unroll
            for (int i = 0; i < 9; ++i) P[i] = M[i];
            tm = __fdiv_rn(rp.density, __fmul_rn(6.0f, det3_rn(M)));
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) out.tets[4 * o + k] = cv[k];
#pragma unroll
        for (int i = 0; i < 9; ++i) out.poses[9 * o + i] = P[i];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            out.stretch[6 * o + i] = sv[i];
            out.lambda[6 * o + i] = lv[i];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) out.materials[3 * o + i] = mat[i];
        rv.tmass[o] = tm;
    }
}

// Lumped masses of the refined mesh: per vertex the tets' density * volume
// / 4 in ascending (old tet, child) order; kinematic vertices stay
// kinematic, the others get 1 / mass.  A pass that splits nothing copies the
// masses through.
__global__ void refine_mass_kernel(RefineViews rv, RefineOut out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool apply = rv.ctrl[kCtrlApply] != 0;
    if (i < rv.n) {
        if (!apply) {
            out.mass[i] = rv.mass[i];
            out.inv_mass[i] = rv.inv_mass[i];
            return;
        }
        float acc = 0.0f;
        for (int k = rv.vert_start[i]; k < rv.vert_start[i + 1]; ++k) {
            const int code = rv.vert_code[k];
            const int t = code >> 2, corner = code & 3;
            const int base = rv.tet_cnt[t];
            if (rv.split_slot[t] < 0) {
                acc = __fadd_rn(acc, __fdiv_rn(rv.tmass[base], 4.0f));
            } else {
                const int pr = rv.split_pair[t];
                const int pi = pr >> 2, pj = pr & 3;
                if (pi != corner) acc = __fadd_rn(acc, __fdiv_rn(rv.tmass[base], 4.0f));
                if (pj != corner) acc = __fadd_rn(acc, __fdiv_rn(rv.tmass[base + 1], 4.0f));
            }
        }
        out.mass[i] = acc;
        out.inv_mass[i] = (rv.inv_mass[i] != 0.0f && acc > 0.0f) ? __fdiv_rn(1.0f, acc) : 0.0f;
        return;
    }
    const int64_t s = i - rv.n;
    if (s >= rv.nnzb || !apply || rv.edge_cnt[s + 1] == rv.edge_cnt[s]) return;
    float acc = 0.0f;
    for (int k = rv.edge_start[s]; k < rv.edge_start[s + 1]; ++k) {
        const int base = rv.tet_cnt[rv.edge_tet[k]];
        acc = __fadd_rn(acc, __fdiv_rn(rv.tmass[base], 4.0f));
        acc = __fadd_rn(acc, __fdiv_rn(rv.tmass[base + 1], 4.0f));
    }
    const int64_t v = rv.n + rv.edge_cnt[s];
    out.mass[v] = acc;
    out.inv_mass[v] = acc > 0.0f ? __fdiv_rn(1.0f, acc) : 0.0f;
}

// Surface tris (get_tri_candidate, scatter_tris: refinement.py:827-911).
__global__ void refine_tri_out_kernel(RefineViews rv, RefineOut out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rv.m) return;
    const bool apply = rv.ctrl[kCtrlApply] != 0;
    const int dst = apply ? rv.tri_cnt[t] : t;
    const int ss = apply ? rv.tri_slot[t] : -1;
    const int v[3] = {rv.tris[3 * t], rv.tris[3 * t + 1], rv.tris[3 * t + 2]};
    if (ss < 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) out.tris[3 * (int64_t)dst + k] = v[k];
        return;
    }
    const int lo = rv.slot_row[ss], hi = rv.col_idx[ss];
    int pi = 0, pj = 0;
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const int a = v[kTriPairI[p]], b = v[kTriPairJ[p]];
        if ((a == lo && b == hi) || (a == hi && b == lo)) {
            pi = kTriPairI[p];
            pj = kTriPairJ[p];
        }
    }
    const int nv = rv.n + rv.edge_cnt[ss];
    for (int c = 0; c < 2; ++c) {
        int cv[3] = {v[0], v[1], v[2]};
        cv[c == 0 ? pi : pj] = nv;
#pragma unroll
        for (int k = 0; k < 3; ++k) out.tris[3 * ((int64_t)dst + c) + k] = cv[k];
    }
}

}  // namespace

cudaError_t launch_refine(const RefineViews &rv, const ContactViews &cv, const RefineParams &rp, int *pass_counter,
                          const RefineOut &out, cudaStream_t s) {
    const int tb = blocks_for(rv.T, kRefineThreads);
    const int vb = blocks_for(rv.n, kRefineThreads);
    const int eb = blocks_for(rv.nnzb, kRefineThreads);
    const int mb = blocks_for(rv.m, kRefineThreads);
    const bool geometric = rp.scoring == 1;
    uint64_t launches = 0;
    refine_begin_kernel<<<1, 1, 0, s>>>(rv.ctrl, pass_counter, rp.refine_every);
    ++launches;
    const bool contact = cv.on && cv.n_shapes > 0;
    if (contact && rv.m > 0 && (geometric ? !rv.tri_distance : !rv.vertex_scores)) {
        refine_tri_inputs_kernel<<<mb, kRefineThreads, 0, s>>>(rv, cv, out.q);
        ++launches;
    }
    if (geometric ? !rv.particle_distance : !rv.vertex_scores) {
        refine_vertex_inputs_kernel<<<vb, kRefineThreads, 0, s>>>(rv, cv, out.q);
        ++launches;
    }
    if (rv.T > 0) {
        refine_tet_kernel<<<tb, kRefineThreads, 0, s>>>(rv, out.q, geometric ? 1 : 0);
        ++launches;
    }
    if (geometric) {
        if (rv.T > 0) {
            refine_stats_kernel<<<1, 32, 0, s>>>(rv, tb);
            ++launches;
        } else {
            cudaMemsetAsync(rv.mean_density, 0, sizeof(float), s);
        }
    }
    refine_score_kernel<<<eb, kRefineThreads, 0, s>>>(rv, cv, rp, out.q);
    ++launches;
    if (geometric && rv.m > 0 && (rv.tri_distance || contact)) {
        refine_tri_score_kernel<<<mb, kRefineThreads, 0, s>>>(rv, rp, out.q);
        ++launches;
    }
    refine_state_kernel<<<eb, kRefineThreads, 0, s>>>(rv, rp.threshold);
    ++launches;
    if (rv.T > 0) {
        for (int k = 0; k < rp.sweeps; ++k) {
            refine_candidate_kernel<<<tb, kRefineThreads, 0, s>>>(rv);
            refine_select_kernel<<<eb, kRefineThreads, 0, s>>>(rv);
            refine_lock_kernel<<<tb, kRefineThreads, 0, s>>>(rv);
            launches += 3;
        }
    }
    const int64_t cnt_n = std::max<int64_t>({(int64_t)rv.T, rv.nnzb, (int64_t)rv.m});
    refine_count_kernel<<<blocks_for(cnt_n, kRefineThreads), kRefineThreads, 0, s>>>(rv);
    ++launches;
    count_launches(launches);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = scan_in_place(rv.tet_cnt, rv.T, rv.scan_tmp, s);
    if (e == cudaSuccess) e = scan_in_place(rv.edge_cnt, rv.nnzb, rv.scan_tmp, s);
    if (e == cudaSuccess) e = scan_in_place(rv.tri_cnt, rv.m, rv.scan_tmp, s);
    if (e != cudaSuccess) return e;
    launches = 0;
    refine_finalize_kernel<<<1, 1, 0, s>>>(rv, rp, out.counts);
    refine_vertex_out_kernel<<<blocks_for((int64_t)rv.n + rv.nnzb, kRefineThreads), kRefineThreads, 0, s>>>(rv, rp,
                                                                                                           out);
    launches += 2;
    if (rv.T > 0) {
        refine_tet_out_kernel<<<tb, kRefineThreads, 0, s>>>(rv, rp, out);
        ++launches;
    }
    refine_mass_kernel<<<blocks_for((int64_t)rv.n + rv.nnzb, kRefineThreads), kRefineThreads, 0, s>>>(rv, out);
    ++launches;
    if (rv.m > 0) {
        refine_tri_out_kernel<<<mb, kRefineThreads, 0, s>>>(rv, out);
        ++launches;
    }
    count_launches(launches);
    return cudaGetLastError();
}

}  // namespace mfem
