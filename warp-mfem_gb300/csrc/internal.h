// Internal definitions shared by the translation units of libmfem_gb300.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "mfem_gb300.h"

namespace mfem {

// Element Hessian blocks kept per tet: the upper (k <= l) 3x3 blocks of the
// symmetric 12x12 G^T H_lambda G, numbered row by row:
//   0:(0,0) 1:(0,1) 2:(0,2) 3:(0,3) 4:(1,1) 5:(1,2) 6:(1,3) 7:(2,2) 8:(2,3) 9:(3,3)
constexpr int kKeBlocks = 10;
constexpr int kKeFloats = kKeBlocks * 9;
constexpr int kFeFloats = 12;

__host__ __device__ __forceinline__ int ke_block(int k, int l) {
    // k <= l
    return k * 4 - (k * (k - 1)) / 2 + (l - k);
}

// Packed upper triangle of a symmetric 6x6, row-major: (0,0)..(0,5),(1,1)..(5,5).
__host__ __device__ __forceinline__ constexpr int sym6_index(int i, int j) {
    return (i <= j) ? (i * 6 - (i * (i - 1)) / 2 + (j - i)) : (j * 6 - (j * (j - 1)) / 2 + (i - j));
}

// Per-solve outcome written by the PCG kernel (same layout as mfem_solve_stats).
struct SolveStats {
    int32_t iterations;
    int32_t status;
    float rel_residual;
    float reserved;
};

// Device views used by the kernels.  All arrays are owned by the plan.
struct TetViews {
    int n_tets;
    const int4 *tets;          // [T]
    const float *dminv;        // [T][9] row-major DmInv
    const float *materials;    // [T][3] (mu, lambda, damping)
    float *stretch;            // [T][6] s
    float *lambda;             // [T][6]
    // per-tet Newton terms, component-major [k][T]
    float *c;                  // [6][T]
    float *G;                  // [72][T]
    float *g_s;                // [6][T]
    float *H_l;                // [21][T]
    float *H_si;               // [21][T]
    float *g_l;                // [6][T]
    // element contributions gathered by the assembly, tet-major
    float *Ke;                 // [T][90]
    float *fe;                 // [T][12]
    const unsigned char *energy_code;  // [T] per-tet energy (batched bodies), or null: the plan's
    // tets with det F < 1e-3, listed by the element kernel for its float64 pass
    int *degenerate;           // [T]
    unsigned *n_degenerate;    // [1]
};

struct VertexViews {
    int n;
    const float *mass;         // [n] particle_mass (kinetic gradient)
    const float *hess_diag;    // [n] Hessian mass + attachment stiffness, (M+Q) diagonal
    const float *pin_k;        // [n] attachment stiffness (0 if free)
    const float *pin_target;   // [n][3]
    float *x_tilde;            // [n][3]
    float *x_start;            // [n][3]
    float *rhs;                // [n][3]
    float *dx;                 // [n][3]
    float *Minv;               // [n_pad][9]
    const int *vertex_body;    // [n] body of each vertex (batched bodies), or null
    const float *body_gravity; // [bodies][3]
};

// Independent bodies solved in one persistent launch (pcg_batched.cu): each
// body's PCG runs on a group of CTAs with its own scalars, barrier and
// stopping test.  A CTA runs the tasks [task_ptr[c], task_ptr[c+1]) in
// order; a task is (body, rank in the group, group size, first CTA of the
// group), and a group of more than one CTA is its CTAs' only task.
struct BatchViews {
    int n_bodies;
    const int *body_row;       // [bodies + 1] vertex (block row) offsets
    const int *task_ptr;       // [ctas + 1]
    const int4 *task;          // [tasks]
    int ctas;
    int threads;               // threads per CTA
    float *partials;           // [2][ctas][4]
    unsigned long long *counter;  // [bodies] group barriers, never reset
    float *z, *p0, *p1, *r, *Ap;  // [n][3]
    SolveStats *stats;         // [max solves per step][bodies]
    // Factor preconditioners on H's lower block pattern (columns <= row,
    // ascending, the diagonal last): use_precond 2 applies M = F^T F (FSAI),
    // 3 applies M = F F^T (learned).  F's blocks sit in the lower CSR; the
    // upper CSR (columns >= row) holds the transposed blocks, (F^T)_ij =
    // F_ji^T, so both passes are row-wise gathers.
    const int *lrow, *lcol;    // [n + 1], [nnzl]
    const int *urow, *ucol;    // [n + 1], [nnzl]
    const int *umap;           // [nnzl] upper entry -> lower entry of the transposed block
    float *Lval;               // [nnzl][9] F, row-major blocks (the setup's output)
    float *Uval;               // [nnzl][9] F^T in upper-CSR order
    // BF16 copies the PCG passes read, kFactorLd values per block (the 10th
    // is padding: 20-byte blocks keep 4-byte loads aligned); M = F^T F or
    // F F^T stays symmetric positive definite whatever F's rounding
    __nv_bfloat16 *Lb, *Ub;
    float *y;                  // [n][3] the first pass's output
    float *dx0;                // [n][3] warm start kept for a block-Jacobi retry
    // FSAI setup: per row, the H slot (or -1) of every pair (a, b), b <= a,
    // of the row's lower columns, a-major; rows with more than kFsaiMaxCols
    // lower blocks have none
    const int64_t *fsai_pair_ptr;  // [n + 1]
    const int *fsai_pairs;
    const int *fsai_big_rows;  // [n_fsai_big] rows with more than 8 lower blocks
    int n_fsai_big;
    int nnzl;
};

// The learned factor net (preconditioner 3): weights in device layout and
// its per-vertex work arrays.  BF16 weight matrices are stored [out][in]
// with the row padded by 8 elements (conflict-free fragment loads).
constexpr int kNetWidth = 64;
constexpr int kNetIn = 16;
constexpr int kMpLd = 2 * kNetWidth + 8;  // message-passing layers: K = 128
constexpr int kNodeLd = kNetWidth + 8;    // node and edge output layers: K = 64
constexpr int kRLd = 16 + 8;              // edge-feature layer: K = 9, padded to 16
constexpr int kNodeOut = 2 * kNetWidth + 8;  // P (64), Q (64), diagonal (6) + 2 zero rows
struct FactorNetViews {
    const float *w_in, *b_in;          // [64][16] (BF16-rounded values), [64]
    const __nv_bfloat16 *w_mp[3];      // [64][kMpLd]
    const float *b_mp[3];              // [64]
    const __nv_bfloat16 *w_node;       // [kNodeOut][kNodeLd]
    const float *b_node;               // [kNodeOut]
    const __nv_bfloat16 *w_r;          // [64][kRLd]
    const __nv_bfloat16 *w_o;          // [16][kNodeLd], rows 9..15 zero
    const float *b_o;                  // [16]
    const float *vstatic;              // [n][4] static vertex features
    float *s, *ld;                     // [n] d^-1/2, log10 d
    float *w;                          // [nnzb] aggregation weights (0 on the diagonal)
    float *winv;                       // [n] 1 / sum of the row's weights
    float *h;                          // [n][64]
    __nv_bfloat16 *hb[2];              // [n][64] BF16 copies of h (ping-pong between layers)
    __nv_bfloat16 *pb, *qb;            // [n][64] P h + b_p, Q h
    const int *lslot;                  // [nnzl] H slot of each lower block
    const int *erow, *elow;            // [n_edges] row and lower entry of each off-diagonal lower block
    int n_edges;
    int ready;                         // weights and static features are set
};

constexpr int kFactorLd = 10;
constexpr int kFsaiMaxCols = 16;  // lower block columns a row may have for FSAI
constexpr int kFsaiDim = 3 * kFsaiMaxCols;

struct BsrViews {
    int n;
    int64_t nnzb;
    const int *row_ptr;        // [n+1]
    const int *col_idx;        // [nnzb]
    float *values;             // [nnzb][9]
    // contribution lists sorted by slot, packed into warp-sized chunks
    int n_chunks;
    const int *chunk_ptr;      // [n_chunks+1]
    const int *contrib_code;   // e*16 + k*4 + l, or -(row+1) for an empty diagonal
    const int *contrib_slot;   // slot of each contribution
};

struct PcgWork {
    int n_pad;                 // rows of the exchanged vectors, n rounded up to 4
    float *pub;                // 6 x [n_pad][3] vectors published between CTAs each iteration
    float *partials;           // [2][256][4] per-CTA partial sums, double buffered by barrier parity
    unsigned long long *counter;  // grid barrier arrivals, never reset
    int *error;                // sticky device error flag (timeouts)
    SolveStats *stats;         // [max solves per step]
};

// Per-Newton-iteration outcome of the line search (same layout as
// mfem_line_search_stats).
struct LineSearchStats {
    int32_t evaluations;
    int32_t accepted;
    float alpha;
    int32_t status;
    double f0, f1, t;
};

constexpr int kLsMaxCtas = 512;  // capacity of the line search's per-CTA partials

struct LineSearchWork {
    float *ds;                     // [6][T] stretch direction of the local solve
    double *local_partials;        // [local_blocks][2] (merit, slope) per local-solve block
    int local_blocks;
    double *partials;              // [2][kLsMaxCtas][3] per-CTA sums, double buffered by round parity
    unsigned long long *counter;   // grid barrier arrivals, never reset
    LineSearchStats *stats;        // [max solves per step]
    int ctas;                      // persistent CTAs, fixed for the plan
    int max_iter;
    float alpha0, tau, c, threshold;
};

// Contact against rigid shapes: per-vertex barrier and lagged friction,
// per-tri barrier against capsules.  on == 0: no contact term at all.
constexpr int kTriData = 12;  // per tri: d, k b, k b', k max(b'', 0), n[3], w[3], shape, unused
constexpr int kMaxShapes = 64;

struct ContactViews {
    int on;
    int n_shapes;
    const int *type;          // [S] shape type (contact.cuh kShape*)
    const float *pose;        // [S][7] shape pose in its body's frame
    const float *scale;       // [S][3] capsule (radius, half height, -)
    const int *body;          // [S] body index, < 0: static
    const float *mu;          // [S] Coulomb coefficient
    const float *body_q;      // [B][7] body poses of the step
    int friction;             // some shape has mu > 0
    float d0, d1, k, eps_v;
    float q[3];               // barrier extrapolation (b, b', b'') at d0
    // lagged friction, frozen at the start of the step
    float *normal_lagged;     // [n][3]
    float *force_lagged;      // [n]
    int *shape_lagged;        // [n]
    // per Newton iteration
    float *vblock;            // [n][9] barrier + friction Hessian block
    float *vgrad;             // [n][3] barrier + friction gradient
    float *venergy;           // [n]
    float *gtot;              // [n][3] vertex + tri gradient
    int n_tris;               // 0: no tri contact
    const int *tris;          // [m][3]
    float *tri;               // [m][kTriData]
    const int *vt_ptr;        // [n+1] incident tri corners per vertex
    const int *vt_code;       // tri * 3 + corner
    int tri_code_base;        // assembly codes >= base are tri blocks
};

// Mixed-precision global solve (pcg_mixed.cu): iterative refinement with an
// fp64 residual around a PCG on 16-bit blocks with per-row scales.
constexpr int kIrBf16 = 1;
constexpr int kIrFp16 = 2;
constexpr int kIrFp32 = 3;  // the fp32 H in the inner PCG from the start: no 16-bit copy

struct IrStats {               // same layout as mfem_mixed_solve_stats
    int32_t outer_iterations;
    int32_t inner_iterations;
    int32_t status;
    int32_t fp32_inner;        // the solve restarted with the fp32 H in the inner PCG
    double rel_residual;       // fp64 ||g - H dx|| / ||g||
};

struct IrWork {
    int mode;                  // kIrBf16, kIrFp16 or kIrFp32
    int ctas;                  // inner PCG CTAs
    int outer_max;
    float inner_tol;
    double outer_tol;
    void *lowp;                // [nnzb][9] bf16 / fp16, H / row scale
    float *row_scale;          // [n]
    float2 *dx_pair;           // [2][n][3] double-buffered solution, each value hi + lo of two floats
    double *dx_out;            // [n][3] the latest iterate
    float *e;                  // [n][3] inner correction
    float *res;                // [n][3] fp32 copy of the fp64 residual (inner rhs)
    float *z, *p0, *p1, *r, *Ap;  // inner PCG vectors [n][3]
    double *partials;          // [2][256][4] fp64 partial sums of the inner PCG
    unsigned long long *counter;  // inner PCG grid barrier, never reset
    double *res_partials;      // [residual blocks][2]
    unsigned *ticket;          // last-block detection of the residual kernel
    int *state;                // done, outer, inner, pending, parity, status, fp32 inner, restart
    float *dx_init;            // [n][3] the warm start, for a restart
    double *best;              // [1] smallest fp64 relative residual of the solve so far
    IrStats *stats;            // [max solves per step]
    // inner solves in the persistent factor PCG (a plan with pcg_variant 4):
    uint32_t *hq_words;        // [nnzb][5] the 16-bit blocks as pairs in words, nine values and a zero
                               // (20 bytes, 4-byte aligned), for the persistent factor PCG (else null)
    float *scale;              // [2] 1 / ||r|| and ||r|| of the latest fp64 residual
    // the whole refinement in one launch of the persistent factor PCG: the
    // iterate as hi + lo planes (rows padded to n_pad for bulk copies)
    float *xf_hi, *xf_lo;      // [n_pad][3]
};

// Row partition and shared-memory plan of the persistent PCG.
struct PcgLayout {
    // kFactor: the persistent PCG with a factor preconditioner (pcg_factor.cu);
    // kGlobalMemory: requested in the config only, the mesh then runs the
    // global-memory PCG as a one-body batch (reported as variant 0)
    enum { kAuto = 0, kStandard = 1, kSingleReduction = 2, kGather = 3, kFactor = 4, kGlobalMemory = 5 };
    const int4 *cta_info;      // device [ctas]: (row_lo, row_hi, win_lo, win_hi)
    const int4 *factor_info = nullptr;  // kFactor, device [ctas]: (y_lo, y_hi, r_lo, r_hi)
    int variant = kSingleReduction;
    int rows_max = 0, blk_max = 0, win_max = 0;
    int y_max = 0, r_max = 0;  // kFactor: longest row ranges Y and R of a CTA
    int f0_max = 0, f1_max = 0;  // kFactor: most first- / second-pass factor blocks of a CTA
    int factor_cache = 0;      // kFactor: factor rows a CTA keeps in shared memory (0 none, 1 row
                               // pointers, 2 row pointers, columns and blocks)
    int cache_matrix = 0;      // 1: each CTA keeps its slice of H in shared memory
    size_t smem = 0;           // dynamic shared memory per CTA
};

// One edge-bisection pass of adaptive refinement (refine.cu) over a plan's
// mesh.  Edges are the upper off-diagonal slots of H's sparsity (row < col),
// so a slot index doubles as the edge's id and ascending slots are ascending
// (min vertex, max vertex) keys.
constexpr int kRefineCtrl = 4;  // device control words: refining pass, pass applied
struct RefineViews {
    // the plan's mesh
    int n, T, m;
    int64_t nnzb;
    int energy;
    const int4 *tets;
    const float *dminv, *materials, *stretch, *lambda;
    const float *rest, *mass, *inv_mass;  // [n][3], [n], [n]
    const int *tris;                      // [m][3] (the plan's contact tris)
    const int *col_idx;                   // [nnzb]
    const int *slot_row;                  // [nnzb] row of each slot
    const int *tet_edge;                  // [T][6] edge of local pair (1,0) (2,0) (2,1) (3,0) (3,1) (3,2)
    const int *tri_edge;                  // [m][3] edge of local pair (1,0) (2,0) (2,1)
    const int *edge_start;                // [nnzb + 1] tets of each edge, ascending, in edge_tet
    const int *edge_tet;                  // [6 T]
    const int *vert_start;                // [n + 1] tets of each vertex, ascending, in vert_code
    const int *vert_code;                 // [4 T] tet * 4 + corner
    // optional inputs (null: computed from the plan's state and contact)
    const float *tet_scores, *vertex_scores, *particle_distance, *tri_distance, *tri_bary;
    const int *particle_shape_id;
    // work
    float *e_tet, *dens, *lmax;          // [T]
    float *vscore, *vdist;               // [n]
    int *vsid;                           // [n]
    float *tdist, *tbary, *tenergy;      // [m], [m][3], [m]
    double *partials;                    // [stat blocks]
    float *mean_density;                 // [1]
    float *score;                        // [nnzb]
    unsigned char *state, *blocked;      // [nnzb]
    int *cand, *split_slot, *split_pair; // [T]
    int *tet_cnt;                        // [T + 1] 1 + split, then its exclusive scan
    int *edge_cnt;                       // [nnzb + 1] selected, then its exclusive scan
    int *tri_slot;                       // [m]
    int *tri_cnt;                        // [m + 1]
    int *scan_tmp;                       // block sums of the scans
    int64_t scan_tmp_len;
    float *tmass;                        // [max_tets] lumped mass of each new tet
    int *ctrl;                           // [kRefineCtrl]
};

struct RefineParams {
    int scoring;  // 0 legacy, 1 geometric
    float threshold, tet_w, vert_w, pen_score, min_edge, d1, el_w, vc_w, tri_w, split_t, density;
    int sweeps, refine_every;
    int max_particles, max_tets, max_tris;
};

struct RefineOut {
    int *tets;
    float *poses, *materials, *stretch, *lambda, *rest, *mass, *inv_mass;
    int *tris;
    int *counts;
    float *q, *qd;  // the caller's positions and velocities, rows [n, n + new) written
};

cudaError_t launch_refine(const RefineViews &rv, const ContactViews &cv, const RefineParams &rp, int *pass_counter,
                          const RefineOut &out, cudaStream_t s);

// Host-side symbolic analysis (symbolic.cpp).
struct Symbolic {
    std::vector<int32_t> row_ptr, col_idx, tet_slots;
    std::vector<int32_t> chunk_ptr, contrib_code, contrib_slot;
};
bool build_sparsity(int n, int T, const int32_t *tets, std::vector<int32_t> &row_ptr,
                    std::vector<int32_t> &col_idx, std::string &err);
bool build_slot_map(int n, int T, const int32_t *tets, const int32_t *row_ptr, const int32_t *col_idx,
                    int32_t *slots, std::string &err);
// Slots of the 9 blocks (i, j) of each surface tri and the incident tri
// corners (tri * 3 + corner) of each vertex.
bool build_tri_slots(int n, int n_tris, const int32_t *tris, const int32_t *row_ptr, const int32_t *col_idx,
                     int32_t *tri_slots, std::vector<int32_t> &vt_ptr, std::vector<int32_t> &vt_code,
                     std::string &err);
bool build_contributions(int n, int T, const int32_t *tets, const int32_t *row_ptr,
                         const int32_t *slots, Symbolic &sym, std::string &err, int n_tris = 0,
                         const int32_t *tri_slots = nullptr);

// Kernel launchers (each returns cudaGetLastError()).
cudaError_t launch_initial_stretch(const float *rest_q, const TetViews &tv, cudaStream_t s);
cudaError_t launch_predict(const float *q_in, const float *qd_in, float *q_out, const float *gravity_dev,
                           float dt, const VertexViews &vv, cudaStream_t s);
// Sets the element kernels' shared-memory limit (once per device, before the
// first launch).  With diagnostics the element stage also writes H_s^-1 and
// g_lambda, which the step itself does not read.
cudaError_t prepare_element_kernels();
cudaError_t launch_element(const float *x, int energy, const TetViews &tv, bool diagnostics, cudaStream_t s);
cudaError_t launch_assemble(const float *x, float dt, float singular_threshold, int use_precond,
                            const TetViews &tv, const VertexViews &vv, const BsrViews &bv, const ContactViews &cv,
                            cudaStream_t s);
cudaError_t launch_contact(const float *x, float dt, const ContactViews &cv, const VertexViews &vv, cudaStream_t s);
cudaError_t launch_contact_begin(const ContactViews &cv, const VertexViews &vv, cudaStream_t s);
cudaError_t launch_local_solve(float *x, const TetViews &tv, const VertexViews &vv, cudaStream_t s);
// Local solve that leaves x and s for the line search: writes lambda, ds and
// the per-block partial sums of the merit function and the slope.
cudaError_t launch_local_solve_deferred(const float *x, int energy, float dt, const TetViews &tv,
                                        const VertexViews &vv, const ContactViews &cv, const LineSearchWork &w,
                                        cudaStream_t s);
// blocks of the deferred local solve: tets, then max(vertices, contact tris)
int local_solve_blocks(int n_tets, int n_vertex_range);
cudaError_t launch_line_search(float *x, int energy, float dt, const TetViews &tv, const VertexViews &vv,
                               const ContactViews &cv, const LineSearchWork &w, int *error, int slot,
                               cudaStream_t s);
cudaError_t line_search_max_ctas(int device, int *ctas);
cudaError_t launch_velocity(const float *q_out, float *qd_out, float dt, const VertexViews &vv, cudaStream_t s);
cudaError_t launch_pcg(const BsrViews &bv, const VertexViews &vv, const PcgWork &w, const PcgLayout &L, int ctas,
                       int slot, float tol, int maxiter, int use_precond, cudaStream_t s);
// The single-reduction PCG (L a kSingleReduction layout) as one inner solve of
// the refinement's launch sequence: block-Jacobi on the fp32 H, ir.res to
// inner_tol from 0, the correction in ir.e, ir.state updated.
cudaError_t launch_pcg_inner(const BsrViews &bv, const VertexViews &vv, const IrWork &ir, const PcgWork &w,
                             const PcgLayout &L, int ctas, int slot, int maxiter, cudaStream_t s);
cudaError_t pcg_max_ctas(int device, int *ctas);
cudaError_t pcg_plan_layout(int device, PcgLayout &L, const int32_t *row_ptr, const int32_t *col_idx, int n,
                            int ctas, int variant, std::vector<int4> &cta_info, std::string &err);
// The persistent PCG with a factor preconditioner (mode 2: M = F^T F, 3: M =
// F F^T; the factor in bw's lower / upper CSR).  The layout fails (err set)
// when a CTA's rows and ranges do not fit in shared memory.  factor = false
// plans it for block-Jacobi inner solves of the mixed refinement only (no
// factor rows in shared memory; mode 2's ranges).
cudaError_t pcg_factor_layout(int device, PcgLayout &L, const int32_t *row_ptr, const int32_t *col_idx, int n,
                              int ctas, int mode, std::vector<int4> &cta_info, std::vector<int4> &factor_info,
                              std::string &err, bool factor = true);
cudaError_t launch_pcg_factor(const BsrViews &bv, const VertexViews &vv, const PcgWork &w, const BatchViews &bw,
                              const PcgLayout &L, int ctas, int slot, float tol, int maxiter, int mode,
                              cudaStream_t s);
cudaError_t launch_true_residual(const BsrViews &bv, const VertexViews &vv, double *out3, cudaStream_t s);
cudaError_t ir_max_ctas(int device, int *ctas);
cudaError_t launch_fsai_setup(const BsrViews &bv, const BatchViews &bw, cudaStream_t s);
cudaError_t launch_factor_transpose(const BatchViews &bw, cudaStream_t s);
cudaError_t launch_factor_net(const BsrViews &bv, const BatchViews &bw, const FactorNetViews &fv, cudaStream_t s);
cudaError_t batch_capacity(int device, int threads, bool factor, int *ctas);
cudaError_t launch_batched_pcg(const BsrViews &bv, const VertexViews &vv, const BatchViews &bw, int *error, int slot,
                               float tol, int maxiter, int use_precond, cudaStream_t s);
int ir_residual_blocks(int n);
// single: the plan's single-reduction layout, or null.  With fp32 blocks and
// block-Jacobi the inner solves run there, one launch a correction.
cudaError_t launch_mixed_solve(const BsrViews &bv, const VertexViews &vv, const IrWork &w, const PcgWork &pw,
                               const BatchViews &fb, const PcgLayout &pl, const PcgLayout *single, int pcg_ctas,
                               int slot, int maxiter, int use_precond, cudaStream_t s);
// The whole mixed refinement in one launch of the persistent factor PCG
// (needs IrWork's xf_hi / xf_lo): the warm start in vv.dx, the solution
// written back there.
cudaError_t launch_pcg_factor_refine(const BsrViews &bv, const VertexViews &vv, const IrWork &ir,
                                     const PcgWork &pw, const BatchViews &bw, const PcgLayout &L, int ctas, int slot,
                                     int maxiter, int mode, cudaStream_t s);
// The inner solve of the mixed refinement, Hq e = r to inner_tol from e = 0,
// in the persistent factor PCG.
cudaError_t launch_pcg_factor_inner(const BsrViews &bv, const VertexViews &vv, const IrWork &w, const PcgWork &pw,
                                    const BatchViews &bw, const PcgLayout &L, int ctas, int slot, int maxiter,
                                    int mode, cudaStream_t s);

// Number of kernels launched by the launchers above (process-wide).
void count_launches(uint64_t k);

// Records the message returned by mfem_plan_last_error(NULL) for a call
// that has no plan; returns `code`.
int set_create_error(int code, const std::string &msg);

}  // namespace mfem
