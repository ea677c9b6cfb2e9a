/*
 * mfem_gb300.h -- C ABI of the GB300 (sm_103a) global step of warp-mfem's
 * mixed variational FEM solver.
 *
 * The reference (gjohns57/warp-mfem) is Python over NVIDIA Warp; it has no
 * FFI.  Each entry point below replaces one stage of its
 * RefinementSolver.step (src/mfem/refinement/solver.py:429-579), cited at the
 * declaration, so a host in any language can drive the same step through
 * plain pointers.  No torch (or other framework) type crosses this boundary.
 *
 * Conventions
 *  - float32 everywhere, like the reference (src/mfem/types.py:4); indices int32.
 *  - vec3 arrays are [n][3], matrices row-major.
 *  - Pointers named d_* are CUDA device pointers, h_* host pointers.
 *  - Every call returns an mfem_status.  Codes >= MFEM_NONFINITE are errors;
 *    mfem_plan_last_error() gives the message.  Solver outcomes of the PCG
 *    (converged / iteration cap / breakdown) are reported per Newton
 *    iteration by mfem_step_stats() and never fail a step, matching the
 *    reference, which uses the CG result whether or not it converged.
 *  - Calls are asynchronous on the given stream unless documented otherwise.
 *    A plan is not thread-safe: one host thread per plan.
 */
#ifndef MFEM_GB300_H
#define MFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mfem_plan mfem_plan;   /* opaque */
typedef struct CUstream_st *mfem_stream; /* a cudaStream_t; NULL = legacy default stream */

typedef enum mfem_status {
    MFEM_OK = 0,
    MFEM_MAXITER = 1,        /* PCG hit cg_max_iterations before the tolerance   */
    MFEM_STAGNATION = 2,     /* PCG broke down (p.Ap <= 0)                       */
    MFEM_NONFINITE = 3,      /* NaN/Inf met in the PCG reductions               */
    MFEM_BAD_ARG = 4,        /* invalid argument or mesh                          */
    MFEM_CUDA_ERROR = 5,     /* a CUDA runtime call failed                        */
    MFEM_TIMEOUT = 6         /* a bounded device-side wait gave up                */
} mfem_status;

typedef enum mfem_energy {
    MFEM_ENERGY_ARAP = 0,        /* src/mfem/refinement/elastic_energy.py:127-253 */
    MFEM_ENERGY_NEOHOOKEAN = 1   /* src/mfem/refinement/elastic_energy.py:255-407 */
} mfem_energy;

/* Solver settings; the fields mirror RefinementSolver's kwargs
 * (src/mfem/refinement/solver.py:56-128). */
typedef struct mfem_config {
    int32_t iterations;                   /* local/global iterations per step (solver.py:304)   */
    int32_t energy;                       /* mfem_energy ("energy", solver.py:108-122)           */
    int32_t cg_max_iterations;            /* solver.py:90, default 1000                          */
    float cg_tolerance;                   /* relative, ||r|| <= tol ||b|| (solver.py:91)         */
    float attachment_stiffness;           /* penalty on inv_mass==0 vertices (solver.py:106)     */
    float preconditioner_singular_threshold; /* |det| below -> identity block (solver.py:93)     */
    int32_t preconditioner;               /* 1 block-Jacobi, 0 none (solver.py:128), 2 FSAI:
                                             M = G^T G, G lower block-triangular on H's pattern,
                                             3 learned: M = L L^T from the factor net
                                             (mfem_plan_set_factor_net); 2 and 3 run the
                                             persistent factor PCG (pcg_variant 4) when its
                                             ranges fit in shared memory, else the
                                             global-memory PCG                                 */
    int32_t use_cuda_graph;               /* capture mfem_step once per argument set and replay  */
    int32_t pcg_ctas;                     /* persistent PCG CTAs; 0 = one per SM                 */
    int32_t pcg_variant;                  /* 0 auto, 1 standard (two reductions per iteration),
                                             2 single-reduction (Chronopoulos-Gear), 3 gather
                                             (standard, no column windows: any vertex order),
                                             4 standard with a factor preconditioner (2 or 3
                                             only), 5 the global-memory PCG as a one-body batch;
                                             factor preconditioners take 0, 4 or 5              */
    /* backtracking line search on the merit function in place of x += dx,
     * s += ds (solver.py:99-103, 185, 539-557; src/mfem/line_search.py:76-163) */
    int32_t line_search;                  /* 1 on (the reference's default), 0 plain update      */
    int32_t line_search_max_iterations;   /* default 20                                          */
    float line_search_alpha0;             /* first step, default 1                               */
    float line_search_tau;                /* step shrink factor, default 0.5                     */
    float line_search_c;                  /* Armijo constant, default 0.01                       */
    float line_search_threshold;          /* slack added to the decrease, default 1e-8           */
} mfem_config;

/* Buffers owned by a plan that mfem_plan_copy_out / _copy_in expose.
 * Layout per tet t (T tets) / vertex v (n vertices) / slot k (nnzb blocks). */
typedef enum mfem_buffer {
    MFEM_BUF_TET_STRETCH = 0,   /* f32 [T][6]  s       (additional_state.tet_stretch)     */
    MFEM_BUF_TET_LAMBDA = 1,    /* f32 [T][6]  lambda  (additional_state.tet_lambda)      */
    MFEM_BUF_CONSTRAINT = 2,    /* f32 [6][T]  c = SYM (sym6(S(F)) - s), component-major  */
    MFEM_BUF_GRAD_CONSTRAINT = 3, /* f32 [72][T] G, entry (i, 3k+a) at (i*12 + 3k+a)*T+t  */
    MFEM_BUF_GRAD_S = 4,        /* f32 [6][T]  g_s                                         */
    MFEM_BUF_H_LAMBDA = 5,      /* f32 [21][T] H_lambda, packed upper triangle row-major  */
    MFEM_BUF_HESS_S_INV = 6,    /* f32 [21][T] H_s^-1, packed upper triangle row-major
                                   (written only with mfem_plan_set_diagnostics on)        */
    MFEM_BUF_G_LAMBDA = 7,      /* f32 [6][T]  g_lambda (diagnostics on only)             */
    MFEM_BUF_ELEMENT_HESSIAN = 8, /* f32 [T][10][3][3] upper blocks (k<=l) of G^T H_l G   */
    MFEM_BUF_ELEMENT_RHS = 9,   /* f32 [T][12] (H_l G)^T g_lambda                          */
    MFEM_BUF_ROW_PTR = 10,      /* i32 [n+1]   BSR row offsets                             */
    MFEM_BUF_COL_IDX = 11,      /* i32 [nnzb]  BSR block columns, ascending per row        */
    MFEM_BUF_TET_SLOTS = 12,    /* i32 [T][16] slot of block (tets[t][k], tets[t][l]) at k*4+l */
    MFEM_BUF_H_VALUES = 13,     /* f32 [nnzb][3][3] global Hessian H                        */
    MFEM_BUF_RHS = 14,          /* f32 [n][3]  g = sum G^T H_l g_l - g_x                    */
    MFEM_BUF_PRECOND = 15,      /* f32 [n][3][3] block-Jacobi inverse diagonal             */
    MFEM_BUF_X_TILDE = 16,      /* f32 [n][3]  predictor x~                                 */
    MFEM_BUF_DX = 17,           /* f32 [n][3]  PCG solution dx (warm start x~ - x)          */
    MFEM_BUF_STRETCH_DIRECTION = 18, /* f32 [6][T] ds of the last local solve (line search on) */
    /* contact (empty until mfem_plan_set_contact turns it on) */
    MFEM_BUF_CONTACT_BLOCK = 19,   /* f32 [n][3][3] barrier + friction Hessian block of each vertex */
    MFEM_BUF_CONTACT_GRADIENT = 20, /* f32 [n][3] barrier + friction + tri barrier gradient      */
    MFEM_BUF_CONTACT_ENERGY = 21,  /* f32 [n]    barrier + friction energy of each vertex        */
    MFEM_BUF_TRI_CONTACT = 22,     /* f32 [m][12] per contact tri: d, k b, k b', k max(b'',0),
                                      n[3], w[3], shape, 0                                     */
    MFEM_BUF_FRICTION_NORMAL = 23, /* f32 [n][3] lagged contact normal of the step               */
    MFEM_BUF_FRICTION_FORCE = 24,  /* f32 [n]    lagged normal force of the step                 */
    MFEM_BUF_MIXED_DX = 25,        /* f64 [n][3] solution of the last mixed-precision solve
                                      (empty with the FP32 solve)                              */
    MFEM_BUF_PRECOND_FACTOR = 26,  /* f32 [nnzl][3][3] factor of preconditioners 2 (G) and 3 (L)
                                      on H's lower block pattern: per row the blocks of
                                      columns <= row, ascending (empty unless
                                      preconditioner >= 2)                                     */
    MFEM_BUF_COUNT = 27
} mfem_buffer;

/* Rigid shapes that contact takes into account (Newton's GeoType PLANE and
 * CAPSULE; the reference ignores the other types, src/mfem/refinement/
 * contact.py:134-141).  A plane passes through its pose's origin with normal
 * local +Z; a capsule is centred on its origin along local +Z with
 * scale = (radius, half height, -) (src/mfem/ipc/distance.py:5-57). */
typedef enum mfem_shape_type {
    MFEM_SHAPE_PLANE = 0,
    MFEM_SHAPE_CAPSULE = 1
} mfem_shape_type;

/* Contact settings: RefinementSolver's contact kwargs
 * (src/mfem/refinement/solver.py:241-265). */
typedef struct mfem_contact_config {
    float d0;               /* contact_d0, default 1e-2: quadratic barrier below   */
    float d1;               /* contact_d1, default 1e-1: barrier support           */
    float stiffness;        /* contact_stiffness, default 1e7                      */
    float friction_eps_v;   /* friction_eps_v, default 1e-3 (static below eps_v dt) */
    int32_t tri_contact;    /* 1 (default): per-tri barrier against capsules       */
    int32_t reserved[3];
} mfem_contact_config;

/* Per Newton iteration outcome of the global solve. */
typedef struct mfem_solve_stats {
    int32_t iterations;     /* PCG iterations taken                       */
    int32_t status;         /* MFEM_OK, MFEM_MAXITER, MFEM_STAGNATION, ... */
    float rel_residual;     /* ||r|| / ||b|| of the recurrence residual    */
    float reserved;
} mfem_solve_stats;

/* Precision of the global solve.  FP32 is the reference's float32 PCG;
 * BF16 / FP16 store the BSR blocks in 16 bits (each block row scaled by its
 * largest |entry|) for an inner PCG with fp32 vectors, inside an iterative
 * refinement whose residual g - H dx is formed in fp64 from the fp32 H. */
typedef enum mfem_precision {
    MFEM_PRECISION_FP32 = 0,
    MFEM_PRECISION_BF16 = 1,
    MFEM_PRECISION_FP16 = 2,
    /* the fp32 blocks in the inner PCG, inside the same fp64 refinement: the
     * plain fp32 PCG brought to an fp64-checked residual */
    MFEM_PRECISION_FP32_REFINED = 3
} mfem_precision;

typedef struct mfem_solver_config {
    int32_t precision;              /* mfem_precision                                   */
    float inner_tolerance;          /* inner PCG: ||r|| <= tol ||rhs||, default 1e-3     */
    int32_t outer_max_iterations;   /* corrections per solve, default 10                */
    int32_t factor_refresh;         /* preconditioners 2 and 3 (FP32 solve): recompute the
                                       factor at the Newton iterations it of a step with
                                       it % factor_refresh == 0 and reuse it in between
                                       (an older factor still gives an SPD M); 0 or 1:
                                       every assembly.  Staged mfem_assemble calls always
                                       recompute it                                      */
    double outer_tolerance;         /* fp64 ||g - H dx|| <= tol ||g||, default 1e-8     */
    int32_t reserved[4];
} mfem_solver_config;

/* Per Newton iteration outcome of a mixed-precision solve. */
typedef struct mfem_mixed_solve_stats {
    int32_t outer_iterations;       /* corrections applied                              */
    int32_t inner_iterations;       /* PCG iterations over all corrections              */
    int32_t status;                 /* MFEM_OK, MFEM_MAXITER (outer cap), ...           */
    int32_t fp32_inner;             /* 1: the refinement diverged (residual above 4x its
                                       best) and the solve restarted from the warm
                                       start with the fp32 H in the inner PCG          */
    double rel_residual;            /* fp64 ||g - H dx|| / ||g|| of the returned dx     */
} mfem_mixed_solve_stats;

/* Per Newton iteration outcome of the line search. */
typedef struct mfem_line_search_stats {
    int32_t evaluations;    /* trial evaluations: the reference's iteration counter     */
    int32_t accepted;       /* 1 if x, s moved to the last trial, 0 if left unchanged   */
    float alpha;            /* step of the last trial                                   */
    int32_t status;         /* MFEM_OK, or MFEM_TIMEOUT if a grid wait gave up          */
    double f0;              /* merit function at (x, s)                                 */
    double f1;              /* merit function at the last trial                         */
    double t;               /* -c (gradient . direction)                                */
} mfem_line_search_stats;

/* ---- configuration / diagnostics ------------------------------------ */

/* Fills the reference's defaults: iterations 8, ARAP, cg_max_iterations 1000,
 * cg_tolerance 1e-6, attachment_stiffness 10, singular threshold 1e-20,
 * block-Jacobi on, line search on with 20 iterations, alpha0 1, tau 0.5,
 * c 0.01, threshold 1e-8 (src/mfem/refinement/solver.py:90-128, 185). */
void mfem_config_default(mfem_config *cfg);

const char *mfem_status_string(int status);

/* Total kernels this library has launched in this process (graph replays
 * count every kernel node). */
uint64_t mfem_kernel_launch_count(void);

/* ---- host-side symbolic analysis (no GPU needed) --------------------- */

/* Exact vertex-adjacency sparsity of the global Hessian, diagonal included,
 * columns ascending.  Replaces the padded bsr_set_from_triplets / bsr_mm
 * topology of src/mfem/refinement/solver.py:201-203, 685-724.
 * Call with row_ptr/col_idx NULL to get *nnzb first. */
int mfem_bsr_sparsity(int32_t n_particles, int32_t n_tets, const int32_t *h_tet_indices,
                      int32_t *h_row_ptr, int32_t *h_col_idx, int64_t *nnzb);

/* Element -> BSR-slot scatter map [T][16] for the sparsity above (the
 * triplets of src/mfem/refinement/kernels.py:105-128 resolved to slots). */
int mfem_tet_slot_map(int32_t n_particles, int32_t n_tets, const int32_t *h_tet_indices,
                      const int32_t *h_row_ptr, const int32_t *h_col_idx, int32_t *h_slots);

/* ---- plan ----------------------------------------------------------- */

/* Builds a plan for one body on device `device`: uploads the model, runs the
 * symbolic analysis, allocates the workspace and sets s = S(F_rest),
 * lambda = 0.  Replaces RefinementSolver.__init__ with refinement and
 * shell off, contact off until mfem_plan_set_contact (src/mfem/refinement/solver.py:41-304;
 * additional_state.py:139-202; the mass/attachment setup of
 * solver.py:320-393).  Host arrays:
 *   tet_indices [T][4], tet_poses [T][3][3] (DmInv, edges as columns),
 *   tet_materials [T][3] (mu, lambda, damping), particle_q_rest [n][3]
 *   (initial stretch and attachment targets), particle_mass [n],
 *   particle_inv_mass [n] (0 = attached), gravity [3].
 * This call synchronises the device. */
int mfem_plan_create(const mfem_config *cfg, int32_t n_particles, int32_t n_tets,
                     const int32_t *h_tet_indices, const float *h_tet_poses,
                     const float *h_tet_materials, const float *h_particle_q_rest,
                     const float *h_particle_mass, const float *h_particle_inv_mass,
                     const float *h_gravity, int32_t device, mfem_plan **out);

void mfem_plan_destroy(mfem_plan *plan);

/* Message of the last error raised on this plan ("" if none). */
const char *mfem_plan_last_error(const mfem_plan *plan);

int mfem_plan_sizes(const mfem_plan *plan, int32_t *n_particles, int32_t *n_tets, int64_t *nnzb);

/* The persistent PCG the plan chose: variant (1 standard, 2 single-reduction,
 * 3 gather, 4 standard with a factor preconditioner; 0 when the global solve
 * runs the global-memory PCG of mfem_plan_set_bodies as a one-body batch: a
 * mesh too large for the shared-memory slices, pcg_variant 5, or bodies
 * set), CTAs, whether each CTA keeps its slice of H in shared
 * memory, and the dynamic shared memory per CTA.  Diagnostics; no reference
 * counterpart. */
int mfem_plan_pcg_layout(const mfem_plan *plan, int32_t *variant, int32_t *ctas, int32_t *cache_matrix,
                         int64_t *smem_bytes);

/* Bytes of an exposed buffer. */
int mfem_plan_buffer_bytes(const mfem_plan *plan, int32_t which, size_t *bytes);

/* cudaMemcpyAsync between an exposed buffer and caller memory (host or
 * device, any kind).  `bytes` must equal mfem_plan_buffer_bytes. */
int mfem_plan_copy_out(const mfem_plan *plan, int32_t which, void *dst, size_t bytes, mfem_stream stream);
int mfem_plan_copy_in(mfem_plan *plan, int32_t which, const void *src, size_t bytes, mfem_stream stream);

/* ---- contact against rigid shapes ------------------------------------ */

void mfem_contact_config_default(mfem_contact_config *cfg);

/* Turns contact on (n_shapes > 0) or off (n_shapes == 0): the per-vertex log
 * barrier against the shapes and the lagged friction, and, with
 * cfg->tri_contact, the per-tri barrier of the surface tris against the
 * capsules (Contact of src/mfem/refinement/contact.py:778-1106, added into
 * H and g at solver.py:734-779 and into the line search's merit at
 * :856-862, 909).  Host arrays:
 *   shape_type [S] (mfem_shape_type; others are ignored),
 *   shape_pose [S][7] (px, py, pz, qx, qy, qz, qw) in the frame of its body,
 *   shape_scale [S][3], shape_body [S] (< 0: static, else < n_bodies),
 *   friction_mu [S] (Coulomb coefficient per shape),
 *   tris [m][3] surface tris (each pair of their vertices must share a tet).
 * Body poses start at the identity; set them with mfem_set_body_poses
 * before each step.  S <= 64.  Synchronises the device and drops the
 * plan's captured graphs. */
int mfem_plan_set_contact(mfem_plan *plan, const mfem_contact_config *cfg, int32_t n_shapes,
                          const int32_t *h_shape_type, const float *h_shape_pose,
                          const float *h_shape_scale, const int32_t *h_shape_body,
                          const float *h_friction_mu, int32_t n_bodies, int32_t n_tris,
                          const int32_t *h_tris);

/* Copies the body poses [n_bodies][7] the next steps read (the
 * reference's state_out.body_q) into the plan, asynchronously on `stream`
 * (host or device memory).  n_bodies must match mfem_plan_set_contact. */
int mfem_set_body_poses(mfem_plan *plan, const float *body_q, int32_t n_bodies, mfem_stream stream);

/* ---- precision of the global solve ----------------------------------- */

void mfem_solver_config_default(mfem_solver_config *cfg);

/* Selects the global solve: the reference's float32 PCG (precision FP32,
 * the default) or the mixed-precision iterative refinement (BF16 / FP16
 * blocks, fp32 inner PCG to inner_tolerance with the plan's preconditioner,
 * fp64 residual; stops at outer_tolerance or after outer_max_iterations
 * corrections, starting from the reference's warm start).  Where the plan
 * has a persistent factor PCG layout (pcg_variant 4, or the block-Jacobi one
 * a one-mesh plan keeps when it fits) the inner solves run there, on an fp32
 * copy of the 16-bit blocks, for the residual scaled to unit norm; else in
 * the global-memory inner PCG.  It has no reference counterpart: it is the
 * mixed-precision variant of src/mfem/refinement/solver.py:581-609.
 * Synchronises the device and drops the plan's captured graphs. */
int mfem_plan_set_solver(mfem_plan *plan, const mfem_solver_config *cfg);

/* Outcomes of the mixed-precision solves of the last step (synchronises the
 * stream; *count = 0 with the FP32 solve).  mfem_step_stats reports the same
 * solves with iterations = inner iterations and rel_residual = the fp64
 * residual. */
int mfem_step_mixed_stats(mfem_plan *plan, mfem_mixed_solve_stats *h_stats, int32_t max_entries,
                          int32_t *count, mfem_stream stream);

/* ---- the learned factor preconditioner (preconditioner = 3) -------------- */

/* Parameters of the factor net, packed as float32 in this order ([out][in]
 * row-major matrices): W_in [64][16], b_in [64]; for l = 0..2: W_l [64][128],
 * b_l [64]; W_d [6][64], b_d [6]; W_p [64][64], b_p [64]; W_q [64][64];
 * W_r [64][9]; W_o [9][64], b_o [9].  Matrices are rounded to BF16 here. */
#define MFEM_FACTOR_NET_PARAMS 35663

/* Loads the net's parameters and the static per-vertex inputs
 * h_vertex_static [n][4] (incident-tet mean log10 E minus 5; rest position
 * minus the body's centroid).  After every assembly the net writes L (lower
 * block-triangular on H's lower block pattern, positive-diagonal diagonal
 * blocks) into MFEM_BUF_PRECOND_FACTOR and the PCG applies M = L L^T; a
 * body whose factor-preconditioned solve breaks down (non-finite values or
 * p.Ap <= 0) is solved again with block-Jacobi.  Net: width 64, three
 * message-passing layers over H's block graph with weights ||(S H S)_ij||_F,
 * S = diag(tr(H_ii)/3)^-1/2; L = S L~ with L~ the net's output.  Needs a plan
 * created with preconditioner = 3.  No reference counterpart (the
 * reference's PCG is block-Jacobi).  Synchronises the device and drops
 * captured graphs. */
int mfem_plan_set_factor_net(mfem_plan *plan, const float *h_params, int64_t n_params,
                             const float *h_vertex_static);

/* ---- training the factor net (no plan) ---------------------------------- */

/* C = op(A) op(B), or C += op(A) op(B) with accumulate != 0, on the tensor
 * cores: device float32 operands rounded to BF16 as they are staged, FP32
 * accumulation.  op(A) is A (stored [M][K], row stride lda) or, with a_trans,
 * A^T (A stored [K][M]); op(B) is B (stored [K][N]) or, with b_trans, B^T
 * (B stored [N][K]); C is [M][N] with row stride ldc.  The three products of
 * a linear layer y = x W^T are forward (A = x, B = W, b_trans), the input
 * gradient (A = dy, B = W) and the weight gradient (A = dy, a_trans, B = x).
 * A long K with a small C is split over CTAs into partial tiles in the
 * optional device workspace (workspace_floats floats; NULL: no split), added
 * in a fixed order.  Asynchronous on `stream`; errors through
 * mfem_train_last_error().  No reference counterpart: the factor net and its
 * training are this library's (mfem_plan_set_factor_net). */
int mfem_train_gemm(int32_t M, int32_t N, int32_t K, const float *d_A, int32_t lda, int32_t a_trans,
                    const float *d_B, int32_t ldb, int32_t b_trans, float *d_C, int32_t ldc, int32_t accumulate,
                    float *d_workspace, int64_t workspace_floats, mfem_stream stream);

/* One Adam step (Kingma & Ba 2015) over n float32 parameters on the device:
 * m = beta1 m + (1 - beta1) g, v = beta2 v + (1 - beta2) g^2,
 * p -= lr m^ / (sqrt(v^) + eps) with the bias corrections of step >= 1.
 * No reference counterpart. */
int mfem_train_adam(float *d_params, const float *d_grads, float *d_m, float *d_v, int64_t n, float lr, float beta1,
                    float beta2, float eps, int32_t step, mfem_stream stream);

/* Message of the last failed mfem_train_* call on this host thread. */
const char *mfem_train_last_error(void);

/* ---- independent bodies in one plan ------------------------------------ */

/* Declares the plan's mesh to be n_bodies independent bodies: the vertices
 * of body b are [vertex_offsets[b], vertex_offsets[b+1]), its tets
 * [tet_offsets[b], tet_offsets[b+1]), and no tet joins two bodies.  Each body
 * has its own energy (mfem_energy) and gravity [3].  The step then solves one
 * block-Jacobi PCG per body (own scalars and stopping test, the reference's
 * solve applied to each body) in a single persistent launch; the other
 * kernels run on the union.  Needs a plan created with line_search = 0 and
 * the FP32 solve.  No reference counterpart (the reference steps one body
 * per solver).  Synchronises the device and drops captured graphs. */
int mfem_plan_set_bodies(mfem_plan *plan, int32_t n_bodies, const int32_t *h_vertex_offsets,
                         const int32_t *h_tet_offsets, const int32_t *h_body_energy,
                         const float *h_body_gravity);

/* CTAs and threads per CTA of the batched PCG's current schedule. */
int mfem_plan_batch_layout(const mfem_plan *plan, int32_t *ctas, int32_t *threads);

/* Solves the system at d_q (at rest) once to learn each body's PCG
 * iterations, then times the batched PCG for each distinct candidate
 * schedule (threads per CTA 128/256/512 x three costs of a group barrier,
 * and for one body x five caps on its group's CTAs, from unbounded to a
 * quarter of the SMs; bodies
 * get CTA groups while that shortens the longest modelled body time,
 * iterations x blocks per CTA) and keeps the fastest; *h_best_ms receives its
 * solve time.  Also serves a one-body plan (a mesh too large for the
 * persistent PCG, or a factor preconditioner).  Synchronises the stream. */
int mfem_plan_autotune_batch(mfem_plan *plan, const float *d_q, float dt, double *h_best_ms, mfem_stream stream);

/* Per-body PCG outcomes of the last step, [iteration][body] (synchronises
 * the stream; *count = 0 without bodies). */
int mfem_step_body_stats(mfem_plan *plan, mfem_solve_stats *h_stats, int32_t max_entries, int32_t *count,
                         mfem_stream stream);

/* ---- the step and its stages ---------------------------------------- */

/* One implicit-Euler step: RefinementSolver.step
 * (src/mfem/refinement/solver.py:429-579) with refinement off; the update is
 * the plain x += dx, s += ds (:555-557) or, with the config's line_search,
 * the backtracking line search (:539-553); contact terms as set by
 * mfem_plan_set_contact.  d_q_out/d_qd_out receive the new
 * positions and velocities; d_q_in/d_qd_in are only read, and may alias the
 * outputs.  s and lambda persist in the plan.  Asynchronous; allocates
 * nothing. */
int mfem_step(mfem_plan *plan, const float *d_q_in, const float *d_qd_in,
              float *d_q_out, float *d_qd_out, float dt, mfem_stream stream);

/* Outcome of the global solves of the last step (synchronises the stream).
 * Writes min(max_entries, iterations) entries; *count = entries written.
 * With several bodies (mfem_plan_set_bodies) each entry summarises the
 * bodies: the most iterations, the largest residual and the first failing
 * body's status; mfem_step_body_stats gives them one by one. */
int mfem_step_stats(mfem_plan *plan, mfem_solve_stats *h_stats, int32_t max_entries,
                    int32_t *count, mfem_stream stream);

/* Outcome of the line searches of the last step, one entry per Newton
 * iteration (synchronises the stream; entries are zero with the line search
 * off).  The reference keeps these in device scalars it does not return
 * (src/mfem/line_search.py:89-94). */
int mfem_step_line_search_stats(mfem_plan *plan, mfem_line_search_stats *h_stats, int32_t max_entries,
                                int32_t *count, mfem_stream stream);

/* Predictor x~ = x + v dt + g dt^2/2 into the plan
 * (integrate_particles, src/mfem/refinement/kernels.py:77-91), and with
 * contact the lagged friction snapshot at x = d_q (Contact.begin_step,
 * src/mfem/refinement/contact.py:937-967). */
int mfem_predict(mfem_plan *plan, const float *d_q, const float *d_qd, float dt, mfem_stream stream);

/* Element stage at (x, s): c, G, g_s, H_s (psd-fixed for Neo-Hookean),
 * H_lambda, g_lambda and the element Hessian/rhs; replaces _update_system
 * plus the per-tet half of _assemble_system
 * (src/mfem/refinement/solver.py:633-679, 695-706, 930-980). */
int mfem_update_system(mfem_plan *plan, const float *d_x, mfem_stream stream);

/* Assembly: H = sum_e G^T H_l G + (M+Q)/dt^2, g = sum_e G^T H_l g_l - g_x,
 * the block-Jacobi inverse and the warm start dx = x~ - x
 * (src/mfem/refinement/solver.py:682-743, 530-531, 591-602); with contact,
 * first the contact terms at x (Contact.evaluate, solver.py:637), whose
 * blocks and gradients go into H and g (:734-779). */
int mfem_assemble(mfem_plan *plan, const float *d_x, float dt, mfem_stream stream);

/* Block-Jacobi PCG on H dx = g (src/mfem/refinement/solver.py:581-609 and
 * warp.optim.linear.cg).  Result in MFEM_BUF_DX; outcome recorded as entry
 * `slot` of the stats that mfem_step_stats reads. */
int mfem_global_solve(mfem_plan *plan, int32_t slot, mfem_stream stream);

/* Local solve and update: lambda = -H_l (g_l - G dx), ds = -H_s^-1 (SYM
 * lambda + g_s) (src/mfem/refinement/kernels.py:252-283), then s += ds,
 * x += dx (solver.py:555-557), or with the line search on, the backtracking
 * search along (dx, ds) (solver.py:539-553, 871-928), recorded as the line
 * search entry of the last mfem_global_solve slot.  Needs the g_x of the
 * assembly at the same x (mfem_assemble). */
int mfem_local_solve(mfem_plan *plan, float *d_x, mfem_stream stream);

/* ||g - H dx|| / ||g|| accumulated in float64 for the current H, g, dx
 * (synchronises the stream).  The reference has no counterpart: it is the
 * true-residual check of the float32 recurrence. */
int mfem_true_residual(mfem_plan *plan, double *h_rel_residual, mfem_stream stream);

/* Turns on (on != 0) or off the element stage's diagnostic outputs H_s^-1
 * (MFEM_BUF_HESS_S_INV) and g_lambda (MFEM_BUF_G_LAMBDA): the reference's
 * intermediates (src/mfem/refinement/kernels.py:189-217), which the step
 * does not read -- its local solve and rhs use the cancellation-free form
 * lambda = -(H_l u + INV_SYM g_s), ds = INV_SYM u, u = c - G dx.  Off by
 * default (those buffers then keep stale contents).  Synchronises the device
 * and drops captured graphs when the setting changes. */
int mfem_plan_set_diagnostics(mfem_plan *plan, int32_t on);

/* Turns on (on != 0) or off the fp64 check of every global solve inside
 * mfem_step: after each Newton iteration's solve the step also forms
 * ||g - H dx|| / ||g|| in float64 for the float32 dx the local solve reads
 * (mfem_true_residual's sum, one entry per Newton iteration).  It reads
 * only, so the trajectory is unchanged.  The reference has no counterpart:
 * it checks the float32 CG's recurrence residual only.  Synchronises the
 * device and drops captured graphs when the setting changes. */
int mfem_plan_set_residual_check(mfem_plan *plan, int32_t on);

/* Failure injection on the host, for tests of the timeout path: sets the
 * plan's sticky device error flag, as a bounded wait that gave up does.  The
 * step's persistent kernels then leave at their first check (no wait, no
 * fault), the step's stats calls return MFEM_TIMEOUT and re-arm every grid
 * barrier of the plan, and the step after that runs normally.  Synchronises
 * the device; launches nothing. */
int mfem_plan_inject_timeout(mfem_plan *plan);

/* The check's results for the last step, one per Newton iteration
 * (synchronises the stream; MFEM_BAD_ARG while the check is off). */
int mfem_step_true_residuals(mfem_plan *plan, double *h_rel_residual, int32_t max_entries, int32_t *count,
                             mfem_stream stream);

/* ---- adaptive refinement ------------------------------------------------- */

typedef enum mfem_refine_scoring {
    MFEM_REFINE_LEGACY = 0,     /* refinement.py:74-121: sum over an edge's tets of
                                   (E_t w_t + min(vs_a, vs_b) w_v) L; an edge whose
                                   midpoint is inside a shape scores penetrating_edge_score */
    MFEM_REFINE_GEOMETRIC = 1   /* refinement.py:157-316: max over an edge's tets and
                                   surface tris of (L/h)(L/L_max)(w_e s_elastic + w_c s_contact) */
} mfem_refine_scoring;

/* refine()'s settings (src/mfem/refinement/refinement.py:914-940) with
 * RefinementSolver's refine_* kwargs (src/mfem/refinement/solver.py:56-87). */
typedef struct mfem_refine_config {
    int32_t scoring;                /* mfem_refine_scoring                                     */
    float threshold;                /* an edge is a candidate when its score exceeds it:
                                       min_refine_score (10.1) for legacy scores,
                                       refine_geometric_threshold (1.0) for geometric ones      */
    float tet_score_weight;         /* legacy: refine_tet_score_weight, default 0             */
    float vertex_score_weight;      /* legacy: refine_vertex_score_weight, default 0.1        */
    float penetrating_edge_score;   /* legacy: default 1e6                                     */
    float min_edge_length;          /* geometric h: edges shorter than 2h are never split      */
    float contact_d1;               /* geometric: the contact barrier range                    */
    float elastic_weight;           /* geometric: refine_elastic_weight, default 1             */
    float vertex_contact_weight;    /* geometric: refine_contact_weight, default 1             */
    float tri_contact_weight;       /* geometric: refine_tri_contact_weight, default 1         */
    float split_position;           /* new vertex at q_lo + (q_hi - q_lo) t, default 0.5       */
    float density;                  /* lumped masses of a refined mesh: density * volume / 4   */
    int32_t conflict_iterations;    /* selection sweeps, default 5                             */
    int32_t refine_every;           /* with a pass counter: split only on passes whose counter
                                       is a multiple (refine_every_n_steps, default 10)       */
    int32_t reserved[4];
} mfem_refine_config;

/* Optional per-element inputs of the scores, device arrays over the plan's
 * current mesh (refine()'s tet_scores / vertex_scores / particle_distance /
 * particle_shape_id / tri_distance / tri_bary).  NULL: the library computes
 * them at the positions given to mfem_refine, from the plan's s (elastic
 * energy per tet) and its contact shapes (barrier energy per vertex plus the
 * tris' weighted barrier energies; nearest-shape distance and shape; tri
 * distance and closest-point weights). */
typedef struct mfem_refine_inputs {
    const float *tet_scores;          /* [T]                                           */
    const float *vertex_scores;       /* [n] legacy                                    */
    const float *particle_distance;   /* [n] geometric                                 */
    const int32_t *particle_shape_id; /* [n] geometric, index into the plan's shapes   */
    const float *tri_distance;        /* [m] geometric                                 */
    const float *tri_bary;            /* [m][3] geometric                              */
} mfem_refine_inputs;

/* The refined mesh: caller-owned device arrays of capacity max_* rows that
 * receive the mesh after the pass (a copy of the plan's mesh when the pass
 * splits nothing).  tris receives the plan's contact tris and may be NULL
 * when the plan has none.  counts (device, 8 int32) receives: particles,
 * tets, tris of the result, edges split, 1 if the pass was dropped for
 * capacity, 1 if the pass was a refining one, 0, 0. */
typedef struct mfem_refine_mesh {
    int32_t max_particles, max_tets, max_tris;
    int32_t reserved;
    int32_t *tet_indices;     /* [max_tets][4]                                          */
    float *tet_poses;         /* [max_tets][3][3] DmInv                                 */
    float *tet_materials;     /* [max_tets][3]                                          */
    float *tet_stretch;       /* [max_tets][6] s, the parent's for both children        */
    float *tet_lambda;        /* [max_tets][6] lambda, likewise                         */
    float *rest_q;            /* [max_particles][3]                                     */
    float *particle_mass;     /* [max_particles]                                        */
    float *particle_inv_mass; /* [max_particles]                                        */
    int32_t *tri_indices;     /* [max_tris][3] or NULL                                  */
    int32_t *counts;          /* [8]                                                    */
} mfem_refine_mesh;

void mfem_refine_config_default(mfem_refine_config *cfg);

/* One refine() pass (src/mfem/refinement/refinement.py:914-1322) over the
 * plan's mesh at positions d_q, velocities d_qd ([max_particles][3]; rows
 * [0, n) are read, and the new vertices' rows [n, n + new) are written there,
 * at split_position along their edges).  Edges are scored, each tet picks its
 * best edge above the threshold, conflicts are resolved over
 * conflict_iterations sweeps so that no tet holds two, and every tet and
 * contact tri around a selected edge splits in two.  The selection is
 * deterministic (ranked by score, ties by the smaller vertex pair) where the
 * reference's depends on thread order; new vertices are numbered in
 * ascending (lower vertex, higher vertex) order; a splitting pass rebuilds
 * the lumped masses from density (vertices with inv_mass 0 stay kinematic).
 * A pass that would exceed a capacity is dropped whole, as the reference's.
 * With d_pass_counter (device int32, may be NULL) only passes whose counter
 * is a multiple of refine_every split, and the counter advances by one
 * (refinement.py:560-575).  The plan itself is unchanged: create a plan
 * from the refined mesh to step it.  The first call on a plan builds its edge
 * lists (synchronises and allocates); later calls are asynchronous on
 * `stream` and allocate only when max_tets grows.  Plans with bodies
 * (mfem_plan_set_bodies) are not refined. */
int mfem_refine(mfem_plan *plan, const mfem_refine_config *cfg, const mfem_refine_inputs *inputs, float *d_q,
                float *d_qd, int32_t *d_pass_counter, const mfem_refine_mesh *out, mfem_stream stream);

/* ---- allocation-free solve ---------------------------------------------- */

/* Block-Jacobi PCG on a caller-provided 3x3-block BSR system that allocates
 * nothing, for callers that cannot call cudaMalloc when they solve (a
 * framework's caching allocator owns the heap, or the host forbids
 * allocation after start-up).  It has no counterpart in the reference.
 * Device arrays, all caller-owned: row_ptr [n+1], col_idx [nnzb], values
 * [nnzb][3][3], precond [n][3][3] block inverse (NULL: unpreconditioned),
 * b [n][3]; x [n][3] holds the warm start and receives the solution;
 * the caller keeps the BSR well formed (row_ptr[0] = 0, non-decreasing,
 * row_ptr[n] = nnzb; 0 <= col_idx < n), which the device does not check;
 * stats (device pointer, may be NULL) receives the outcome.  Stops when
 * ||r|| <= tol ||b|| or after maxiter iterations.
 * Its scratch is a fixed array of about 2 MB inside the library (every GPU
 * that loads the library holds it until exit) serving at most 32768 block
 * rows; larger systems return MFEM_BAD_ARG.  All calls share that array:
 * calls whose kernels overlap on the GPU race and must be serialised.  Each
 * call looks up the array's address with the caller's device current; the
 * first lookup on a device loads the module, so make the first call before
 * any stream capture.  Asynchronous on `stream`;
 * errors are reported by mfem_plan_last_error(NULL). */
int mfem_pcg_solve_noalloc(int32_t n, const int32_t *d_row_ptr, const int32_t *d_col_idx,
                           const float *d_values, const float *d_precond, const float *d_b, float *d_x,
                           float tol, int32_t maxiter, mfem_solve_stats *d_stats, mfem_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* MFEM_GB300_H */
