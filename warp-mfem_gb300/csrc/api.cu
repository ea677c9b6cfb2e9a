// C ABI of libmfem_gb300: plan lifecycle, the step, its stages and the
// buffer/diagnostic accessors declared in include/mfem_gb300.h.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "internal.h"

namespace mfem {

static std::atomic<uint64_t> g_launches{0};
static thread_local bool t_capturing = false;
static thread_local std::string t_create_error;

void count_launches(uint64_t k) {
    if (!t_capturing) g_launches += k;
}

int set_create_error(int code, const std::string &msg) {
    t_create_error = msg;
    return code;
}

}  // namespace mfem

using namespace mfem;

struct mfem_plan {
    mfem_config cfg{};
    int device = 0;
    int n = 0;
    int T = 0;
    int64_t nnzb = 0;
    int pcg_ctas = 1;
    int max_stats = 1;
    float gravity[3] = {0.0f, 0.0f, 0.0f};
    std::string last_error;
    std::vector<void *> allocs;
    TetViews tv{};
    VertexViews vv{};
    BsrViews bv{};
    PcgWork pw{};
    PcgLayout pl{};
    // block-Jacobi plans: the persistent factor PCG's layout (block-Jacobi
    // only) for the inner solves of the mixed refinement, when it fits
    PcgLayout ir_pl{};
    LineSearchWork ls{};
    float stage_dt = 0.0f;     // dt of the last mfem_assemble (the line search's 1/dt^2)
    int stage_slot = 0;        // slot of the last mfem_global_solve
    // contact against rigid shapes (mfem_plan_set_contact); off until set
    ContactViews cv{};
    int n_bodies = 0;
    int n_tris = 0;
    std::vector<void *> contact_allocs;
    // host copies kept to rebuild the assembly's contribution lists
    std::vector<int32_t> h_tets, h_row_ptr, h_col_idx, h_tet_slots;
    const int32_t *base_chunk_ptr = nullptr, *base_code = nullptr, *base_slot = nullptr;
    int base_chunks = 0;
    // mixed-precision global solve (mfem_plan_set_solver); mode 0 = the
    // reference's float32 PCG
    IrWork ir{};
    std::vector<void *> ir_allocs;
    // independent bodies (mfem_plan_set_bodies): per-body PCGs in one launch
    BatchViews bw{};
    std::vector<void *> batch_allocs;
    int factor_refresh = 1;      // recompute a factor preconditioner every this many Newton iterations
    int bw_max_group = INT_MAX;  // the schedule's group cap and barrier cost
    double bw_c0 = 2048.0;
    // the learned factor net (preconditioner 3)
    FactorNetViews fv{};
    std::vector<void *> net_allocs;
    std::vector<void *> layout_allocs;  // the current schedule's task arrays and partials
    std::vector<int32_t> h_body_row, h_body_nnzb, h_body_its;
    bool global_memory_pcg = false;  // the mesh is solved as a one-body batch
    int32_t *tet_slots = nullptr;
    float *rest_q = nullptr;    // [n][3] rest positions
    float *inv_mass = nullptr;  // [n] particle_inv_mass as given
    float *mass = nullptr;      // [n] particle_mass as given
    std::vector<int32_t> h_tris;  // the contact tris, host copy
    // adaptive refinement (mfem_refine): edge lists built on the first call
    RefineViews rv{};
    bool refine_ready = false;
    int64_t refine_tmass_cap = 0;
    int64_t refine_scan_cap = 0;
    std::vector<void *> refine_allocs;
    double *resid = nullptr;
    // per-solve fp64 check of the step's global solves (mfem_plan_set_residual_check)
    double *check_resid = nullptr;  // [max_stats][2]: ||g - H dx||^2, ||g||^2
    bool check_on = false;
    bool diagnostics = false;  // the element stage also writes H_s^-1 and g_lambda
    cudaStream_t capture_stream = nullptr;
    // captured steps, keyed by (q_in, qd_in, q_out, qd_out, dt); a simulation
    // loop that swaps two states alternates between two entries
    static constexpr int kGraphSlots = 4;
    struct GraphEntry {
        cudaGraphExec_t exec = nullptr;
        const void *key[4] = {nullptr, nullptr, nullptr, nullptr};
        float dt = 0.0f;
        uint64_t kernels = 0;
        uint64_t last_use = 0;
    } graphs[kGraphSlots];
    uint64_t graph_clock = 0;
};

namespace {

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) {
            int cur = -1;
            if (cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
        }
    }
};

int fail(mfem_plan *p, int code, const std::string &msg) {
    if (p) p->last_error = msg;
    else t_create_error = msg;
    return code;
}

int cuda_fail(mfem_plan *p, cudaError_t err, const char *what) {
    return fail(p, MFEM_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(err));
}

// After a bounded wait gave up (the sticky error flag is set), with no kernel
// of the plan in flight: every grid barrier counter of the plan back to 0 (a
// barrier that timed out leaves partial arrivals, which would release the
// next launch's barriers early) and the flag cleared.
cudaError_t rearm_barriers(mfem_plan *p) {
    cudaError_t e = cudaMemset(p->pw.counter, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(p->ls.counter, 0, sizeof(unsigned long long));
    if (e == cudaSuccess && p->ir.counter) e = cudaMemset(p->ir.counter, 0, sizeof(unsigned long long));
    if (e == cudaSuccess && p->bw.n_bodies > 0 && p->bw.counter)
        e = cudaMemset(p->bw.counter, 0, (size_t)p->bw.n_bodies * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(p->pw.error, 0, sizeof(int));
    return e;
}

template <class T>
cudaError_t dev_alloc(mfem_plan *p, T **ptr, size_t count) {
    void *raw = nullptr;
    cudaError_t err = cudaMalloc(&raw, count == 0 ? 16 : count * sizeof(T));
    if (err != cudaSuccess) return err;
    p->allocs.push_back(raw);
    *ptr = static_cast<T *>(raw);
    return cudaSuccess;
}

template <class T>
cudaError_t upload(T *dst, const T *src, size_t count) {
    if (count == 0) return cudaSuccess;
    return cudaMemcpy(dst, src, count * sizeof(T), cudaMemcpyHostToDevice);
}

struct BufferRef {
    void *ptr;
    size_t bytes;
};

bool buffer_ref(const mfem_plan *p, int which, BufferRef &ref) {
    const size_t T = p->T, n = p->n, nnzb = (size_t)p->nnzb;
    switch (which) {
        case MFEM_BUF_TET_STRETCH: ref = {p->tv.stretch, T * 6 * 4}; return true;
        case MFEM_BUF_TET_LAMBDA: ref = {p->tv.lambda, T * 6 * 4}; return true;
        case MFEM_BUF_CONSTRAINT: ref = {p->tv.c, T * 6 * 4}; return true;
        case MFEM_BUF_GRAD_CONSTRAINT: ref = {p->tv.G, T * 72 * 4}; return true;
        case MFEM_BUF_GRAD_S: ref = {p->tv.g_s, T * 6 * 4}; return true;
        case MFEM_BUF_H_LAMBDA: ref = {p->tv.H_l, T * 21 * 4}; return true;
        case MFEM_BUF_HESS_S_INV: ref = {p->tv.H_si, T * 21 * 4}; return true;
        case MFEM_BUF_G_LAMBDA: ref = {p->tv.g_l, T * 6 * 4}; return true;
        case MFEM_BUF_ELEMENT_HESSIAN: ref = {p->tv.Ke, T * kKeFloats * 4}; return true;
        case MFEM_BUF_ELEMENT_RHS: ref = {p->tv.fe, T * kFeFloats * 4}; return true;
        case MFEM_BUF_ROW_PTR: ref = {(void *)p->bv.row_ptr, (n + 1) * 4}; return true;
        case MFEM_BUF_COL_IDX: ref = {(void *)p->bv.col_idx, nnzb * 4}; return true;
        case MFEM_BUF_TET_SLOTS: ref = {p->tet_slots, T * 16 * 4}; return true;
        case MFEM_BUF_H_VALUES: ref = {p->bv.values, nnzb * 9 * 4}; return true;
        case MFEM_BUF_RHS: ref = {p->vv.rhs, n * 3 * 4}; return true;
        case MFEM_BUF_PRECOND: ref = {p->vv.Minv, n * 9 * 4}; return true;
        case MFEM_BUF_X_TILDE: ref = {p->vv.x_tilde, n * 3 * 4}; return true;
        case MFEM_BUF_DX: ref = {p->vv.dx, n * 3 * 4}; return true;
        case MFEM_BUF_STRETCH_DIRECTION: ref = {p->ls.ds, T * 6 * 4}; return true;
        case MFEM_BUF_CONTACT_BLOCK: ref = {p->cv.vblock, p->cv.on ? n * 9 * 4 : 0}; return true;
        case MFEM_BUF_CONTACT_GRADIENT: ref = {p->cv.gtot, p->cv.on ? n * 3 * 4 : 0}; return true;
        case MFEM_BUF_CONTACT_ENERGY: ref = {p->cv.venergy, p->cv.on ? n * 4 : 0}; return true;
        case MFEM_BUF_TRI_CONTACT: ref = {p->cv.tri, p->cv.on ? (size_t)p->n_tris * kTriData * 4 : 0}; return true;
        case MFEM_BUF_FRICTION_NORMAL: ref = {p->cv.normal_lagged, p->cv.on ? n * 3 * 4 : 0}; return true;
        case MFEM_BUF_FRICTION_FORCE: ref = {p->cv.force_lagged, p->cv.on ? n * 4 : 0}; return true;
        case MFEM_BUF_MIXED_DX: ref = {p->ir.dx_out, p->ir.mode ? n * 3 * 8 : 0}; return true;
        case MFEM_BUF_PRECOND_FACTOR: ref = {(void *)p->bw.Lval, (size_t)p->bw.nnzl * 9 * 4}; return true;
        default: return false;
    }
}

bool valid_config(const mfem_config *cfg, std::string &err) {
    if (cfg->iterations < 0 || cfg->iterations > 4096) err = "iterations must be in [0, 4096]";
    else if (cfg->energy != MFEM_ENERGY_ARAP && cfg->energy != MFEM_ENERGY_NEOHOOKEAN) err = "unknown energy";
    else if (cfg->cg_max_iterations < 0) err = "cg_max_iterations must be >= 0";
    else if (!(cfg->cg_tolerance >= 0.0f) || !std::isfinite(cfg->cg_tolerance)) err = "cg_tolerance must be finite and >= 0";
    else if (!std::isfinite(cfg->attachment_stiffness) || cfg->attachment_stiffness < 0.0f)
        err = "attachment_stiffness must be finite and >= 0";
    else if (!(cfg->preconditioner_singular_threshold >= 0.0f)) err = "preconditioner_singular_threshold must be >= 0";
    else if (cfg->preconditioner < 0 || cfg->preconditioner > 3)
        err = "preconditioner must be 0 (none), 1 (block-Jacobi), 2 (FSAI) or 3 (learned)";
    else if (cfg->pcg_variant < 0 || cfg->pcg_variant > 5) err = "pcg_variant must be in [0, 5]";
    else if (cfg->preconditioner >= 2 && cfg->pcg_variant != 0 && cfg->pcg_variant != 4 && cfg->pcg_variant != 5)
        err = "factor preconditioners take pcg_variant 0 (auto), 4 (persistent) or 5 (global memory)";
    else if (cfg->preconditioner < 2 && cfg->pcg_variant == 4)
        err = "pcg_variant 4 needs a factor preconditioner (2 or 3)";
    else if (cfg->pcg_ctas < 0) err = "pcg_ctas must be >= 0";
    else if (cfg->line_search != 0 && cfg->line_search != 1) err = "line_search must be 0 or 1";
    else if (cfg->line_search_max_iterations < 0 || cfg->line_search_max_iterations > (1 << 20))
        err = "line_search_max_iterations must be in [0, 2^20]";
    else if (!std::isfinite(cfg->line_search_alpha0) || !std::isfinite(cfg->line_search_tau) ||
             !std::isfinite(cfg->line_search_c) || !std::isfinite(cfg->line_search_threshold))
        err = "line search parameters must be finite";
    else return true;
    return false;
}

// A plan with the learned preconditioner needs its net before any assembly.
bool net_ready(const mfem_plan *p) { return p->cfg.preconditioner != 3 || p->fv.ready; }

// The whole step as a launch sequence on one stream.
// The reference's float32 PCG, or the mixed-precision iterative refinement.
cudaError_t global_solve(mfem_plan *p, int slot, cudaStream_t s) {
    if (p->ir.mode != 0)
        return launch_mixed_solve(p->bv, p->vv, p->ir, p->pw, p->bw,
                                  p->pl.variant == PcgLayout::kFactor ? p->pl : p->ir_pl,
                                  p->pl.variant == PcgLayout::kSingleReduction ? &p->pl : nullptr, p->pcg_ctas, slot,
                                  p->cfg.cg_max_iterations, p->cfg.preconditioner, s);
    if (p->pl.variant == PcgLayout::kFactor)
        return launch_pcg_factor(p->bv, p->vv, p->pw, p->bw, p->pl, p->pcg_ctas, slot, p->cfg.cg_tolerance,
                                 p->cfg.cg_max_iterations, p->cfg.preconditioner, s);
    if (p->bw.n_bodies > 0)
        return launch_batched_pcg(p->bv, p->vv, p->bw, p->pw.error, slot, p->cfg.cg_tolerance,
                                  p->cfg.cg_max_iterations, p->cfg.preconditioner, s);
    return launch_pcg(p->bv, p->vv, p->pw, p->pl, p->pcg_ctas, slot, p->cfg.cg_tolerance, p->cfg.cg_max_iterations,
                      p->cfg.preconditioner, s);
}

// Local solve then either the plain update x += dx, s += ds or the line
// search (solver.py:539-557).
cudaError_t local_update(mfem_plan *p, float *x, float dt, int slot, cudaStream_t s) {
    if (!p->cfg.line_search) return launch_local_solve(x, p->tv, p->vv, s);
    cudaError_t err = launch_local_solve_deferred(x, p->cfg.energy, dt, p->tv, p->vv, p->cv, p->ls, s);
    if (err == cudaSuccess)
        err = launch_line_search(x, p->cfg.energy, dt, p->tv, p->vv, p->cv, p->ls, p->pw.error, slot, s);
    return err;
}

// Contact terms at x, then the assembly (Contact.evaluate runs in
// _update_system, solver.py:637; it needs dt for the friction threshold).
cudaError_t contact_and_assemble(mfem_plan *p, const float *x, float dt, cudaStream_t s, bool factor_setup = true) {
    cudaError_t err = launch_contact(x, dt, p->cv, p->vv, s);
    if (err == cudaSuccess)
        err = launch_assemble(x, dt, p->cfg.preconditioner_singular_threshold, p->cfg.preconditioner, p->tv, p->vv,
                              p->bv, p->cv, s);
    if (factor_setup) {
        if (err == cudaSuccess && p->cfg.preconditioner == 2) err = launch_fsai_setup(p->bv, p->bw, s);
        if (err == cudaSuccess && p->cfg.preconditioner == 2) err = launch_factor_transpose(p->bw, s);
        if (err == cudaSuccess && p->cfg.preconditioner == 3) err = launch_factor_net(p->bv, p->bw, p->fv, s);
    }
    return err;
}

cudaError_t run_step(mfem_plan *p, const float *q_in, const float *qd_in, float *q_out, float *qd_out, float dt,
                     cudaStream_t s) {
    cudaError_t err = launch_predict(q_in, qd_in, q_out, p->gravity, dt, p->vv, s);
    // lagged friction anchor at the start-of-step positions (solver.py:515-520)
    if (err == cudaSuccess) err = launch_contact_begin(p->cv, p->vv, s);
    for (int it = 0; err == cudaSuccess && it < p->cfg.iterations; ++it) {
        err = launch_element(q_out, p->cfg.energy, p->tv, p->diagnostics, s);
        if (err == cudaSuccess) err = contact_and_assemble(p, q_out, dt, s, it % p->factor_refresh == 0);
        if (err == cudaSuccess) err = global_solve(p, it, s);
        if (err == cudaSuccess && p->check_on)
            err = launch_true_residual(p->bv, p->vv, p->check_resid + 2 * it, s);
        if (err == cudaSuccess) err = local_update(p, q_out, dt, it, s);
    }
    if (err == cudaSuccess) err = launch_velocity(q_out, qd_out, dt, p->vv, s);
    return err;
}

// CTA tasks for the batched PCG.  The time of body b on g CTAs is modelled
// as its_b * (nnzb_b / g + c0 [g > 1]) (block products per iteration, plus
// the cost of a group barrier pair in the same unit); starting from one CTA
// per body, the body with the largest modelled time gets one more CTA while
// CTAs are left and that shortens it.  With more bodies than CTAs, bodies are
// dealt to CTAs largest first onto the least-loaded CTA (each alone).
void batch_schedule(const std::vector<int32_t> &nnzb, const std::vector<int32_t> &its, int capacity, double c0,
                    int max_group, std::vector<int> &task_ptr, std::vector<int4> &tasks, int &ctas) {
    const int B = (int)nnzb.size();
    task_ptr.clear();
    tasks.clear();
    auto work = [&](int b) { return (double)std::max(its[b], 1) * (double)nnzb[b]; };
    if (B <= capacity) {
        std::vector<int> g(B, 1);
        auto model = [&](int b, int gb) {
            return (double)std::max(its[b], 1) * ((double)nnzb[b] / gb + (gb > 1 ? c0 : 0.0));
        };
        std::vector<std::pair<double, int>> heap;
        for (int b = 0; b < B; ++b) heap.push_back({model(b, 1), b});
        std::make_heap(heap.begin(), heap.end());
        int spare = capacity - B;
        while (spare > 0 && !heap.empty()) {
            std::pop_heap(heap.begin(), heap.end());
            auto [t, b] = heap.back();
            heap.pop_back();
            // a group's barrier serialises its arrivals: groups stay at most
            // max_group CTAs
            const double t1 = g[b] < max_group ? model(b, g[b] + 1) : t;
            if (!(t1 < t)) break;  // the critical body gains nothing from another CTA
            ++g[b];
            --spare;
            heap.push_back({t1, b});
            std::push_heap(heap.begin(), heap.end());
        }
        int c = 0;
        task_ptr.push_back(0);
        for (int b = 0; b < B; ++b)
            for (int r = 0; r < g[b]; ++r) {
                tasks.push_back(make_int4(b, r, g[b], c - r));
                task_ptr.push_back((int)tasks.size());
                ++c;
            }
        ctas = c;
        return;
    }
    std::vector<int> order(B);
    for (int b = 0; b < B; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work(a) > work(b); });
    std::vector<std::vector<int>> bins(capacity);
    std::vector<double> load(capacity, 0.0);
    for (int b : order) {
        const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        bins[c].push_back(b);
        load[c] += work(b);
    }
    task_ptr.push_back(0);
    for (int c = 0; c < capacity; ++c) {
        std::sort(bins[c].begin(), bins[c].end());
        for (int b : bins[c]) tasks.push_back(make_int4(b, 0, 1, c));
        task_ptr.push_back((int)tasks.size());
    }
    ctas = capacity;
}

uint64_t count_kernel_nodes(cudaGraph_t g) {
    size_t num = 0;
    if (cudaGraphGetNodes(g, nullptr, &num) != cudaSuccess || num == 0) return 0;
    std::vector<cudaGraphNode_t> nodes(num);
    if (cudaGraphGetNodes(g, nodes.data(), &num) != cudaSuccess) return 0;
    uint64_t k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType ty;
        if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

}  // namespace

int install_bodies(mfem_plan *p, int n_bodies, const int32_t *voff, const int32_t *toff, const int32_t *energy,
                   const float *gravity);

extern "C" {

void mfem_config_default(mfem_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->iterations = 8;
    cfg->energy = MFEM_ENERGY_ARAP;
    cfg->cg_max_iterations = 1000;
    cfg->cg_tolerance = 1.0e-6f;
    cfg->attachment_stiffness = 10.0f;
    cfg->preconditioner_singular_threshold = 1.0e-20f;
    cfg->preconditioner = 1;
    cfg->use_cuda_graph = 1;
    cfg->pcg_ctas = 0;
    cfg->pcg_variant = 0;
    cfg->line_search = 1;
    cfg->line_search_max_iterations = 20;
    cfg->line_search_alpha0 = 1.0f;
    cfg->line_search_tau = 0.5f;
    cfg->line_search_c = 0.01f;
    cfg->line_search_threshold = 1.0e-8f;
}

const char *mfem_status_string(int status) {
    switch (status) {
        case MFEM_OK: return "ok";
        case MFEM_MAXITER: return "PCG reached cg_max_iterations";
        case MFEM_STAGNATION: return "PCG broke down (p.Ap <= 0)";
        case MFEM_NONFINITE: return "non-finite value in the PCG";
        case MFEM_BAD_ARG: return "invalid argument";
        case MFEM_CUDA_ERROR: return "CUDA error";
        case MFEM_TIMEOUT: return "device-side wait timed out";
        default: return "unknown status";
    }
}

uint64_t mfem_kernel_launch_count(void) { return g_launches.load(); }

int mfem_bsr_sparsity(int32_t n_particles, int32_t n_tets, const int32_t *h_tet_indices, int32_t *h_row_ptr,
                      int32_t *h_col_idx, int64_t *nnzb) {
    std::vector<int32_t> rp, ci;
    std::string err;
    if (!build_sparsity(n_particles, n_tets, h_tet_indices, rp, ci, err)) return fail(nullptr, MFEM_BAD_ARG, err);
    if (nnzb) *nnzb = (int64_t)ci.size();
    if (h_row_ptr) std::memcpy(h_row_ptr, rp.data(), rp.size() * sizeof(int32_t));
    if (h_col_idx && !ci.empty()) std::memcpy(h_col_idx, ci.data(), ci.size() * sizeof(int32_t));
    return MFEM_OK;
}

int mfem_tet_slot_map(int32_t n_particles, int32_t n_tets, const int32_t *h_tet_indices, const int32_t *h_row_ptr,
                      const int32_t *h_col_idx, int32_t *h_slots) {
    if (n_tets > 0 && (!h_row_ptr || !h_col_idx || !h_slots)) return fail(nullptr, MFEM_BAD_ARG, "NULL argument");
    std::string err;
    if (!build_slot_map(n_particles, n_tets, h_tet_indices, h_row_ptr, h_col_idx, h_slots, err))
        return fail(nullptr, MFEM_BAD_ARG, err);
    return MFEM_OK;
}

void mfem_plan_destroy(mfem_plan *p) {
    if (!p) return;
    {
        DeviceGuard g(p->device);
        for (auto &ge : p->graphs)
            if (ge.exec) cudaGraphExecDestroy(ge.exec);
        if (p->capture_stream) cudaStreamDestroy(p->capture_stream);
        for (void *a : p->allocs) cudaFree(a);
        for (void *a : p->contact_allocs) cudaFree(a);
        for (void *a : p->ir_allocs) cudaFree(a);
        for (void *a : p->batch_allocs) cudaFree(a);
        for (void *a : p->layout_allocs) cudaFree(a);
        for (void *a : p->net_allocs) cudaFree(a);
        for (void *a : p->refine_allocs) cudaFree(a);
    }
    delete p;
}

int mfem_plan_create(const mfem_config *cfg_in, int32_t n, int32_t T, const int32_t *h_tets, const float *h_poses,
                     const float *h_materials, const float *h_rest_q, const float *h_mass, const float *h_inv_mass,
                     const float *h_gravity, int32_t device, mfem_plan **out) {
    t_create_error.clear();
    if (!out) return fail(nullptr, MFEM_BAD_ARG, "out is NULL");
    *out = nullptr;
    mfem_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else mfem_config_default(&cfg);
    std::string err;
    if (!valid_config(&cfg, err)) return fail(nullptr, MFEM_BAD_ARG, err);
    if (n <= 0) return fail(nullptr, MFEM_BAD_ARG, "n_particles must be > 0");
    if (T < 0) return fail(nullptr, MFEM_BAD_ARG, "n_tets must be >= 0");
    if ((T > 0 && (!h_tets || !h_poses || !h_materials)) || !h_rest_q || !h_mass || !h_inv_mass || !h_gravity)
        return fail(nullptr, MFEM_BAD_ARG, "NULL model array");
    for (int v = 0; v < n; ++v)
        if (!(h_inv_mass[v] >= 0.0f) || !std::isfinite(h_inv_mass[v]))
            return fail(nullptr, MFEM_BAD_ARG, "particle_inv_mass must be finite and >= 0");

    Symbolic sym;
    if (!build_sparsity(n, T, h_tets, sym.row_ptr, sym.col_idx, err)) return fail(nullptr, MFEM_BAD_ARG, err);
    sym.tet_slots.resize((size_t)T * 16);
    if (!build_slot_map(n, T, h_tets, sym.row_ptr.data(), sym.col_idx.data(), sym.tet_slots.data(), err))
        return fail(nullptr, MFEM_BAD_ARG, err);
    if (!build_contributions(n, T, h_tets, sym.row_ptr.data(), sym.tet_slots.data(), sym, err))
        return fail(nullptr, MFEM_BAD_ARG, err);

    // (M + Q) diagonal: Hessian mass is identity on attached vertices and
    // I / inv_mass elsewhere (kernels.py:21-27); Q = k I on attached ones
    // (boundary_condition.py:18-42); summed in float32 like bsr_axpy.
    std::vector<float> hess_diag(n), pin_k(n);
    for (int v = 0; v < n; ++v) {
        const bool att = h_inv_mass[v] == 0.0f;
        const float m_h = att ? 1.0f : 1.0f / h_inv_mass[v];
        pin_k[v] = att ? cfg.attachment_stiffness : 0.0f;
        hess_diag[v] = att ? (m_h + cfg.attachment_stiffness) : m_h;
    }

    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || device < 0 || device >= dev_count)
        return fail(nullptr, MFEM_BAD_ARG, "no such CUDA device");
    DeviceGuard guard(device);
    if (!guard.ok) return fail(nullptr, MFEM_CUDA_ERROR, "cudaSetDevice failed");

    mfem_plan *p = new mfem_plan();
    p->cfg = cfg;
    p->device = device;
    p->n = n;
    p->T = T;
    p->nnzb = (int64_t)sym.col_idx.size();
    p->max_stats = cfg.iterations > 0 ? cfg.iterations : 1;
    for (int a = 0; a < 3; ++a) p->gravity[a] = h_gravity[a];

    const size_t nT = T, nn = n, nz = (size_t)p->nnzb;
    const int n_chunks = (int)sym.chunk_ptr.size() - 1;
    cudaError_t e = cudaSuccess;
    int4 *tets = nullptr;
    float *dminv = nullptr, *materials = nullptr, *mass = nullptr, *hd = nullptr, *pk = nullptr, *pt = nullptr;
    int32_t *row_ptr = nullptr, *col_idx = nullptr, *chunk_ptr = nullptr, *ccode = nullptr, *cslot = nullptr;
    float *rest = nullptr;
#define ALLOC(ptr, count)                                  \
    if (e == cudaSuccess) e = dev_alloc(p, &(ptr), (count));
    ALLOC(tets, nT);
    ALLOC(dminv, nT * 9);
    ALLOC(materials, nT * 3);
    ALLOC(p->tv.stretch, nT * 6);
    ALLOC(p->tv.lambda, nT * 6);
    ALLOC(p->tv.c, nT * 6);
    ALLOC(p->tv.G, nT * 72);
    ALLOC(p->tv.g_s, nT * 6);
    ALLOC(p->tv.H_l, nT * 21);
    ALLOC(p->tv.H_si, nT * 21);
    ALLOC(p->tv.g_l, nT * 6);
    ALLOC(p->tv.Ke, nT * kKeFloats);
    ALLOC(p->tv.fe, nT * kFeFloats);
    ALLOC(p->tv.degenerate, nT);
    ALLOC(p->tv.n_degenerate, 1);
    ALLOC(p->tet_slots, nT * 16);
    ALLOC(mass, nn);
    ALLOC(hd, nn);
    ALLOC(pk, nn);
    ALLOC(pt, nn * 3);
    ALLOC(rest, nn * 3);
    ALLOC(p->inv_mass, nn);
    ALLOC(p->vv.x_tilde, nn * 3);
    ALLOC(p->vv.x_start, nn * 3);
    ALLOC(p->vv.rhs, nn * 3);
    const size_t n_pad = (nn + 3) & ~(size_t)3;
    ALLOC(p->vv.dx, n_pad * 3);
    ALLOC(p->vv.Minv, n_pad * 9);
    ALLOC(row_ptr, nn + 1);
    ALLOC(col_idx, nz);
    ALLOC(p->bv.values, nz * 9);
    ALLOC(chunk_ptr, (size_t)n_chunks + 1);
    ALLOC(ccode, sym.contrib_code.size());
    ALLOC(cslot, sym.contrib_slot.size());
    ALLOC(p->pw.pub, 6 * n_pad * 3);
    ALLOC(p->pw.partials, 2 * 256 * 4);
    ALLOC(p->pw.counter, 1);
    ALLOC(p->pw.error, 1);
    ALLOC(p->pw.stats, (size_t)p->max_stats);
    ALLOC(p->resid, 2);
    const int local_blocks = std::max(1, local_solve_blocks(T, n));  // grown by mfem_plan_set_contact
    ALLOC(p->ls.ds, nT * 6);
    ALLOC(p->ls.local_partials, (size_t)local_blocks * 2);
    ALLOC(p->ls.partials, (size_t)2 * kLsMaxCtas * 3);
    ALLOC(p->ls.counter, 1);
    ALLOC(p->ls.stats, (size_t)p->max_stats);
#undef ALLOC
    if (e != cudaSuccess) {
        int rc = cuda_fail(nullptr, e, "cudaMalloc");
        mfem_plan_destroy(p);
        return rc;
    }
    int max_ctas = 1;
    p->pw.n_pad = (int)n_pad;
    e = pcg_max_ctas(device, &max_ctas);
    std::vector<int4> cta_info;
    if (e == cudaSuccess) {
        int want = cfg.pcg_ctas > 0 ? cfg.pcg_ctas : std::max(1, std::min(max_ctas, (n + 63) / 64));
        p->pcg_ctas = std::max(1, std::min(want, max_ctas));
    }
    if (e == cudaSuccess) {
        int ls_max = 1;
        e = line_search_max_ctas(device, &ls_max);
        // one trial touches every tet and vertex once: about one per thread
        const int want = std::max(1, (std::max(T, n) + 255) / 256);
        p->ls.ctas = std::max(1, std::min(want, ls_max));
        p->ls.local_blocks = local_blocks;
        p->ls.max_iter = cfg.line_search_max_iterations;
        p->ls.alpha0 = cfg.line_search_alpha0;
        p->ls.tau = cfg.line_search_tau;
        p->ls.c = cfg.line_search_c;
        p->ls.threshold = cfg.line_search_threshold;
    }
    std::vector<int4> factor_info;
    if (e == cudaSuccess && (cfg.preconditioner >= 2 || cfg.pcg_variant == PcgLayout::kGlobalMemory)) {
        // the factor structures and the block-Jacobi retry live in the
        // one-body batch views; the persistent factor PCG runs when its
        // ranges fit in shared memory, else the global-memory PCG
        p->pl = PcgLayout{};
        p->pl.variant = 0;
        p->global_memory_pcg = true;
        cta_info.assign(1, make_int4(0, 0, 0, 0));
        if (cfg.preconditioner >= 2 && cfg.pcg_variant != PcgLayout::kGlobalMemory) {
            std::string lerr;
            PcgLayout fl{};
            std::vector<int4> fcta;
            e = pcg_factor_layout(device, fl, sym.row_ptr.data(), sym.col_idx.data(), n, p->pcg_ctas,
                                  cfg.preconditioner, fcta, factor_info, lerr);
            if (e == cudaSuccess) {
                p->pl = fl;
                cta_info = fcta;
            } else if (!lerr.empty()) {
                if (cfg.pcg_variant == PcgLayout::kFactor) {
                    mfem_plan_destroy(p);
                    return fail(nullptr, MFEM_BAD_ARG, lerr);
                }
                cudaGetLastError();
                e = cudaSuccess;
                factor_info.clear();
            }
        }
    } else if (e == cudaSuccess) {
        std::string lerr;
        e = pcg_plan_layout(device, p->pl, sym.row_ptr.data(), sym.col_idx.data(), n, p->pcg_ctas, cfg.pcg_variant,
                            cta_info, lerr);
        if (e != cudaSuccess && !lerr.empty()) {
            if (cfg.pcg_variant != PcgLayout::kAuto) {
                mfem_plan_destroy(p);
                return fail(nullptr, MFEM_BAD_ARG, lerr);
            }
            // too large for the shared-memory PCG: the global solve runs the
            // global-memory PCG of the batched kernel as a one-body batch
            cudaGetLastError();
            e = cudaSuccess;
            p->pl = PcgLayout{};
            p->pl.variant = 0;
            p->global_memory_pcg = true;
            cta_info.assign(1, make_int4(0, 0, 0, 0));
        }
    }
    std::vector<int4> ir_cta, ir_fcta;
    if (e == cudaSuccess && !p->global_memory_pcg && cfg.preconditioner == 1) {
        std::string lerr;
        PcgLayout il{};
        if (pcg_factor_layout(device, il, sym.row_ptr.data(), sym.col_idx.data(), n, p->pcg_ctas, 2, ir_cta, ir_fcta,
                              lerr, false) == cudaSuccess) {
            p->ir_pl = il;
        } else {
            cudaGetLastError();
            ir_cta.clear();
            ir_fcta.clear();
        }
    }
    int4 *d_cta = nullptr;
    if (e == cudaSuccess) e = dev_alloc(p, &d_cta, cta_info.size());
    if (e == cudaSuccess) e = upload(d_cta, cta_info.data(), cta_info.size());
    p->pl.cta_info = d_cta;
    if (e == cudaSuccess && !factor_info.empty()) {
        int4 *d_fcta = nullptr;
        e = dev_alloc(p, &d_fcta, factor_info.size());
        if (e == cudaSuccess) e = upload(d_fcta, factor_info.data(), factor_info.size());
        p->pl.factor_info = d_fcta;
    }
    if (e == cudaSuccess && p->ir_pl.variant == PcgLayout::kFactor) {
        int4 *d_icta = nullptr, *d_ifcta = nullptr;
        e = dev_alloc(p, &d_icta, ir_cta.size());
        if (e == cudaSuccess) e = upload(d_icta, ir_cta.data(), ir_cta.size());
        if (e == cudaSuccess) e = dev_alloc(p, &d_ifcta, ir_fcta.size());
        if (e == cudaSuccess) e = upload(d_ifcta, ir_fcta.data(), ir_fcta.size());
        p->ir_pl.cta_info = d_icta;
        p->ir_pl.factor_info = d_ifcta;
    }
    if (e == cudaSuccess) e = upload(tets, reinterpret_cast<const int4 *>(h_tets), nT);
    if (e == cudaSuccess) e = upload(dminv, h_poses, nT * 9);
    if (e == cudaSuccess) e = upload(materials, h_materials, nT * 3);
    if (e == cudaSuccess) e = upload(p->tet_slots, sym.tet_slots.data(), nT * 16);
    if (e == cudaSuccess) e = upload(mass, h_mass, nn);
    if (e == cudaSuccess) e = upload(hd, hess_diag.data(), nn);
    if (e == cudaSuccess) e = upload(pk, pin_k.data(), nn);
    if (e == cudaSuccess) e = upload(pt, h_rest_q, nn * 3);
    if (e == cudaSuccess) e = upload(rest, h_rest_q, nn * 3);
    if (e == cudaSuccess) e = upload(p->inv_mass, h_inv_mass, nn);
    if (e == cudaSuccess) e = upload(row_ptr, sym.row_ptr.data(), nn + 1);
    if (e == cudaSuccess) e = upload(col_idx, sym.col_idx.data(), nz);
    if (e == cudaSuccess) e = upload(chunk_ptr, sym.chunk_ptr.data(), (size_t)n_chunks + 1);
    if (e == cudaSuccess) e = upload(ccode, sym.contrib_code.data(), sym.contrib_code.size());
    if (e == cudaSuccess) e = upload(cslot, sym.contrib_slot.data(), sym.contrib_slot.size());
    if (e == cudaSuccess) e = cudaMemset(p->pw.partials, 0, 2 * 256 * 4 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->pw.counter, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(p->pw.error, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->ls.counter, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(p->ls.stats, 0, sizeof(LineSearchStats) * p->max_stats);
    if (e == cudaSuccess) e = cudaMemset(p->ls.ds, 0, nT * 6 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->ls.local_partials, 0, (size_t)local_blocks * 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(p->pw.stats, 0, sizeof(SolveStats) * p->max_stats);
    if (e == cudaSuccess) e = cudaMemset(p->vv.dx, 0, n_pad * 3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->pw.pub, 0, 6 * n_pad * 3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->vv.Minv, 0, n_pad * 9 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->bv.values, 0, nz * 9 * sizeof(float));
    if (e != cudaSuccess) {
        int rc = cuda_fail(nullptr, e, "plan upload");
        mfem_plan_destroy(p);
        return rc;
    }
    p->tv.n_tets = T;
    p->tv.tets = tets;
    p->tv.dminv = dminv;
    p->tv.materials = materials;
    p->rest_q = rest;
    p->mass = mass;
    p->vv.n = n;
    p->vv.mass = mass;
    p->vv.hess_diag = hd;
    p->vv.pin_k = pk;
    p->vv.pin_target = pt;
    p->bv.n = n;
    p->bv.nnzb = p->nnzb;
    p->bv.row_ptr = row_ptr;
    p->bv.col_idx = col_idx;
    p->bv.n_chunks = n_chunks;
    p->bv.chunk_ptr = chunk_ptr;
    p->bv.contrib_code = ccode;
    p->bv.contrib_slot = cslot;
    p->base_chunk_ptr = chunk_ptr;
    p->base_code = ccode;
    p->base_slot = cslot;
    p->base_chunks = n_chunks;
    p->h_tets.assign(h_tets, h_tets + (size_t)T * 4);
    p->h_row_ptr = sym.row_ptr;
    p->h_col_idx = sym.col_idx;
    p->h_tet_slots = sym.tet_slots;
    p->cv.tri_code_base = INT32_MAX;

    // s = S(F) at rest, lambda = 0 (additional_state.py:146-189)
    e = prepare_element_kernels();
    if (e == cudaSuccess) e = launch_initial_stretch(rest, p->tv, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        int rc = cuda_fail(nullptr, e, "plan initialisation");
        mfem_plan_destroy(p);
        return rc;
    }
    if (p->global_memory_pcg) {
        const int32_t voff[2] = {0, n}, toff[2] = {0, T};
        const int rc = install_bodies(p, 1, voff, toff, nullptr, nullptr);
        if (rc != MFEM_OK) {
            const std::string msg = p->last_error;
            mfem_plan_destroy(p);
            return fail(nullptr, rc, msg);
        }
    }
    *out = p;
    return MFEM_OK;
}

const char *mfem_plan_last_error(const mfem_plan *p) { return p ? p->last_error.c_str() : t_create_error.c_str(); }

int mfem_plan_sizes(const mfem_plan *p, int32_t *n, int32_t *T, int64_t *nnzb) {
    if (!p) return MFEM_BAD_ARG;
    if (n) *n = p->n;
    if (T) *T = p->T;
    if (nnzb) *nnzb = p->nnzb;
    return MFEM_OK;
}

int mfem_plan_pcg_layout(const mfem_plan *p, int32_t *variant, int32_t *ctas, int32_t *cache_matrix,
                         int64_t *smem_bytes) {
    if (!p) return MFEM_BAD_ARG;
    if (variant) *variant = p->pl.variant;
    if (ctas) *ctas = p->pcg_ctas;
    if (cache_matrix) *cache_matrix = p->pl.cache_matrix;
    if (smem_bytes) *smem_bytes = (int64_t)p->pl.smem;
    return MFEM_OK;
}

int mfem_plan_buffer_bytes(const mfem_plan *p, int32_t which, size_t *bytes) {
    if (!p || !bytes) return MFEM_BAD_ARG;
    BufferRef ref;
    if (!buffer_ref(p, which, ref)) return fail(const_cast<mfem_plan *>(p), MFEM_BAD_ARG, "unknown buffer");
    *bytes = ref.bytes;
    return MFEM_OK;
}

int mfem_plan_copy_out(const mfem_plan *pc, int32_t which, void *dst, size_t bytes, mfem_stream stream) {
    mfem_plan *p = const_cast<mfem_plan *>(pc);
    if (!p) return MFEM_BAD_ARG;
    BufferRef ref;
    if (!buffer_ref(p, which, ref)) return fail(p, MFEM_BAD_ARG, "unknown buffer");
    if (bytes != ref.bytes) return fail(p, MFEM_BAD_ARG, "byte count does not match the buffer");
    if (bytes == 0) return MFEM_OK;
    if (!dst) return fail(p, MFEM_BAD_ARG, "dst is NULL");
    DeviceGuard g(p->device);
    cudaError_t e = cudaMemcpyAsync(dst, ref.ptr, bytes, cudaMemcpyDefault, (cudaStream_t)stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "copy_out");
}

int mfem_plan_copy_in(mfem_plan *p, int32_t which, const void *src, size_t bytes, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    BufferRef ref;
    if (!buffer_ref(p, which, ref)) return fail(p, MFEM_BAD_ARG, "unknown buffer");
    if (which == MFEM_BUF_ROW_PTR || which == MFEM_BUF_COL_IDX || which == MFEM_BUF_TET_SLOTS)
        return fail(p, MFEM_BAD_ARG, "the sparsity and slot map are read-only");
    if (bytes != ref.bytes) return fail(p, MFEM_BAD_ARG, "byte count does not match the buffer");
    if (bytes == 0) return MFEM_OK;
    if (!src) return fail(p, MFEM_BAD_ARG, "src is NULL");
    DeviceGuard g(p->device);
    cudaError_t e = cudaMemcpyAsync(ref.ptr, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "copy_in");
}

int mfem_step(mfem_plan *p, const float *q_in, const float *qd_in, float *q_out, float *qd_out, float dt,
              mfem_stream stream_) {
    if (!p) return MFEM_BAD_ARG;
    if (!q_in || !qd_in || !q_out || !qd_out) return fail(p, MFEM_BAD_ARG, "NULL state pointer");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(p, MFEM_BAD_ARG, "dt must be finite and > 0");
    if (!net_ready(p)) return fail(p, MFEM_BAD_ARG, "preconditioner 3 needs mfem_plan_set_factor_net");
    if ((const void *)qd_in == (const void *)q_out || (const void *)q_in == (const void *)qd_out)
        return fail(p, MFEM_BAD_ARG, "positions and velocities must not alias");
    cudaStream_t stream = (cudaStream_t)stream_;
    DeviceGuard g(p->device);
    cudaError_t e = cudaSuccess;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (stream) e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamIsCapturing");
    if (p->cfg.use_cuda_graph && cap == cudaStreamCaptureStatusNone) {
        const void *key[4] = {q_in, qd_in, q_out, qd_out};
        mfem_plan::GraphEntry *ge = nullptr;
        for (auto &cand : p->graphs) {
            bool hit = cand.exec && cand.dt == dt;
            for (int i = 0; i < 4 && hit; ++i) hit = cand.key[i] == key[i];
            if (hit) {
                ge = &cand;
                break;
            }
        }
        if (!ge) {
            ge = &p->graphs[0];
            for (auto &cand : p->graphs)
                if (!cand.exec || cand.last_use < ge->last_use) ge = &cand;
            if (ge->exec) {
                cudaGraphExecDestroy(ge->exec);
                ge->exec = nullptr;
            }
            cudaGraph_t graph = nullptr;
            t_capturing = true;
            e = cudaStreamBeginCapture(p->capture_stream, cudaStreamCaptureModeThreadLocal);
            cudaError_t run_err = cudaSuccess;
            if (e == cudaSuccess) {
                run_err = run_step(p, q_in, qd_in, q_out, qd_out, dt, p->capture_stream);
                e = cudaStreamEndCapture(p->capture_stream, &graph);
            }
            t_capturing = false;
            if (e == cudaSuccess && run_err != cudaSuccess) e = run_err;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&ge->exec, graph, 0);
            if (graph) {
                ge->kernels = count_kernel_nodes(graph);
                cudaGraphDestroy(graph);
            }
            if (e != cudaSuccess) {
                ge->exec = nullptr;
                cudaGetLastError();
                return cuda_fail(p, e, "step graph capture");
            }
            for (int i = 0; i < 4; ++i) ge->key[i] = key[i];
            ge->dt = dt;
        }
        ge->last_use = ++p->graph_clock;
        e = cudaGraphLaunch(ge->exec, stream);
        if (e != cudaSuccess) return cuda_fail(p, e, "cudaGraphLaunch");
        count_launches(ge->kernels);
        return MFEM_OK;
    }
    e = run_step(p, q_in, qd_in, q_out, qd_out, dt, stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "step launch");
}

int mfem_step_stats(mfem_plan *p, mfem_solve_stats *h_stats, int32_t max_entries, int32_t *count,
                    mfem_stream stream) {
    if (!p || (max_entries > 0 && !h_stats)) return MFEM_BAD_ARG;
    DeviceGuard g(p->device);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamSynchronize");
    const int k = std::max(0, std::min<int>(max_entries, p->cfg.iterations));
    std::vector<SolveStats> tmp(p->max_stats);
    if (p->bw.n_bodies > 0 && p->ir.mode == 0) {
        // the global-memory PCG's per-body records, [slot][body]: a single
        // body's own, else per slot the most iterations, the largest
        // residual and the first body's failure
        const int B = p->bw.n_bodies;
        std::vector<SolveStats> all((size_t)p->max_stats * B);
        e = cudaMemcpy(all.data(), p->bw.stats, all.size() * sizeof(SolveStats), cudaMemcpyDeviceToHost);
        for (int i = 0; e == cudaSuccess && i < p->max_stats; ++i) {
            SolveStats agg = all[(size_t)i * B];
            for (int b = 1; b < B; ++b) {
                const SolveStats &sb = all[(size_t)i * B + b];
                agg.iterations = std::max(agg.iterations, sb.iterations);
                agg.rel_residual = std::max(agg.rel_residual, sb.rel_residual);
                if (agg.status == MFEM_OK && sb.status != MFEM_OK) agg.status = sb.status;
            }
            tmp[i] = agg;
        }
    } else {
        e = cudaMemcpy(tmp.data(), p->pw.stats, sizeof(SolveStats) * p->max_stats, cudaMemcpyDeviceToHost);
    }
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&flag, p->pw.error, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p, e, "stats readback");
    for (int i = 0; i < k; ++i) std::memcpy(&h_stats[i], &tmp[i], sizeof(mfem_solve_stats));
    if (count) *count = k;
    if (flag) {
        // a bounded wait gave up: re-arm the grid barriers for the next solve
        e = rearm_barriers(p);
        if (e != cudaSuccess) return cuda_fail(p, e, "re-arming the grid barriers");
        return fail(p, MFEM_TIMEOUT, "a PCG or line-search grid barrier timed out");
    }
    return MFEM_OK;
}

void mfem_contact_config_default(mfem_contact_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->d0 = 1.0e-2f;
    cfg->d1 = 1.0e-1f;
    cfg->stiffness = 1.0e7f;
    cfg->friction_eps_v = 1.0e-3f;
    cfg->tri_contact = 1;
}

int mfem_plan_set_contact(mfem_plan *p, const mfem_contact_config *cfg_in, int32_t n_shapes,
                          const int32_t *h_shape_type, const float *h_shape_pose, const float *h_shape_scale,
                          const int32_t *h_shape_body, const float *h_friction_mu, int32_t n_bodies, int32_t n_tris,
                          const int32_t *h_tris) {
    if (!p) return MFEM_BAD_ARG;
    mfem_contact_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else mfem_contact_config_default(&cfg);
    if (n_shapes < 0 || n_shapes > kMaxShapes) return fail(p, MFEM_BAD_ARG, "n_shapes must be in [0, 64]");
    if (n_bodies < 0 || n_tris < 0) return fail(p, MFEM_BAD_ARG, "negative n_bodies or n_tris");
    if (n_shapes > 0 && (!h_shape_type || !h_shape_pose || !h_shape_scale || !h_shape_body || !h_friction_mu))
        return fail(p, MFEM_BAD_ARG, "NULL shape array");
    if (n_tris > 0 && !h_tris) return fail(p, MFEM_BAD_ARG, "h_tris is NULL");
    if (!(cfg.d1 > cfg.d0) || !(cfg.d0 > 0.0f) || !std::isfinite(cfg.d1))
        return fail(p, MFEM_BAD_ARG, "contact distances need 0 < d0 < d1");
    if (!(cfg.stiffness >= 0.0f) || !std::isfinite(cfg.stiffness) || !(cfg.friction_eps_v >= 0.0f) ||
        !std::isfinite(cfg.friction_eps_v))
        return fail(p, MFEM_BAD_ARG, "contact stiffness and friction_eps_v must be finite and >= 0");
    bool friction = false;
    for (int s = 0; s < n_shapes; ++s) {
        if (h_shape_body[s] >= n_bodies) return fail(p, MFEM_BAD_ARG, "shape body index out of range");
        if (!(h_friction_mu[s] >= 0.0f) || !std::isfinite(h_friction_mu[s]))
            return fail(p, MFEM_BAD_ARG, "friction_mu must be finite and >= 0");
        for (int i = 0; i < 7; ++i)
            if (!std::isfinite(h_shape_pose[7 * s + i])) return fail(p, MFEM_BAD_ARG, "non-finite shape pose");
        friction = friction || h_friction_mu[s] > 0.0f;
    }
    const int m = (cfg.tri_contact && n_shapes > 0) ? n_tris : 0;
    std::vector<int32_t> tri_slots((size_t)m * 9), vt_ptr, vt_code;
    std::string err;
    if (m > 0 && !build_tri_slots(p->n, m, h_tris, p->h_row_ptr.data(), p->h_col_idx.data(), tri_slots.data(),
                                  vt_ptr, vt_code, err))
        return fail(p, MFEM_BAD_ARG, err);
    Symbolic sym;
    sym.col_idx = p->h_col_idx;
    if (m > 0 && !build_contributions(p->n, p->T, p->h_tets.data(), p->h_row_ptr.data(), p->h_tet_slots.data(), sym,
                                      err, m, tri_slots.data()))
        return fail(p, MFEM_BAD_ARG, err);

    DeviceGuard g(p->device);
    cudaError_t e = cudaDeviceSynchronize();  // no step of this plan may still read the old buffers
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaDeviceSynchronize");
    for (auto &ge : p->graphs) {
        if (ge.exec) cudaGraphExecDestroy(ge.exec);
        ge = mfem_plan::GraphEntry{};
    }
    for (void *a : p->contact_allocs) cudaFree(a);
    p->contact_allocs.clear();
    p->cv = ContactViews{};
    p->cv.tri_code_base = INT32_MAX;
    p->bv.chunk_ptr = p->base_chunk_ptr;
    p->bv.contrib_code = p->base_code;
    p->bv.contrib_slot = p->base_slot;
    p->bv.n_chunks = p->base_chunks;
    p->n_bodies = 0;
    p->n_tris = 0;
    p->h_tris.clear();
    p->refine_ready = false;
    if (n_shapes == 0) return MFEM_OK;  // contact off

    const size_t n = p->n;
    auto alloc = [&](auto **ptr, size_t count) {
        if (e != cudaSuccess) return;
        void *raw = nullptr;
        e = cudaMalloc(&raw, std::max<size_t>(count, 1) * sizeof(**ptr));
        if (e == cudaSuccess) {
            p->contact_allocs.push_back(raw);
            *ptr = static_cast<std::remove_reference_t<decltype(*ptr)>>(raw);
        }
    };
    int *type = nullptr, *body = nullptr, *tris = nullptr, *vtp = nullptr, *vtc = nullptr;
    float *pose = nullptr, *scale = nullptr, *mu = nullptr, *body_q = nullptr;
    int32_t *chunk_ptr = nullptr, *ccode = nullptr, *cslot = nullptr;
    ContactViews &cv = p->cv;
    alloc(&type, n_shapes);
    alloc(&pose, (size_t)n_shapes * 7);
    alloc(&scale, (size_t)n_shapes * 3);
    alloc(&body, n_shapes);
    alloc(&mu, n_shapes);
    alloc(&body_q, (size_t)std::max(n_bodies, 1) * 7);
    alloc(&cv.normal_lagged, n * 3);
    alloc(&cv.force_lagged, n);
    alloc(&cv.shape_lagged, n);
    alloc(&cv.vblock, n * 9);
    alloc(&cv.vgrad, n * 3);
    alloc(&cv.venergy, n);
    alloc(&cv.gtot, n * 3);
    alloc(&cv.tri, (size_t)m * kTriData);
    alloc(&tris, (size_t)m * 3);
    alloc(&vtp, n + 1);
    alloc(&vtc, (size_t)m * 3);
    const int n_chunks = m > 0 ? (int)sym.chunk_ptr.size() - 1 : 0;
    if (m > 0) {
        alloc(&chunk_ptr, sym.chunk_ptr.size());
        alloc(&ccode, sym.contrib_code.size());
        alloc(&cslot, sym.contrib_slot.size());
    }
    // the deferred local solve's partials cover max(vertices, tris); they
    // live as long as the plan
    const int local_blocks = std::max(1, local_solve_blocks(p->T, std::max(p->n, m)));
    double *local_partials = nullptr;
    if (e == cudaSuccess && local_blocks > p->ls.local_blocks) e = dev_alloc(p, &local_partials, (size_t)local_blocks * 2);
    std::vector<float> ident((size_t)std::max(n_bodies, 1) * 7, 0.0f);
    for (size_t b = 0; b < ident.size() / 7; ++b) ident[7 * b + 6] = 1.0f;
    if (e == cudaSuccess) e = upload(type, h_shape_type, n_shapes);
    if (e == cudaSuccess) e = upload(pose, h_shape_pose, (size_t)n_shapes * 7);
    if (e == cudaSuccess) e = upload(scale, h_shape_scale, (size_t)n_shapes * 3);
    if (e == cudaSuccess) e = upload(body, h_shape_body, n_shapes);
    if (e == cudaSuccess) e = upload(mu, h_friction_mu, n_shapes);
    if (e == cudaSuccess) e = upload(body_q, ident.data(), ident.size());
    if (e == cudaSuccess && m > 0) e = upload(tris, h_tris, (size_t)m * 3);
    if (e == cudaSuccess && m > 0) e = upload(vtp, vt_ptr.data(), n + 1);
    else if (e == cudaSuccess) e = cudaMemset(vtp, 0, (n + 1) * sizeof(int));
    if (e == cudaSuccess && m > 0) e = upload(vtc, vt_code.data(), (size_t)m * 3);
    if (e == cudaSuccess && m > 0) e = upload(chunk_ptr, sym.chunk_ptr.data(), sym.chunk_ptr.size());
    if (e == cudaSuccess && m > 0) e = upload(ccode, sym.contrib_code.data(), sym.contrib_code.size());
    if (e == cudaSuccess && m > 0) e = upload(cslot, sym.contrib_slot.data(), sym.contrib_slot.size());
    if (e == cudaSuccess) e = cudaMemset(cv.normal_lagged, 0, n * 3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(cv.force_lagged, 0, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(cv.shape_lagged, 0xff, n * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(cv.vblock, 0, n * 9 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(cv.vgrad, 0, n * 3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(cv.venergy, 0, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(cv.gtot, 0, n * 3 * sizeof(float));
    if (e == cudaSuccess && m > 0) e = cudaMemset(cv.tri, 0, (size_t)m * kTriData * sizeof(float));
    if (e != cudaSuccess) {
        for (void *a : p->contact_allocs) cudaFree(a);
        p->contact_allocs.clear();
        p->cv = ContactViews{};
        p->cv.tri_code_base = INT32_MAX;
        return cuda_fail(p, e, "contact buffers");
    }
    if (local_partials) {
        p->ls.local_partials = local_partials;
        p->ls.local_blocks = local_blocks;
    }
    float q0, q1, q2;
    {
        // (b, b', b'') of the log branch at d0 (contact.py:799)
        const float d = cfg.d0, d1 = cfg.d1;
        const float l = std::log(d / d1), a = d - d1;
        q0 = -a * a * l;
        q1 = -(2.0f * a * l + a * a / d);
        q2 = -(2.0f * l + 4.0f * a / d - a * a / (d * d));
    }
    cv.on = 1;
    cv.n_shapes = n_shapes;
    cv.type = type;
    cv.pose = pose;
    cv.scale = scale;
    cv.body = body;
    cv.mu = mu;
    cv.body_q = body_q;
    cv.friction = friction ? 1 : 0;
    cv.d0 = cfg.d0;
    cv.d1 = cfg.d1;
    cv.k = cfg.stiffness;
    cv.eps_v = cfg.friction_eps_v;
    cv.q[0] = q0;
    cv.q[1] = q1;
    cv.q[2] = q2;
    cv.n_tris = m;
    cv.tris = tris;
    cv.vt_ptr = vtp;
    cv.vt_code = vtc;
    cv.tri_code_base = m > 0 ? 16 * p->T : INT32_MAX;
    if (m > 0) {
        p->bv.chunk_ptr = chunk_ptr;
        p->bv.contrib_code = ccode;
        p->bv.contrib_slot = cslot;
        p->bv.n_chunks = n_chunks;
    }
    p->n_bodies = n_bodies;
    p->n_tris = m;
    p->h_tris.assign(h_tris, h_tris + (size_t)m * 3);
    p->refine_ready = false;  // the refinement's tri edge lists follow the tris
    return MFEM_OK;
}

int mfem_set_body_poses(mfem_plan *p, const float *body_q, int32_t n_bodies, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    if (n_bodies != p->n_bodies) return fail(p, MFEM_BAD_ARG, "n_bodies does not match mfem_plan_set_contact");
    if (n_bodies == 0) return MFEM_OK;
    if (!body_q) return fail(p, MFEM_BAD_ARG, "body_q is NULL");
    DeviceGuard g(p->device);
    cudaError_t e = cudaMemcpyAsync(const_cast<float *>(p->cv.body_q), body_q, (size_t)n_bodies * 7 * sizeof(float),
                                    cudaMemcpyDefault, (cudaStream_t)stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "set_body_poses");
}

void mfem_solver_config_default(mfem_solver_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->precision = MFEM_PRECISION_FP32;
    cfg->inner_tolerance = 1.0e-3f;
    cfg->outer_max_iterations = 10;
    cfg->factor_refresh = 1;
    cfg->outer_tolerance = 1.0e-8;
}

int mfem_plan_set_solver(mfem_plan *p, const mfem_solver_config *cfg_in) {
    if (!p) return MFEM_BAD_ARG;
    mfem_solver_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else mfem_solver_config_default(&cfg);
    if (cfg.precision != MFEM_PRECISION_FP32 && cfg.precision != MFEM_PRECISION_BF16 &&
        cfg.precision != MFEM_PRECISION_FP16 && cfg.precision != MFEM_PRECISION_FP32_REFINED)
        return fail(p, MFEM_BAD_ARG, "unknown precision");
    if (!(cfg.inner_tolerance > 0.0f) || !(cfg.inner_tolerance < 1.0f))
        return fail(p, MFEM_BAD_ARG, "inner_tolerance must be in (0, 1)");
    if (!(cfg.outer_tolerance > 0.0) || !std::isfinite(cfg.outer_tolerance))
        return fail(p, MFEM_BAD_ARG, "outer_tolerance must be finite and > 0");
    if (cfg.outer_max_iterations < 1 || cfg.outer_max_iterations > 100)
        return fail(p, MFEM_BAD_ARG, "outer_max_iterations must be in [1, 100]");
    if (p->bw.n_bodies > 1 && cfg.precision != MFEM_PRECISION_FP32)
        return fail(p, MFEM_BAD_ARG, "batched bodies use the fp32 PCG");

    DeviceGuard g(p->device);
    cudaError_t e = cudaDeviceSynchronize();  // no step of this plan may still use the old buffers
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaDeviceSynchronize");
    for (auto &ge : p->graphs) {
        if (ge.exec) cudaGraphExecDestroy(ge.exec);
        ge = mfem_plan::GraphEntry{};
    }
    for (void *a : p->ir_allocs) cudaFree(a);
    p->ir_allocs.clear();
    p->ir = IrWork{};
    if (cfg.factor_refresh < 0) return fail(p, MFEM_BAD_ARG, "factor_refresh must be >= 0");
    p->factor_refresh = std::max(1, cfg.factor_refresh);
    if (cfg.precision == MFEM_PRECISION_FP32) return MFEM_OK;

    const size_t n3 = (size_t)p->n * 3, nz = (size_t)p->nnzb;
    auto alloc = [&](auto **ptr, size_t bytes) {
        if (e != cudaSuccess) return;
        void *raw = nullptr;
        e = cudaMalloc(&raw, std::max<size_t>(bytes, 16));
        if (e == cudaSuccess) {
            p->ir_allocs.push_back(raw);
            *ptr = static_cast<std::remove_reference_t<decltype(*ptr)>>(raw);
        }
    };
    IrWork w{};
    const bool refined32 = cfg.precision == MFEM_PRECISION_FP32_REFINED;
    w.mode = refined32 ? kIrFp32 : (cfg.precision == MFEM_PRECISION_BF16 ? kIrBf16 : kIrFp16);
    w.outer_max = cfg.outer_max_iterations;
    w.inner_tol = cfg.inner_tolerance;
    w.outer_tol = cfg.outer_tolerance;
    alloc(&w.lowp, refined32 ? 16 : nz * 9 * 2);
    alloc(&w.row_scale, (size_t)p->n * sizeof(float));
    alloc(&w.dx_pair, 2 * n3 * sizeof(float2));
    alloc(&w.dx_out, n3 * sizeof(double));
    alloc(&w.e, n3 * sizeof(float));
    alloc(&w.res, n3 * sizeof(float));
    alloc(&w.z, n3 * sizeof(float));
    alloc(&w.p0, n3 * sizeof(float));
    alloc(&w.p1, n3 * sizeof(float));
    alloc(&w.r, n3 * sizeof(float));
    alloc(&w.Ap, n3 * sizeof(float));
    alloc(&w.partials, 2 * 256 * 4 * sizeof(double));
    alloc(&w.counter, sizeof(unsigned long long));
    alloc(&w.res_partials, (size_t)2 * ir_residual_blocks(p->n) * sizeof(double));
    alloc(&w.ticket, sizeof(unsigned));
    alloc(&w.state, 8 * sizeof(int));
    alloc(&w.dx_init, n3 * sizeof(float));
    alloc(&w.best, sizeof(double));
    alloc(&w.stats, (size_t)p->max_stats * sizeof(IrStats));
    alloc(&w.scale, 2 * sizeof(float));
    // a plan on the persistent factor PCG runs its inner solves there, on a
    // copy of the 16-bit blocks padded to 20 bytes (4-byte aligned loads)
    const bool persistent = (p->pl.variant == PcgLayout::kFactor || p->ir_pl.variant == PcgLayout::kFactor) &&
                            p->cfg.preconditioner >= 1;
    if (!refined32 && persistent) alloc(&w.hq_words, nz * 5 * sizeof(uint32_t));
    // ... and the whole refinement in one launch there, with the iterate
    // as hi / lo planes padded like the PCG's exchanged vectors
    if (persistent) {
        alloc(&w.xf_hi, (size_t)p->pw.n_pad * 3 * sizeof(float));
        alloc(&w.xf_lo, (size_t)p->pw.n_pad * 3 * sizeof(float));
    }
    int max_ctas = 1;
    if (e == cudaSuccess) e = ir_max_ctas(p->device, &max_ctas);
    if (e == cudaSuccess) e = cudaMemset(w.counter, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(w.ticket, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(w.state, 0, 8 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(w.stats, 0, (size_t)p->max_stats * sizeof(IrStats));
    if (e == cudaSuccess) e = cudaMemset(w.e, 0, n3 * sizeof(float));
    if (e == cudaSuccess && w.xf_hi) e = cudaMemset(w.xf_hi, 0, (size_t)p->pw.n_pad * 3 * sizeof(float));
    if (e == cudaSuccess && w.xf_lo) e = cudaMemset(w.xf_lo, 0, (size_t)p->pw.n_pad * 3 * sizeof(float));
    if (e != cudaSuccess) {
        for (void *a : p->ir_allocs) cudaFree(a);
        p->ir_allocs.clear();
        return cuda_fail(p, e, "mixed-precision buffers");
    }
    w.ctas = std::max(1, std::min(max_ctas, (p->n + 63) / 64));
    p->ir = w;
    return MFEM_OK;
}

int mfem_step_mixed_stats(mfem_plan *p, mfem_mixed_solve_stats *h_stats, int32_t max_entries, int32_t *count,
                          mfem_stream stream) {
    static_assert(sizeof(mfem_mixed_solve_stats) == sizeof(IrStats), "stats layout");
    if (!p || (max_entries > 0 && !h_stats)) return MFEM_BAD_ARG;
    if (p->ir.mode == 0) {
        if (count) *count = 0;
        return MFEM_OK;
    }
    DeviceGuard g(p->device);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamSynchronize");
    const int k = std::max(0, std::min<int>(max_entries, p->cfg.iterations));
    std::vector<IrStats> tmp(p->max_stats);
    e = cudaMemcpy(tmp.data(), p->ir.stats, sizeof(IrStats) * p->max_stats, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p, e, "stats readback");
    for (int i = 0; i < k; ++i) std::memcpy(&h_stats[i], &tmp[i], sizeof(IrStats));
    if (count) *count = k;
    return MFEM_OK;
}

int mfem_plan_set_diagnostics(mfem_plan *p, int32_t on) {
    if (!p) return MFEM_BAD_ARG;
    DeviceGuard g(p->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaDeviceSynchronize");
    if ((on != 0) != p->diagnostics) {
        for (auto &ge : p->graphs) {
            if (ge.exec) cudaGraphExecDestroy(ge.exec);
            ge = mfem_plan::GraphEntry{};
        }
    }
    p->diagnostics = on != 0;
    return MFEM_OK;
}

int mfem_plan_inject_timeout(mfem_plan *p) {
    if (!p) return MFEM_BAD_ARG;
    DeviceGuard g(p->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaDeviceSynchronize");
    const int one = 1;
    e = cudaMemcpy(p->pw.error, &one, sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(p, e, "setting the error flag");
    return MFEM_OK;
}

int mfem_plan_set_residual_check(mfem_plan *p, int32_t on) {
    if (!p) return MFEM_BAD_ARG;
    DeviceGuard g(p->device);
    cudaError_t e = cudaDeviceSynchronize();  // no step of this plan may still run the old graphs
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaDeviceSynchronize");
    if (on && !p->check_resid) {
        void *raw = nullptr;
        e = cudaMalloc(&raw, (size_t)2 * p->max_stats * sizeof(double));
        if (e != cudaSuccess) return cuda_fail(p, e, "residual check buffer");
        p->allocs.push_back(raw);
        p->check_resid = static_cast<double *>(raw);
        e = cudaMemset(raw, 0, (size_t)2 * p->max_stats * sizeof(double));
        if (e != cudaSuccess) return cuda_fail(p, e, "residual check buffer");
    }
    if ((on != 0) != p->check_on) {
        for (auto &ge : p->graphs) {
            if (ge.exec) cudaGraphExecDestroy(ge.exec);
            ge = mfem_plan::GraphEntry{};
        }
    }
    p->check_on = on != 0;
    return MFEM_OK;
}

int mfem_step_true_residuals(mfem_plan *p, double *h_rel, int32_t max_entries, int32_t *count, mfem_stream stream) {
    if (!p || (max_entries > 0 && !h_rel)) return MFEM_BAD_ARG;
    if (!p->check_on || !p->check_resid) return fail(p, MFEM_BAD_ARG, "the residual check is off");
    DeviceGuard g(p->device);
    const int m = std::min<int>(std::max(0, max_entries), std::min(p->max_stats, p->cfg.iterations));
    std::vector<double> buf((size_t)2 * std::max(1, m));
    cudaError_t e = cudaSuccess;
    if (m > 0)
        e = cudaMemcpyAsync(buf.data(), p->check_resid, (size_t)2 * m * sizeof(double), cudaMemcpyDeviceToHost,
                            (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(p, e, "step true residuals");
    for (int i = 0; i < m; ++i)
        h_rel[i] = buf[2 * i + 1] > 0.0 ? std::sqrt(buf[2 * i] / buf[2 * i + 1]) : std::sqrt(buf[2 * i]);
    if (count) *count = m;
    return MFEM_OK;
}

}  // extern "C"

namespace {

// Uploads a schedule for `threads` threads per CTA and a group-barrier cost
// of `c0` block products (batch_schedule), with the plan's iteration
// estimates per body.
int apply_batch_layout(mfem_plan *p, int threads, double c0, int max_group) {
    int capacity = 0;
    cudaError_t e = batch_capacity(p->device, threads, p->cfg.preconditioner >= 2, &capacity);
    if (e != cudaSuccess) return cuda_fail(p, e, "batch capacity");
    if (capacity < 1) return fail(p, MFEM_CUDA_ERROR, "the batched PCG does not fit on an SM");
    std::vector<int> task_ptr;
    std::vector<int4> tasks;
    int ctas = 0;
    if (p->h_body_its.size() != p->h_body_nnzb.size()) p->h_body_its.assign(p->h_body_nnzb.size(), 1);
    batch_schedule(p->h_body_nnzb, p->h_body_its, capacity, c0, std::max(1, max_group), task_ptr, tasks, ctas);
    // the previous schedule's arrays: every caller has synchronised the
    // device, so no launch still reads them
    for (void *a : p->layout_allocs) cudaFree(a);
    p->layout_allocs.clear();
    int *d_ptr = nullptr;
    int4 *d_task = nullptr;
    float *partials = nullptr;
    e = cudaMalloc(&d_ptr, task_ptr.size() * sizeof(int));
    if (e == cudaSuccess) p->layout_allocs.push_back(d_ptr);
    if (e == cudaSuccess) e = cudaMalloc(&d_task, tasks.size() * sizeof(int4));
    if (e == cudaSuccess) p->layout_allocs.push_back(d_task);
    if (e == cudaSuccess) e = cudaMalloc(&partials, (size_t)2 * ctas * 4 * sizeof(float));
    if (e == cudaSuccess) p->layout_allocs.push_back(partials);
    if (e == cudaSuccess) e = upload(d_ptr, task_ptr.data(), task_ptr.size());
    if (e == cudaSuccess) e = upload(d_task, tasks.data(), tasks.size());
    // a group's barrier base is its counter rounded down to the group size,
    // so the counters restart with every schedule (group sizes change)
    if (e == cudaSuccess) e = cudaMemset(p->bw.counter, 0, (size_t)p->bw.n_bodies * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(p, e, "batch schedule");
    p->bw.task_ptr = d_ptr;
    p->bw.task = d_task;
    p->bw.partials = partials;
    p->bw.ctas = ctas;
    p->bw.threads = threads;
    p->bw_max_group = max_group;
    p->bw_c0 = c0;
    return MFEM_OK;
}

void drop_graphs(mfem_plan *p) {
    for (auto &ge : p->graphs) {
        if (ge.exec) cudaGraphExecDestroy(ge.exec);
        ge = mfem_plan::GraphEntry{};
    }
}

}  // namespace

// Installs validated bodies: per-body rows, energies and gravity (null
// energy / gravity: the plan's, for the one-body batch of a mesh too large for
// the shared-memory PCG), the per-body work arrays and a first schedule.
int install_bodies(mfem_plan *p, int n_bodies, const int32_t *voff, const int32_t *toff, const int32_t *energy,
                   const float *gravity) {
    std::vector<int32_t> vb, nnzb(n_bodies, 0);
    std::vector<unsigned char> code;
    if (gravity) {
        vb.resize(p->n);
        for (int b = 0; b < n_bodies; ++b)
            for (int v = voff[b]; v < voff[b + 1]; ++v) vb[v] = b;
    }
    if (energy) {
        code.resize(p->T);
        for (int b = 0; b < n_bodies; ++b)
            for (int t = toff[b]; t < toff[b + 1]; ++t) code[t] = (unsigned char)energy[b];
    }
    for (int b = 0; b < n_bodies; ++b) nnzb[b] = p->h_row_ptr[voff[b + 1]] - p->h_row_ptr[voff[b]];
    DeviceGuard g(p->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaDeviceSynchronize");
    drop_graphs(p);
    for (void *a : p->batch_allocs) cudaFree(a);
    p->batch_allocs.clear();
    p->bw = BatchViews{};
    p->tv.energy_code = nullptr;
    p->vv.vertex_body = nullptr;
    p->vv.body_gravity = nullptr;
    p->h_body_row.assign(voff, voff + n_bodies + 1);
    p->h_body_nnzb = nnzb;
    p->h_body_its.assign(n_bodies, 1);
    const size_t n3 = (size_t)p->n * 3;
    auto alloc = [&](auto **ptr, size_t bytes) {
        if (e != cudaSuccess) return;
        void *raw = nullptr;
        e = cudaMalloc(&raw, std::max<size_t>(bytes, 16));
        if (e == cudaSuccess) {
            p->batch_allocs.push_back(raw);
            *ptr = static_cast<std::remove_reference_t<decltype(*ptr)>>(raw);
        }
    };
    int *body_row = nullptr, *vbody = nullptr;
    unsigned char *ecode = nullptr;
    float *grav = nullptr;
    BatchViews &bw = p->bw;
    alloc(&body_row, (size_t)(n_bodies + 1) * sizeof(int));
    if (gravity) {
        alloc(&vbody, (size_t)p->n * sizeof(int));
        alloc(&grav, (size_t)n_bodies * 3 * sizeof(float));
    }
    if (energy) alloc(&ecode, (size_t)p->T);
    alloc(&bw.counter, (size_t)n_bodies * sizeof(unsigned long long));
    alloc(&bw.z, n3 * sizeof(float));
    alloc(&bw.p0, n3 * sizeof(float));
    alloc(&bw.p1, n3 * sizeof(float));
    alloc(&bw.r, n3 * sizeof(float));
    alloc(&bw.Ap, n3 * sizeof(float));
    alloc(&bw.stats, (size_t)p->max_stats * n_bodies * sizeof(SolveStats));
    if (p->cfg.preconditioner >= 2) {
        // factor preconditioner: H's lower block pattern (columns <= row) and
        // its transpose as two CSRs; the pattern of tets is symmetric, so
        // the upper CSR's row i lists the rows j >= i whose lower part holds
        // column i, in ascending order
        const int n = p->n;
        std::vector<int32_t> lrow(n + 1, 0), lcol, urow(n + 1, 0), ucol, umap;
        for (int r = 0; r < n; ++r) {
            for (int k = p->h_row_ptr[r]; k < p->h_row_ptr[r + 1]; ++k)
                if (p->h_col_idx[k] <= r) lcol.push_back(p->h_col_idx[k]);
            lrow[r + 1] = (int32_t)lcol.size();
        }
        const size_t nnzl = lcol.size();
        for (size_t l = 0; l < nnzl; ++l) ++urow[lcol[l] + 1];
        for (int r = 0; r < n; ++r) urow[r + 1] += urow[r];
        ucol.assign(nnzl, 0);
        umap.assign(nnzl, 0);
        std::vector<int32_t> fill(urow.begin(), urow.end() - 1);
        for (int r = 0; r < n; ++r)  // rows ascending: each upper row fills in column order
            for (int l = lrow[r]; l < lrow[r + 1]; ++l) {
                const int u = fill[lcol[l]]++;
                ucol[u] = r;
                umap[u] = l;
            }
        int *d_lrow = nullptr, *d_lcol = nullptr, *d_urow = nullptr, *d_ucol = nullptr, *d_umap = nullptr;
        alloc(&d_lrow, (size_t)(n + 1) * sizeof(int));
        alloc(&d_urow, (size_t)(n + 1) * sizeof(int));
        alloc(&d_lcol, nnzl * sizeof(int));
        alloc(&d_ucol, nnzl * sizeof(int));
        alloc(&d_umap, nnzl * sizeof(int));
        alloc(&bw.Lval, nnzl * 9 * sizeof(float));
        alloc(&bw.Uval, nnzl * 9 * sizeof(float));
        alloc(&bw.Lb, nnzl * kFactorLd * sizeof(__nv_bfloat16));
        alloc(&bw.Ub, nnzl * kFactorLd * sizeof(__nv_bfloat16));
        alloc(&bw.y, n3 * sizeof(float));
        alloc(&bw.dx0, n3 * sizeof(float));
        if (p->cfg.preconditioner == 2) {
            // the H slot of every pair of a row's lower columns (FSAI setup)
            std::vector<int64_t> pptr(n + 1, 0);
            std::vector<int32_t> pairs;
            for (int r = 0; r < n; ++r) {
                const int m = lrow[r + 1] - lrow[r];
                if (m <= kFsaiMaxCols)
                    for (int a = 0; a < m; ++a) {
                        const int ca = lcol[lrow[r] + a];
                        const int32_t *b0 = p->h_col_idx.data() + p->h_row_ptr[ca];
                        const int32_t *b1 = p->h_col_idx.data() + p->h_row_ptr[ca + 1];
                        for (int b = 0; b <= a; ++b) {
                            const int32_t *q = std::lower_bound(b0, b1, lcol[lrow[r] + b]);
                            pairs.push_back(q != b1 && *q == lcol[lrow[r] + b] ? (int32_t)(q - p->h_col_idx.data())
                                                                               : -1);
                        }
                    }
                pptr[r + 1] = (int64_t)pairs.size();
            }
            // rows the register kernel does not take (more than 8 lower blocks)
            std::vector<int32_t> big;
            for (int r = 0; r < n; ++r)
                if (lrow[r + 1] - lrow[r] > 8) big.push_back(r);
            int64_t *d_pptr = nullptr;
            int *d_pairs = nullptr, *d_big = nullptr;
            alloc(&d_pptr, pptr.size() * sizeof(int64_t));
            alloc(&d_pairs, pairs.size() * sizeof(int));
            alloc(&d_big, big.size() * sizeof(int));
            if (e == cudaSuccess) e = upload(d_pptr, pptr.data(), pptr.size());
            if (e == cudaSuccess) e = upload(d_pairs, pairs.data(), pairs.size());
            if (e == cudaSuccess) e = upload(d_big, big.data(), big.size());
            bw.fsai_pair_ptr = d_pptr;
            bw.fsai_pairs = d_pairs;
            bw.fsai_big_rows = d_big;
            bw.n_fsai_big = (int)big.size();
        }
        if (e == cudaSuccess) e = upload(d_lrow, lrow.data(), lrow.size());
        if (e == cudaSuccess) e = upload(d_urow, urow.data(), urow.size());
        if (e == cudaSuccess) e = upload(d_lcol, lcol.data(), nnzl);
        if (e == cudaSuccess) e = upload(d_ucol, ucol.data(), nnzl);
        if (e == cudaSuccess) e = upload(d_umap, umap.data(), nnzl);
        if (e == cudaSuccess) e = cudaMemset(bw.Lval, 0, nnzl * 9 * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(bw.Uval, 0, nnzl * 9 * sizeof(float));
        bw.lrow = d_lrow;
        bw.lcol = d_lcol;
        bw.urow = d_urow;
        bw.ucol = d_ucol;
        bw.umap = d_umap;
        bw.nnzl = (int)nnzl;
    }
    if (e == cudaSuccess) e = upload(body_row, voff, (size_t)n_bodies + 1);
    if (e == cudaSuccess && gravity) e = upload(vbody, vb.data(), vb.size());
    if (e == cudaSuccess && gravity) e = upload(grav, gravity, (size_t)n_bodies * 3);
    if (e == cudaSuccess && energy && p->T > 0) e = upload(ecode, code.data(), code.size());
    if (e == cudaSuccess) e = cudaMemset(bw.counter, 0, (size_t)n_bodies * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(bw.stats, 0, (size_t)p->max_stats * n_bodies * sizeof(SolveStats));
    if (e != cudaSuccess) {
        for (void *a : p->batch_allocs) cudaFree(a);
        p->batch_allocs.clear();
        p->bw = BatchViews{};
        return cuda_fail(p, e, "batch buffers");
    }
    bw.n_bodies = n_bodies;
    bw.body_row = body_row;
    p->tv.energy_code = ecode;
    p->vv.vertex_body = vbody;
    p->vv.body_gravity = grav;
    // one body: one 512-thread CTA per SM, like the persistent PCG; many
    // bodies: the work-weighted schedule, groups as large as helps
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
    const int rc = n_bodies == 1 ? apply_batch_layout(p, 512, 2048.0, std::max(1, sms))
                                 : apply_batch_layout(p, 256, 2048.0, INT_MAX);
    if (rc != MFEM_OK) {
        for (void *a : p->batch_allocs) cudaFree(a);
        p->batch_allocs.clear();
        p->bw = BatchViews{};
        p->tv.energy_code = nullptr;
        p->vv.vertex_body = nullptr;
        p->vv.body_gravity = nullptr;
    }
    return rc;
}

extern "C" {

int mfem_plan_set_bodies(mfem_plan *p, int32_t n_bodies, const int32_t *h_vertex_offsets,
                         const int32_t *h_tet_offsets, const int32_t *h_body_energy, const float *h_body_gravity) {
    if (!p) return MFEM_BAD_ARG;
    if (n_bodies < 1 || !h_vertex_offsets || !h_tet_offsets || !h_body_energy || !h_body_gravity)
        return fail(p, MFEM_BAD_ARG, "need n_bodies >= 1 and every array");
    if (p->cfg.line_search && n_bodies > 1)
        return fail(p, MFEM_BAD_ARG, "batched bodies run the plain update: create the plan with line_search = 0");
    if (p->ir.mode != 0) return fail(p, MFEM_BAD_ARG, "batched bodies use the fp32 PCG");
    if (h_vertex_offsets[0] != 0 || h_vertex_offsets[n_bodies] != p->n || h_tet_offsets[0] != 0 ||
        h_tet_offsets[n_bodies] != p->T)
        return fail(p, MFEM_BAD_ARG, "body offsets must start at 0 and end at n / T");
    for (int b = 0; b < n_bodies; ++b) {
        if (h_vertex_offsets[b + 1] <= h_vertex_offsets[b] || h_tet_offsets[b + 1] < h_tet_offsets[b])
            return fail(p, MFEM_BAD_ARG, "body offsets must increase (every body needs a vertex)");
        if (h_body_energy[b] != MFEM_ENERGY_ARAP && h_body_energy[b] != MFEM_ENERGY_NEOHOOKEAN)
            return fail(p, MFEM_BAD_ARG, "unknown body energy");
        for (int i = 0; i < 3; ++i)
            if (!std::isfinite(h_body_gravity[3 * b + i])) return fail(p, MFEM_BAD_ARG, "non-finite body gravity");
        for (int t = h_tet_offsets[b]; t < h_tet_offsets[b + 1]; ++t)
            for (int k = 0; k < 4; ++k) {
                const int v = p->h_tets[4 * (size_t)t + k];
                if (v < h_vertex_offsets[b] || v >= h_vertex_offsets[b + 1])
                    return fail(p, MFEM_BAD_ARG, "tet " + std::to_string(t) + " uses a vertex of another body");
            }
    }
    if (p->pl.variant == PcgLayout::kFactor) {
        // per-body solves run in the global-memory PCG
        p->pl.variant = 0;
        p->pl.cache_matrix = 0;
        p->pl.smem = 0;
    }
    return install_bodies(p, n_bodies, h_vertex_offsets, h_tet_offsets, h_body_energy, h_body_gravity);
}

int mfem_plan_set_factor_net(mfem_plan *p, const float *h_params, int64_t n_params, const float *h_vertex_static) {
    if (!p) return MFEM_BAD_ARG;
    if (p->cfg.preconditioner != 3)
        return fail(p, MFEM_BAD_ARG, "the factor net needs a plan created with preconditioner = 3");
    if (!h_params || n_params != MFEM_FACTOR_NET_PARAMS)
        return fail(p, MFEM_BAD_ARG, "need MFEM_FACTOR_NET_PARAMS parameters");
    if (!h_vertex_static && p->n > 0) return fail(p, MFEM_BAD_ARG, "h_vertex_static is NULL");
    for (int64_t i = 0; i < n_params; ++i)
        if (!std::isfinite(h_params[i])) return fail(p, MFEM_BAD_ARG, "non-finite net parameter");
    for (int64_t i = 0; i < (int64_t)p->n * 4; ++i)
        if (!std::isfinite(h_vertex_static[i])) return fail(p, MFEM_BAD_ARG, "non-finite static vertex feature");
    constexpr int W = kNetWidth;
    // unpack in the documented order
    const float *q = h_params;
    auto take = [&](int64_t count) {
        const float *r = q;
        q += count;
        return r;
    };
    const float *w_in = take(W * kNetIn), *b_in = take(W);
    const float *w_mp[3], *b_mp[3];
    for (int l = 0; l < 3; ++l) {
        w_mp[l] = take(W * 2 * W);
        b_mp[l] = take(W);
    }
    const float *w_d = take(6 * W), *b_d = take(6), *w_p = take(W * W), *b_p = take(W), *w_q = take(W * W);
    const float *w_r = take(W * 9), *w_o = take(9 * W), *b_o = take(9);
    auto bf = [](float v) { return __float2bfloat16_rn(v); };
    std::vector<float> h_w_in(W * kNetIn);
    for (int i = 0; i < W * kNetIn; ++i) h_w_in[i] = __bfloat162float(bf(w_in[i]));
    const __nv_bfloat16 zero = bf(0.0f);
    std::vector<__nv_bfloat16> h_mp[3];
    for (int l = 0; l < 3; ++l) {
        h_mp[l].assign((size_t)W * kMpLd, zero);
        for (int o = 0; o < W; ++o)
            for (int k = 0; k < 2 * W; ++k) h_mp[l][(size_t)o * kMpLd + k] = bf(w_mp[l][o * 2 * W + k]);
    }
    std::vector<__nv_bfloat16> h_node((size_t)kNodeOut * kNodeLd, zero);
    std::vector<float> h_bnode(kNodeOut, 0.0f);
    for (int o = 0; o < W; ++o) {
        for (int k = 0; k < W; ++k) {
            h_node[(size_t)o * kNodeLd + k] = bf(w_p[o * W + k]);
            h_node[(size_t)(W + o) * kNodeLd + k] = bf(w_q[o * W + k]);
        }
        h_bnode[o] = b_p[o];
    }
    for (int o = 0; o < 6; ++o) {
        for (int k = 0; k < W; ++k) h_node[(size_t)(2 * W + o) * kNodeLd + k] = bf(w_d[o * W + k]);
        h_bnode[2 * W + o] = b_d[o];
    }
    std::vector<__nv_bfloat16> h_r((size_t)W * kRLd, zero), h_o((size_t)16 * kNodeLd, zero);
    std::vector<float> h_bo(16, 0.0f);
    for (int o = 0; o < W; ++o)
        for (int k = 0; k < 9; ++k) h_r[(size_t)o * kRLd + k] = bf(w_r[o * 9 + k]);
    for (int o = 0; o < 9; ++o) {
        for (int k = 0; k < W; ++k) h_o[(size_t)o * kNodeLd + k] = bf(w_o[o * W + k]);
        h_bo[o] = b_o[o];
    }
    // lower pattern: H slot of each lower block, and the off-diagonal ones
    std::vector<int32_t> lslot, erow, elow;
    for (int r = 0; r < p->n; ++r)
        for (int k = p->h_row_ptr[r]; k < p->h_row_ptr[r + 1]; ++k) {
            const int c = p->h_col_idx[k];
            if (c > r) continue;
            if (c < r) {
                erow.push_back(r);
                elow.push_back((int32_t)lslot.size());
            }
            lslot.push_back(k);
        }
    DeviceGuard g(p->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaDeviceSynchronize");
    drop_graphs(p);
    for (void *a : p->net_allocs) cudaFree(a);
    p->net_allocs.clear();
    p->fv = FactorNetViews{};
    FactorNetViews fv{};
    const size_t n = (size_t)p->n;
    auto put = [&](auto **dst, const auto *src, size_t count) {
        if (e != cudaSuccess) return;
        void *raw = nullptr;
        const size_t bytes = std::max<size_t>(count * sizeof(**dst), 16);
        e = cudaMalloc(&raw, bytes);
        if (e != cudaSuccess) return;
        p->net_allocs.push_back(raw);
        if (src && count) e = cudaMemcpy(raw, src, count * sizeof(**dst), cudaMemcpyHostToDevice);
        *dst = static_cast<std::remove_reference_t<decltype(*dst)>>(raw);
    };
    const float *nf = nullptr;
    const __nv_bfloat16 *nb = nullptr;
    put(&fv.w_in, h_w_in.data(), h_w_in.size());
    put(&fv.b_in, b_in, W);
    for (int l = 0; l < 3; ++l) {
        put(&fv.w_mp[l], h_mp[l].data(), h_mp[l].size());
        put(&fv.b_mp[l], b_mp[l], W);
    }
    put(&fv.w_node, h_node.data(), h_node.size());
    put(&fv.b_node, h_bnode.data(), h_bnode.size());
    put(&fv.w_r, h_r.data(), h_r.size());
    put(&fv.w_o, h_o.data(), h_o.size());
    put(&fv.b_o, h_bo.data(), h_bo.size());
    put(&fv.vstatic, h_vertex_static, n * 4);
    put(&fv.s, nf, n);
    put(&fv.ld, nf, n);
    put(&fv.w, nf, (size_t)p->nnzb);
    put(&fv.winv, nf, n);
    put(&fv.h, nf, n * W);
    put(&fv.hb[0], nb, n * W);
    put(&fv.hb[1], nb, n * W);
    put(&fv.pb, nb, n * W);
    put(&fv.qb, nb, n * W);
    put(&fv.lslot, lslot.data(), lslot.size());
    put(&fv.erow, erow.data(), erow.size());
    put(&fv.elow, elow.data(), elow.size());
    if (e != cudaSuccess) {
        for (void *a : p->net_allocs) cudaFree(a);
        p->net_allocs.clear();
        return cuda_fail(p, e, "factor net buffers");
    }
    fv.n_edges = (int)erow.size();
    fv.ready = 1;
    p->fv = fv;
    return MFEM_OK;
}

int mfem_plan_batch_layout(const mfem_plan *p, int32_t *ctas, int32_t *threads) {
    if (!p) return MFEM_BAD_ARG;
    if (ctas) *ctas = p->bw.ctas;
    if (threads) *threads = p->bw.threads;
    return MFEM_OK;
}

int mfem_plan_autotune_batch(mfem_plan *p, const float *d_q, float dt, double *h_best_ms, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    if (p->bw.n_bodies == 0) return fail(p, MFEM_BAD_ARG, "no bodies: call mfem_plan_set_bodies first");
    if (p->pl.variant == PcgLayout::kFactor)
        return fail(p, MFEM_BAD_ARG, "the plan runs the persistent factor PCG: nothing to tune");
    if (!d_q || !(dt > 0.0f)) return fail(p, MFEM_BAD_ARG, "need q and dt > 0");
    if (!net_ready(p)) return fail(p, MFEM_BAD_ARG, "preconditioner 3 needs mfem_plan_set_factor_net");
    DeviceGuard g(p->device);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t es = cudaStreamSynchronize(s);
    if (es != cudaSuccess) return cuda_fail(p, es, "cudaStreamSynchronize");
    drop_graphs(p);  // captured steps point at the schedule arrays replaced below
    // one system at q (at rest), solved from the same warm start by every
    // candidate layout
    float *x = nullptr, *dx0 = nullptr;
    const size_t bytes = (size_t)p->n * 3 * sizeof(float);
    cudaError_t e = cudaMalloc(&x, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dx0, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(dx0, 0, bytes, s);
    if (e == cudaSuccess) e = launch_predict(d_q, dx0, x, p->gravity, dt, p->vv, s);
    if (e == cudaSuccess) e = launch_element(x, p->cfg.energy, p->tv, p->diagnostics, s);
    if (e == cudaSuccess) e = contact_and_assemble(p, x, dt, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx0, p->vv.dx, bytes, cudaMemcpyDeviceToDevice, s);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    // per-body iteration counts of this system weight the schedules
    if (e == cudaSuccess) e = global_solve(p, 0, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) {
        std::vector<SolveStats> st(p->bw.n_bodies);
        e = cudaMemcpy(st.data(), p->bw.stats, st.size() * sizeof(SolveStats), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) {
            p->h_body_its.resize(st.size());
            for (size_t b = 0; b < st.size(); ++b) p->h_body_its[b] = std::max(1, st[b].iterations + 1);
        }
    }
    const int threads_opts[3] = {128, 256, 512};
    const double c0_opts[3] = {512.0, 2048.0, 8192.0};
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device);
    // group caps for one body: unbounded, and 2, 1, 1/2 and 1/4 CTAs per
    // SM; many bodies keep unbounded groups (a capped schedule timed best on
    // the tuning system but not along trajectories)
    const int group_opts[5] = {INT_MAX, 2 * sms, sms, std::max(1, sms / 2), std::max(1, sms / 4)};
    const int n_caps = p->bw.n_bodies == 1 ? 5 : 1;
    int best_t = p->bw.threads, best_g = p->bw_max_group;
    double best_m = p->bw_c0;
    float best = 1e30f;
    std::vector<std::vector<int4>> tried;
    for (int cand = 0; e == cudaSuccess && cand < 3 * 3 * n_caps; ++cand) {
        const int threads = threads_opts[cand / (3 * n_caps)], cap = group_opts[cand % n_caps];
        const double c0 = c0_opts[(cand / n_caps) % 3];
        // skip a schedule already timed (c0 and the cap often do not change it)
        int capacity = 0;
        if (batch_capacity(p->device, threads, p->cfg.preconditioner >= 2, &capacity) != cudaSuccess ||
            capacity < 1)
            continue;
        std::vector<int> tp;
        std::vector<int4> tk;
        int nc = 0;
        batch_schedule(p->h_body_nnzb, p->h_body_its, capacity, c0, cap, tp, tk, nc);
        tk.push_back(make_int4(threads, nc, 0, 0));
        bool seen = false;
        for (const auto &t : tried) {
            seen = t.size() == tk.size();
            for (size_t q = 0; seen && q < t.size(); ++q)
                seen = t[q].x == tk[q].x && t[q].y == tk[q].y && t[q].z == tk[q].z && t[q].w == tk[q].w;
            if (seen) break;
        }
        if (seen) continue;
        tried.push_back(std::move(tk));
        const int rc = apply_batch_layout(p, threads, c0, cap);
        if (rc != MFEM_OK) {
            e = cudaErrorUnknown;
            break;
        }
        float ms = 0.0f;
        int flag = 0;
        for (int rep = 0; e == cudaSuccess && rep < 2; ++rep) {
            e = cudaMemcpyAsync(p->vv.dx, dx0, bytes, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = cudaEventRecord(e0, s);
            if (e == cudaSuccess) e = global_solve(p, 0, s);
            if (e == cudaSuccess) e = cudaEventRecord(e1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        }
        if (e == cudaSuccess) e = cudaMemcpy(&flag, p->pw.error, sizeof(int), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && flag) {
            // a wait gave up: this schedule is not a candidate
            e = rearm_barriers(p);
            continue;
        }
        if (e == cudaSuccess && ms < best) {
            best = ms;
            best_t = threads;
            best_m = c0;
            best_g = cap;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (x) cudaFree(x);
    if (dx0) cudaFree(dx0);
    if (e != cudaSuccess) return cuda_fail(p, e, "autotune");
    drop_graphs(p);
    const int rc = apply_batch_layout(p, best_t, best_m, best_g);
    if (rc == MFEM_OK && h_best_ms) *h_best_ms = best;
    return rc;
}

int mfem_step_body_stats(mfem_plan *p, mfem_solve_stats *h_stats, int32_t max_entries, int32_t *count,
                         mfem_stream stream) {
    if (!p || (max_entries > 0 && !h_stats)) return MFEM_BAD_ARG;
    const int B = p->bw.n_bodies;
    if (B == 0) {
        if (count) *count = 0;
        return MFEM_OK;
    }
    DeviceGuard g(p->device);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamSynchronize");
    const int k = std::max(0, std::min<int>(max_entries, p->cfg.iterations * B));
    std::vector<SolveStats> tmp((size_t)p->max_stats * B);
    e = cudaMemcpy(tmp.data(), p->bw.stats, tmp.size() * sizeof(SolveStats), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p, e, "stats readback");
    for (int i = 0; i < k; ++i) std::memcpy(&h_stats[i], &tmp[i], sizeof(mfem_solve_stats));
    if (count) *count = k;
    int flag = 0;
    e = cudaMemcpy(&flag, p->pw.error, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p, e, "stats readback");
    if (flag) {
        e = rearm_barriers(p);
        if (e != cudaSuccess) return cuda_fail(p, e, "re-arming the grid barriers");
        return fail(p, MFEM_TIMEOUT, "a batched PCG barrier timed out");
    }
    return MFEM_OK;
}

int mfem_step_line_search_stats(mfem_plan *p, mfem_line_search_stats *h_stats, int32_t max_entries, int32_t *count,
                           mfem_stream stream) {
    static_assert(sizeof(mfem_line_search_stats) == sizeof(LineSearchStats), "stats layout");
    if (!p || (max_entries > 0 && !h_stats)) return MFEM_BAD_ARG;
    DeviceGuard g(p->device);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(p, e, "cudaStreamSynchronize");
    const int k = std::max(0, std::min<int>(max_entries, p->cfg.iterations));
    std::vector<LineSearchStats> tmp(p->max_stats);
    e = cudaMemcpy(tmp.data(), p->ls.stats, sizeof(LineSearchStats) * p->max_stats, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(p, e, "stats readback");
    for (int i = 0; i < k; ++i) std::memcpy(&h_stats[i], &tmp[i], sizeof(mfem_line_search_stats));
    if (count) *count = k;
    return MFEM_OK;
}

int mfem_predict(mfem_plan *p, const float *q, const float *qd, float dt, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    if (!q || !qd) return fail(p, MFEM_BAD_ARG, "NULL state pointer");
    DeviceGuard g(p->device);
    // the predictor also snapshots x and copies it to q_out; pass x_start as
    // the output so the caller's q is left untouched
    cudaError_t e = launch_predict(q, qd, p->vv.x_start, p->gravity, dt, p->vv, (cudaStream_t)stream);
    if (e == cudaSuccess) e = launch_contact_begin(p->cv, p->vv, (cudaStream_t)stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "predict");
}

int mfem_update_system(mfem_plan *p, const float *x, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    if (!x) return fail(p, MFEM_BAD_ARG, "x is NULL");
    DeviceGuard g(p->device);
    cudaError_t e = launch_element(x, p->cfg.energy, p->tv, p->diagnostics, (cudaStream_t)stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "update_system");
}

int mfem_assemble(mfem_plan *p, const float *x, float dt, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    if (!net_ready(p)) return fail(p, MFEM_BAD_ARG, "preconditioner 3 needs mfem_plan_set_factor_net");
    if (!x) return fail(p, MFEM_BAD_ARG, "x is NULL");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(p, MFEM_BAD_ARG, "dt must be finite and > 0");
    DeviceGuard g(p->device);
    cudaError_t e = contact_and_assemble(p, x, dt, (cudaStream_t)stream);
    p->stage_dt = dt;
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "assemble");
}

int mfem_global_solve(mfem_plan *p, int32_t slot, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    if (slot < 0 || slot >= p->max_stats) return fail(p, MFEM_BAD_ARG, "stats slot out of range");
    DeviceGuard g(p->device);
    cudaError_t e = global_solve(p, slot, (cudaStream_t)stream);
    p->stage_slot = slot;
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "global_solve");
}

int mfem_local_solve(mfem_plan *p, float *x, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    if (!x) return fail(p, MFEM_BAD_ARG, "x is NULL");
    if (p->cfg.line_search && !(p->stage_dt > 0.0f))
        return fail(p, MFEM_BAD_ARG, "the line search needs mfem_assemble (its dt) first");
    DeviceGuard g(p->device);
    cudaError_t e = local_update(p, x, p->stage_dt, p->stage_slot, (cudaStream_t)stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "local_solve");
}

int mfem_true_residual(mfem_plan *p, double *h_rel, mfem_stream stream) {
    if (!p || !h_rel) return MFEM_BAD_ARG;
    DeviceGuard g(p->device);
    cudaError_t e = launch_true_residual(p->bv, p->vv, p->resid, (cudaStream_t)stream);
    double out[2] = {0.0, 0.0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, p->resid, sizeof(out), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(p, e, "true_residual");
    *h_rel = out[1] > 0.0 ? std::sqrt(out[0] / out[1]) : std::sqrt(out[0]);
    return MFEM_OK;
}

}  // extern "C"

// ---- adaptive refinement -------------------------------------------------

namespace {

// Per-edge and per-vertex tet lists of the plan's mesh in ascending tet
// order, each tet's and tri's edge slots, and the work arrays of a pass.
int refine_prepare(mfem_plan *p) {
    if (p->refine_ready) return MFEM_OK;
    for (void *a : p->refine_allocs) cudaFree(a);
    p->refine_allocs.clear();
    p->refine_tmass_cap = 0;
    const int n = p->n, T = p->T, m = p->n_tris;
    const int64_t nnzb = p->nnzb;
    std::vector<int32_t> slot_row(nnzb), tet_edge((size_t)T * 6), tri_edge((size_t)m * 3);
    for (int r = 0; r < n; ++r)
        for (int k = p->h_row_ptr[r]; k < p->h_row_ptr[r + 1]; ++k) slot_row[k] = r;
    static const int pi[6] = {1, 2, 2, 3, 3, 3}, pj[6] = {0, 0, 1, 0, 1, 2};
    for (int t = 0; t < T; ++t) {
        const int32_t *v = p->h_tets.data() + 4 * (size_t)t;
        const int32_t *sl = p->h_tet_slots.data() + 16 * (size_t)t;
        for (int q = 0; q < 6; ++q) {
            const int i = pi[q], j = pj[q];
            tet_edge[6 * (size_t)t + q] = v[i] < v[j] ? sl[4 * i + j] : sl[4 * j + i];
        }
    }
    auto slot_of = [&](int a, int b) -> int32_t {
        if (a > b) std::swap(a, b);
        const int32_t *lo = p->h_col_idx.data() + p->h_row_ptr[a], *hi = p->h_col_idx.data() + p->h_row_ptr[a + 1];
        const int32_t *it = std::lower_bound(lo, hi, b);
        return (it != hi && *it == b) ? (int32_t)(it - p->h_col_idx.data()) : -1;
    };
    for (int t = 0; t < m; ++t) {
        const int32_t *v = p->h_tris.data() + 3 * (size_t)t;
        for (int q = 0; q < 3; ++q) {
            const int32_t s = slot_of(v[pi[q]], v[pj[q]]);
            if (s < 0) return fail(p, MFEM_BAD_ARG, "a contact tri joins vertices that share no tet");
            tri_edge[3 * (size_t)t + q] = s;
        }
    }
    // counting sorts keep ascending tet order within each edge and vertex
    std::vector<int32_t> edge_start(nnzb + 1, 0), edge_tet((size_t)T * 6);
    for (size_t i = 0; i < tet_edge.size(); ++i) edge_start[tet_edge[i] + 1]++;
    for (int64_t s = 0; s < nnzb; ++s) edge_start[s + 1] += edge_start[s];
    {
        std::vector<int32_t> fill(edge_start.begin(), edge_start.end() - 1);
        for (int t = 0; t < T; ++t)
            for (int q = 0; q < 6; ++q) edge_tet[fill[tet_edge[6 * (size_t)t + q]]++] = t;
    }
    std::vector<int32_t> vert_start(n + 1, 0), vert_code((size_t)T * 4);
    for (size_t i = 0; i < (size_t)T * 4; ++i) vert_start[p->h_tets[i] + 1]++;
    for (int v = 0; v < n; ++v) vert_start[v + 1] += vert_start[v];
    {
        std::vector<int32_t> fill(vert_start.begin(), vert_start.end() - 1);
        for (int t = 0; t < T; ++t)
            for (int k = 0; k < 4; ++k) vert_code[fill[p->h_tets[4 * (size_t)t + k]]++] = 4 * t + k;
    }
    DeviceGuard g(p->device);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto **ptr, size_t count) {
        if (e != cudaSuccess) return;
        void *raw = nullptr;
        e = cudaMalloc(&raw, std::max<size_t>(count, 1) * sizeof(**ptr));
        if (e == cudaSuccess) {
            p->refine_allocs.push_back(raw);
            *ptr = static_cast<std::remove_reference_t<decltype(*ptr)>>(raw);
        }
    };
    RefineViews rv{};
    int32_t *d_slot_row = nullptr, *d_tet_edge = nullptr, *d_tri_edge = nullptr, *d_es = nullptr, *d_et = nullptr,
            *d_vs = nullptr, *d_vc = nullptr;
    alloc(&d_slot_row, nnzb);
    alloc(&d_tet_edge, (size_t)T * 6);
    alloc(&d_tri_edge, (size_t)m * 3);
    alloc(&d_es, nnzb + 1);
    alloc(&d_et, (size_t)T * 6);
    alloc(&d_vs, n + 1);
    alloc(&d_vc, (size_t)T * 4);
    alloc(&rv.e_tet, T);
    alloc(&rv.dens, T);
    alloc(&rv.lmax, T);
    alloc(&rv.vscore, n);
    alloc(&rv.vdist, n);
    alloc(&rv.vsid, n);
    alloc(&rv.tdist, m);
    alloc(&rv.tbary, (size_t)m * 3);
    alloc(&rv.tenergy, m);
    const int stat_blocks = std::max(1, (T + 255) / 256);
    alloc(&rv.partials, stat_blocks);
    alloc(&rv.mean_density, 1);
    alloc(&rv.score, nnzb);
    alloc(&rv.state, nnzb);
    alloc(&rv.blocked, nnzb);
    alloc(&rv.cand, T);
    alloc(&rv.split_slot, T);
    alloc(&rv.split_pair, T);
    alloc(&rv.tet_cnt, (size_t)T + 1);
    alloc(&rv.edge_cnt, nnzb + 1);
    alloc(&rv.tri_slot, m);
    alloc(&rv.tri_cnt, (size_t)m + 1);
    const int64_t longest = std::max<int64_t>({(int64_t)T, nnzb, (int64_t)m});
    rv.scan_tmp_len = (longest + 1023) / 1024 + 2;
    alloc(&rv.scan_tmp, rv.scan_tmp_len);
    alloc(&rv.ctrl, kRefineCtrl);
    if (e == cudaSuccess) e = upload(d_slot_row, slot_row.data(), nnzb);
    if (e == cudaSuccess) e = upload(d_tet_edge, tet_edge.data(), tet_edge.size());
    if (e == cudaSuccess) e = upload(d_tri_edge, tri_edge.data(), tri_edge.size());
    if (e == cudaSuccess) e = upload(d_es, edge_start.data(), edge_start.size());
    if (e == cudaSuccess) e = upload(d_et, edge_tet.data(), edge_tet.size());
    if (e == cudaSuccess) e = upload(d_vs, vert_start.data(), vert_start.size());
    if (e == cudaSuccess) e = upload(d_vc, vert_code.data(), vert_code.size());
    if (e == cudaSuccess) e = cudaMemset(rv.split_pair, 0, std::max<size_t>(T, 1) * sizeof(int));
    if (e != cudaSuccess) {
        for (void *a : p->refine_allocs) cudaFree(a);
        p->refine_allocs.clear();
        return cuda_fail(p, e, "refinement buffers");
    }
    rv.n = n;
    rv.T = T;
    rv.m = m;
    rv.nnzb = nnzb;
    rv.energy = p->cfg.energy;
    rv.tets = p->tv.tets;
    rv.dminv = p->tv.dminv;
    rv.materials = p->tv.materials;
    rv.stretch = p->tv.stretch;
    rv.lambda = p->tv.lambda;
    rv.rest = p->rest_q;
    rv.mass = p->mass;
    rv.inv_mass = p->inv_mass;
    rv.tris = p->cv.tris;
    rv.col_idx = p->bv.col_idx;
    rv.slot_row = d_slot_row;
    rv.tet_edge = d_tet_edge;
    rv.tri_edge = d_tri_edge;
    rv.edge_start = d_es;
    rv.edge_tet = d_et;
    rv.vert_start = d_vs;
    rv.vert_code = d_vc;
    p->rv = rv;
    p->refine_ready = true;
    return MFEM_OK;
}

bool finite_all(std::initializer_list<float> v) {
    for (float x : v)
        if (!std::isfinite(x)) return false;
    return true;
}

}  // namespace

extern "C" {

void mfem_refine_config_default(mfem_refine_config *cfg) {
    if (!cfg) return;
    *cfg = mfem_refine_config{};
    cfg->scoring = MFEM_REFINE_LEGACY;
    cfg->threshold = 10.1f;
    cfg->tet_score_weight = 0.0f;
    cfg->vertex_score_weight = 0.1f;
    cfg->penetrating_edge_score = 1.0e6f;
    cfg->min_edge_length = 0.1f;
    cfg->contact_d1 = 0.1f;
    cfg->elastic_weight = 1.0f;
    cfg->vertex_contact_weight = 1.0f;
    cfg->tri_contact_weight = 1.0f;
    cfg->split_position = 0.5f;
    cfg->density = 1.0f;
    cfg->conflict_iterations = 5;
    cfg->refine_every = 10;
}

int mfem_refine(mfem_plan *p, const mfem_refine_config *cfg_in, const mfem_refine_inputs *inputs, float *d_q,
                float *d_qd, int32_t *d_pass_counter, const mfem_refine_mesh *out, mfem_stream stream) {
    if (!p) return MFEM_BAD_ARG;
    mfem_refine_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else mfem_refine_config_default(&cfg);
    if (!d_q || !d_qd || !out) return fail(p, MFEM_BAD_ARG, "mfem_refine: q, qd and out are required");
    if (cfg.scoring != MFEM_REFINE_LEGACY && cfg.scoring != MFEM_REFINE_GEOMETRIC)
        return fail(p, MFEM_BAD_ARG, "mfem_refine: unknown scoring");
    if (!finite_all({cfg.threshold, cfg.tet_score_weight, cfg.vertex_score_weight, cfg.penetrating_edge_score,
                     cfg.min_edge_length, cfg.contact_d1, cfg.elastic_weight, cfg.vertex_contact_weight,
                     cfg.tri_contact_weight, cfg.split_position, cfg.density}))
        return fail(p, MFEM_BAD_ARG, "mfem_refine: non-finite setting");
    if (cfg.scoring == MFEM_REFINE_GEOMETRIC && !(cfg.min_edge_length > 0.0f && cfg.contact_d1 > 0.0f))
        return fail(p, MFEM_BAD_ARG, "mfem_refine: geometric scoring needs min_edge_length > 0 and contact_d1 > 0");
    if (!(cfg.density > 0.0f)) return fail(p, MFEM_BAD_ARG, "mfem_refine: density must be > 0");
    if (cfg.conflict_iterations < 0 || cfg.conflict_iterations > 1000 || cfg.refine_every < 0)
        return fail(p, MFEM_BAD_ARG, "mfem_refine: conflict_iterations in [0, 1000], refine_every >= 0");
    if (p->bw.n_bodies > 1) return fail(p, MFEM_BAD_ARG, "mfem_refine: plans with several bodies are not refined");
    if (out->max_particles < p->n || out->max_tets < p->T || out->max_tris < p->n_tris)
        return fail(p, MFEM_BAD_ARG, "mfem_refine: the output capacities are below the plan's mesh");
    if (!out->tet_indices || !out->tet_poses || !out->tet_materials || !out->tet_stretch || !out->tet_lambda ||
        !out->rest_q || !out->particle_mass || !out->particle_inv_mass || !out->counts ||
        (p->n_tris > 0 && !out->tri_indices))
        return fail(p, MFEM_BAD_ARG, "mfem_refine: NULL output array");
    int rc = refine_prepare(p);
    if (rc != MFEM_OK) return rc;
    DeviceGuard g(p->device);
    cudaError_t e = cudaSuccess;
    if (out->max_tets > p->refine_tmass_cap) {
        float *tm = nullptr;
        e = cudaMalloc(&tm, (size_t)std::max(out->max_tets, 1) * sizeof(float));
        if (e != cudaSuccess) return cuda_fail(p, e, "mfem_refine: cudaMalloc");
        if (p->rv.tmass) {
            // a pass still in flight may read the old array
            cudaError_t se = cudaStreamSynchronize((cudaStream_t)stream);
            if (se != cudaSuccess) {
                cudaFree(tm);
                return cuda_fail(p, se, "mfem_refine: cudaStreamSynchronize");
            }
            auto it = std::find(p->refine_allocs.begin(), p->refine_allocs.end(), (void *)p->rv.tmass);
            if (it != p->refine_allocs.end()) p->refine_allocs.erase(it);
            cudaFree(p->rv.tmass);
        }
        p->refine_allocs.push_back(tm);
        p->rv.tmass = tm;
        p->refine_tmass_cap = out->max_tets;
    }
    RefineViews rv = p->rv;
    if (inputs) {
        rv.tet_scores = inputs->tet_scores;
        rv.vertex_scores = inputs->vertex_scores;
        rv.particle_distance = inputs->particle_distance;
        rv.particle_shape_id = inputs->particle_shape_id;
        rv.tri_distance = inputs->tri_distance;
        rv.tri_bary = inputs->tri_bary;
    }
    if (cfg.scoring == MFEM_REFINE_GEOMETRIC && (!rv.tri_distance) != (!rv.tri_bary))
        return fail(p, MFEM_BAD_ARG, "mfem_refine: give both tri_distance and tri_bary, or neither");
    RefineParams rp{};
    rp.scoring = cfg.scoring;
    rp.threshold = cfg.threshold;
    rp.tet_w = cfg.tet_score_weight;
    rp.vert_w = cfg.vertex_score_weight;
    rp.pen_score = cfg.penetrating_edge_score;
    rp.min_edge = cfg.min_edge_length;
    rp.d1 = cfg.contact_d1;
    rp.el_w = cfg.elastic_weight;
    rp.vc_w = cfg.vertex_contact_weight;
    rp.tri_w = cfg.tri_contact_weight;
    rp.split_t = cfg.split_position;
    rp.density = cfg.density;
    rp.sweeps = cfg.conflict_iterations;
    rp.refine_every = cfg.refine_every;
    rp.max_particles = out->max_particles;
    rp.max_tets = out->max_tets;
    rp.max_tris = out->max_tris;
    RefineOut ro{};
    ro.tets = out->tet_indices;
    ro.poses = out->tet_poses;
    ro.materials = out->tet_materials;
    ro.stretch = out->tet_stretch;
    ro.lambda = out->tet_lambda;
    ro.rest = out->rest_q;
    ro.mass = out->particle_mass;
    ro.inv_mass = out->particle_inv_mass;
    ro.tris = out->tri_indices;
    ro.counts = out->counts;
    ro.q = d_q;
    ro.qd = d_qd;
    e = launch_refine(rv, p->cv, rp, d_pass_counter, ro, (cudaStream_t)stream);
    return e == cudaSuccess ? MFEM_OK : cuda_fail(p, e, "mfem_refine");
}

}  // extern "C"
