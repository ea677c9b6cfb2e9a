"""The learned factor preconditioner: a message-passing net on the vertex
graph that writes a lower block-triangular L on H's lower block pattern;
the PCG applies M = L L^T (preconditioner="learned").

The net (width 64, BF16 weights, FP32 accumulation):

* Per-vertex scale d_i = tr(H_ii) / 3 and s_i = d_i^-1/2; every quantity the
  net sees is of the scaled system S H S (S = diag(s)), and L = S L~ with L~
  the net's output, so that M = S L~ L~^T S.
* Inputs x_i (16, zero padded): the scaled diagonal block (its diagonal
  minus 1 and its three off-diagonal entries), log10 d_i minus the mean of
  log10 d over the neighbours, the incident-tet mean of log10 E minus 5, the
  rest position minus the body's centroid, and the block count of row i / 15.
* h = relu(W_in x + b_in); three layers h += relu(W_l [h, a] + b_l), with
  a_i = sum_j w_ij h_j / sum_j w_ij over the off-diagonal blocks of row i,
  w_ij = ||(S H S)_ij||_F.
* Diagonal block: o = W_d h_i + b_d, L~_ii = [[sp(o0), 0, 0], [o3, sp(o1), 0],
  [o4, o5, sp(o2)]] with sp = softplus (a positive diagonal: L is
  nonsingular, so M is symmetric positive definite whatever L's rounding).
* Off-diagonal block (i, j), j < i: z = relu(P h_i + b_p + Q h_j + R e_ij),
  e_ij = (S H S)_ij as 9 values; L~_ij = W_o z + b_o (row-major 3x3).

The device computes the GEMMs from BF16 operands: h, a, P h, Q h, e and z
are rounded to BF16 where they enter a tensor-core product, which
``reference_factor`` reproduces.

Training (``train``) minimises ||r - K M r||^2 / ||r||^2 over (K, r) pairs of
the scaled systems that this library's solver assembles along trajectories
with random initial velocities N(0, 0.1 m/s) and random gravity directions;
r is the scaled right-hand side or a random normal vector.
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Optional

import numpy as np
import torch
import torch.nn as nn

WIDTH = 64
N_IN = 16
WEIGHTS_FILE = Path(__file__).with_name("factor_net_weights.npz")

# packed parameter order of mfem_plan_set_factor_net
LAYOUT = [
    ("inp.weight", (WIDTH, N_IN)), ("inp.bias", (WIDTH,)),
    ("mp.0.weight", (WIDTH, 2 * WIDTH)), ("mp.0.bias", (WIDTH,)),
    ("mp.1.weight", (WIDTH, 2 * WIDTH)), ("mp.1.bias", (WIDTH,)),
    ("mp.2.weight", (WIDTH, 2 * WIDTH)), ("mp.2.bias", (WIDTH,)),
    ("diag.weight", (6, WIDTH)), ("diag.bias", (6,)),
    ("P.weight", (WIDTH, WIDTH)), ("P.bias", (WIDTH,)),
    ("Q.weight", (WIDTH, WIDTH)),
    ("R.weight", (WIDTH, 9)),
    ("out.weight", (9, WIDTH)), ("out.bias", (9,)),
]
N_PARAMS = sum(int(np.prod(s)) for _, s in LAYOUT)


class FactorNet(nn.Module):
    def __init__(self):
        super().__init__()
        W = WIDTH
        self.inp = nn.Linear(N_IN, W)
        self.mp = nn.ModuleList([nn.Linear(2 * W, W) for _ in range(3)])
        self.diag = nn.Linear(W, 6)
        self.P = nn.Linear(W, W)
        self.Q = nn.Linear(W, W, bias=False)
        self.R = nn.Linear(9, W, bias=False)
        self.out = nn.Linear(W, 9)
        # start from block-Jacobi-like factors: L~ = I, no off-diagonal blocks
        nn.init.zeros_(self.out.weight)
        nn.init.zeros_(self.out.bias)
        nn.init.zeros_(self.diag.weight)
        with torch.no_grad():
            self.diag.bias.zero_()
            self.diag.bias[:3] = math.log(math.e - 1.0)

    def pack(self) -> np.ndarray:
        sd = self.state_dict()
        return np.concatenate([sd[k].detach().cpu().numpy().astype(np.float32).reshape(-1) for k, _ in LAYOUT])

    def unpack(self, flat: np.ndarray) -> "FactorNet":
        flat = np.asarray(flat, dtype=np.float32).reshape(-1)
        if flat.size != N_PARAMS:
            raise ValueError(f"expected {N_PARAMS} parameters, got {flat.size}")
        sd = self.state_dict()
        o = 0
        for k, shape in LAYOUT:
            m = int(np.prod(shape))
            sd[k] = torch.as_tensor(flat[o:o + m].reshape(shape))
            o += m
        self.load_state_dict(sd)
        return self


def load_weights(path: Optional[Path] = None) -> np.ndarray:
    """The packed float32 parameters shipped with the package."""
    with np.load(path or WEIGHTS_FILE) as z:
        return z["params"].astype(np.float32)


def static_features(rest_q: np.ndarray, tets: np.ndarray, materials: np.ndarray,
                    vertex_offsets: Optional[np.ndarray] = None) -> np.ndarray:
    """[n, 4] float32: incident-tet mean of log10 E minus 5, and the rest
    position minus its body's centroid.  E = mu (3 lambda + 2 mu) / (lambda +
    mu) from the tets' Lame parameters."""
    rest = np.asarray(rest_q, dtype=np.float64)
    n = rest.shape[0]
    mu = materials[:, 0].astype(np.float64)
    lam = materials[:, 1].astype(np.float64)
    E = mu * (3.0 * lam + 2.0 * mu) / np.maximum(lam + mu, 1e-30)
    logE = np.log10(np.maximum(E, 1e-30))
    acc = np.zeros(n)
    cnt = np.zeros(n)
    tv = np.asarray(tets, dtype=np.int64).reshape(-1)
    np.add.at(acc, tv, np.repeat(logE, 4))
    np.add.at(cnt, tv, 1.0)
    out = np.zeros((n, 4), dtype=np.float64)
    out[:, 0] = np.where(cnt > 0, acc / np.maximum(cnt, 1.0), 5.0) - 5.0
    offs = np.asarray(vertex_offsets if vertex_offsets is not None else [0, n], dtype=np.int64)
    for b in range(len(offs) - 1):
        sl = slice(offs[b], offs[b + 1])
        out[sl, 1:4] = rest[sl] - rest[sl].mean(axis=0)
    return out.astype(np.float32)


# -- graph of one system ------------------------------------------------------
class Graph:
    """Index arrays of H's block pattern that the net and its loss use."""

    def __init__(self, row_ptr, col_idx, device="cpu"):
        rp = np.asarray(row_ptr, dtype=np.int64)
        ci = np.asarray(col_idx, dtype=np.int64)
        n = rp.size - 1
        rows = np.repeat(np.arange(n), np.diff(rp))
        self.n = n
        self.rows = torch.as_tensor(rows, device=device)
        self.cols = torch.as_tensor(ci, device=device)
        self.diag = torch.as_tensor(np.flatnonzero(rows == ci), device=device)
        off = np.flatnonzero(rows != ci)
        self.off = torch.as_tensor(off, device=device)
        lo = np.flatnonzero(rows > ci)
        self.lo = torch.as_tensor(lo, device=device)
        self.deg = torch.as_tensor(np.diff(rp).astype(np.float32), device=device)
        # the lower pattern (columns <= row, ascending): entry index of each
        # diagonal and off-diagonal lower block
        lmask = rows >= ci
        lidx = np.cumsum(lmask) - 1
        self.nnzl = int(lmask.sum())
        self.l_of_diag = torch.as_tensor(lidx[rows == ci], device=device)
        self.l_of_lo = torch.as_tensor(lidx[lo], device=device)


def _bf16(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).to(torch.float32)


def scaled_system(G: Graph, values: torch.Tensor):
    """(s [n], d [n], scaled blocks [nnzb, 3, 3]) of S H S: d = tr(H_ii)/3,
    s = d^-1/2 (1 where d is not positive and finite)."""
    Hd = values[G.diag]
    d = (Hd[:, 0, 0] + Hd[:, 1, 1] + Hd[:, 2, 2]) / 3.0
    ok = torch.isfinite(d) & (d > 0)
    s = torch.where(ok, torch.rsqrt(torch.where(ok, d, torch.ones_like(d))), torch.ones_like(d))
    Ks = values * (s[G.rows] * s[G.cols])[:, None, None]
    return s, d, Ks


def forward(net: FactorNet, G: Graph, values: torch.Tensor, vstatic: torch.Tensor, emulate_bf16: bool = False):
    """(s, L~ diagonal blocks [n, 3, 3], L~ off-diagonal lower blocks
    [n_lo, 3, 3]) for one system.  ``emulate_bf16`` rounds weights and GEMM
    operands as the device does."""
    r = _bf16 if emulate_bf16 else (lambda t: t)
    n = G.n
    s, d, Ks = scaled_system(G, values)
    Kd = Ks[G.diag]
    ld = torch.log10(torch.where(d > 0, d, torch.ones_like(d)))
    offr, offc = G.rows[G.off], G.cols[G.off]
    cnt = torch.zeros(n, device=values.device).index_add_(0, offr, torch.ones_like(offr, dtype=torch.float32))
    ldn = torch.zeros(n, device=values.device).index_add_(0, offr, ld[offc]) / cnt.clamp_min(1.0)
    x = torch.zeros(n, N_IN, device=values.device)
    x[:, 0] = Kd[:, 0, 0] - 1.0
    x[:, 1] = Kd[:, 1, 1] - 1.0
    x[:, 2] = Kd[:, 2, 2] - 1.0
    x[:, 3] = Kd[:, 0, 1]
    x[:, 4] = Kd[:, 0, 2]
    x[:, 5] = Kd[:, 1, 2]
    x[:, 6] = torch.where(cnt > 0, ld - ldn, torch.zeros_like(ld))
    x[:, 7:11] = vstatic
    x[:, 11] = G.deg / 15.0
    w = torch.linalg.vector_norm(Ks[G.off].reshape(-1, 9), dim=1)
    wsum = torch.zeros(n, device=values.device).index_add_(0, offr, w)
    winv = torch.where(wsum > 0, 1.0 / wsum.clamp_min(1e-30), torch.zeros_like(wsum))
    h = torch.relu(x @ r(net.inp.weight).t() + net.inp.bias)
    for lin in net.mp:
        hb = r(h)
        a = torch.zeros_like(h).index_add_(0, offr, w[:, None] * hb[offc]) * winv[:, None]
        h = h + torch.relu(torch.cat([hb, r(a)], 1) @ r(lin.weight).t() + lin.bias)
    hb = r(h)
    o = hb @ r(net.diag.weight).t() + net.diag.bias
    sp = nn.functional.softplus
    z0 = torch.zeros(n, device=values.device)
    Ld = torch.stack([torch.stack([sp(o[:, 0]), z0, z0], 1),
                      torch.stack([o[:, 3], sp(o[:, 1]), z0], 1),
                      torch.stack([o[:, 4], o[:, 5], sp(o[:, 2])], 1)], 1)
    Ph = r(hb @ r(net.P.weight).t() + net.P.bias)
    Qh = r(hb @ r(net.Q.weight).t())
    li, lj = G.rows[G.lo], G.cols[G.lo]
    e = r(Ks[G.lo].reshape(-1, 9))
    z = torch.relu(Ph[li] + Qh[lj] + e @ r(net.R.weight).t())
    Lo = (r(z) @ r(net.out.weight).t() + net.out.bias).reshape(-1, 3, 3)
    return s, Ld, Lo


def reference_factor(net: FactorNet, row_ptr, col_idx, values, vstatic, emulate_bf16: bool = True) -> np.ndarray:
    """L = S L~ on the lower pattern [nnzl, 3, 3], float64 numpy: what the
    device writes into the factor buffer."""
    G = Graph(row_ptr, col_idx)
    with torch.no_grad():
        vals = torch.as_tensor(np.asarray(values, dtype=np.float32).reshape(-1, 3, 3))
        s, Ld, Lo = forward(net, G, vals, torch.as_tensor(np.asarray(vstatic, dtype=np.float32)), emulate_bf16)
        L = torch.zeros(G.nnzl, 3, 3)
        L[G.l_of_diag] = Ld * s[:, None, None]
        L[G.l_of_lo] = Lo * s[G.rows[G.lo]][:, None, None]
    return L.numpy().astype(np.float64)


def apply_scaled_M(G: Graph, Ld, Lo, r):
    """z = L~ (L~^T r) for r [n, 3, k]."""
    li, lj = G.rows[G.lo], G.cols[G.lo]
    y = torch.einsum("nji,njk->nik", Ld, r)
    y = y.index_add(0, lj, torch.einsum("eji,ejk->eik", Lo, r[li]))
    z = torch.einsum("nij,njk->nik", Ld, y)
    return z.index_add(0, li, torch.einsum("eij,ejk->eik", Lo, y[lj]))


def apply_blocks(G: Graph, Ks, v):
    return torch.zeros_like(v).index_add_(0, G.rows, torch.einsum("kij,kjm->kim", Ks, v[G.cols]))


def smooth_fields(rest_q: np.ndarray, k: int, rng, kmax: float = 1.5) -> np.ndarray:
    """k random low-frequency vector fields [n, 3, k] over the rest positions
    (sums of sinusoids with wave vectors ~ N(0, kmax) on the unit-scaled
    body): the smooth modes that set CG's iteration count."""
    X = np.asarray(rest_q, dtype=np.float64)
    X = (X - X.min(0)) / max(float(np.ptp(X, axis=0).max()), 1e-30)
    out = np.zeros((X.shape[0], 3, k))
    for j in range(k):
        for c in range(3):
            for _ in range(3):
                kv = rng.normal(0.0, kmax, 3)
                out[:, c, j] += rng.normal() * np.sin(2.0 * np.pi * (X @ kv) + rng.uniform(0.0, 2.0 * np.pi))
    return out.astype(np.float32)


def probe_vectors(G: Graph, s, rhs, k: int, generator=None):
    """k unit vectors [n, 3, k] of the scaled system: the scaled rhs S g and
    k - 1 normal ones."""
    r = torch.randn(G.n, 3, k, device=rhs.device, generator=generator)
    r[:, :, 0] = rhs * s[:, None]
    return r / torch.linalg.vector_norm(r.reshape(-1, k), dim=0).clamp_min(1e-30)


def loss(net: FactorNet, G: Graph, values, vstatic, rhs, k: int = 8, generator=None, smooth=None,
         smooth_weight: float = 0.0, r=None):
    """||r - K M r||^2 / ||r||^2 over k vectors r (the scaled rhs and normal
    noise, or the given r), plus, with ``smooth`` fields [n, 3, k'] and
    smooth_weight > 0, that weight times ||z - M K z||^2 / ||z||^2 over the
    fields z (in the scaled system's variables): the residual form with white
    noise weights every eigenmode alike, the smooth term the low-frequency
    ones.  A torch autograd expression: the float32 reference that the
    hand-written training gradients (``HandGrad``) are checked against."""
    s, Ld, Lo = forward(net, G, values, vstatic)
    _, _, Ks = scaled_system(G, values)
    if r is None:
        r = probe_vectors(G, s, rhs, k, generator)
    k = r.shape[2]
    res = r - apply_blocks(G, Ks, apply_scaled_M(G, Ld, Lo, r))
    out = (torch.linalg.vector_norm(res.reshape(-1, k), dim=0) ** 2).mean()
    if smooth is None or smooth_weight <= 0.0:
        return out
    z = smooth / s[:, None, None]  # fields of x; the scaled system's variables are S^-1 x
    kz = z.shape[2]
    z = z / torch.linalg.vector_norm(z.reshape(-1, kz), dim=0).clamp_min(1e-30)
    e = z - apply_scaled_M(G, Ld, Lo, apply_blocks(G, Ks, z))
    return out + smooth_weight * (torch.linalg.vector_norm(e.reshape(-1, kz), dim=0) ** 2).mean()


# -- training data from this library's solver --------------------------------
def solver_systems(mesh, n_steps: int, seed: int, device: str = "cuda:0", velocity_std: float = 0.1):
    """(row_ptr, col_idx, [(H values, rhs)], static features) along a
    trajectory of ``mesh`` with random initial velocities and a random
    gravity direction (|g| = 9.81)."""
    import dataclasses
    from .model import Model
    from .solver import MixedFEMSolver
    rng = np.random.default_rng(seed)
    free = mesh.particle_inv_mass > 0
    qd = (rng.normal(0.0, velocity_std, size=(mesh.n, 3)) * free[:, None]).astype(np.float32)
    g = rng.normal(size=3)
    g = (9.81 * g / np.linalg.norm(g)).astype(np.float32)
    mesh = dataclasses.replace(mesh, qd0=qd, gravity=g)
    model = Model.from_beam(mesh, device=device)
    solver = MixedFEMSolver(model, iterations=mesh.spec.iterations, energy=mesh.spec.energy, line_search=False,
                            cg_tolerance=mesh.spec.cg_tolerance, cg_max_iterations=mesh.spec.cg_max_iterations)
    q = torch.as_tensor(mesh.q0, device=device)
    v = torch.as_tensor(qd, device=device)
    x = q.clone()
    out = []
    for _ in range(n_steps):
        solver.predict(q, v, mesh.spec.dt)
        x.copy_(q)
        for it in range(solver.iterations):
            solver.update_system(x)
            solver.assemble(x, mesh.spec.dt)
            out.append((solver.read_buffer("h_values").reshape(-1, 3, 3).clone(),
                        solver.read_buffer("rhs").reshape(-1, 3).clone()))
            solver.global_solve(it)
            solver.local_solve(x)
        v = (x - q) / mesh.spec.dt
        q = x.clone()
    rp = solver.read_buffer("row_ptr").cpu().numpy()
    ci = solver.read_buffer("col_idx").cpu().numpy()
    vs = static_features(mesh.rest_q, mesh.tet_indices, mesh.tet_materials)
    solver.close()
    return rp, ci, out, vs


# -- hand-written training: BF16 tensor-core GEMMs, manual backward, Adam --
def param_views(flat: torch.Tensor) -> dict:
    """Views of a packed [N_PARAMS] tensor by LAYOUT name."""
    out, o = {}, 0
    for k, shape in LAYOUT:
        m = int(np.prod(shape))
        out[k] = flat[o:o + m].view(shape)
        o += m
    return out


class TrainKernels:
    """The library's training kernels through its C ABI: mfem_train_gemm
    (BF16 operands, FP32 accumulation, tensor cores) and mfem_train_adam."""

    def __init__(self, device):
        from . import _lib
        self._libmod = _lib
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.ws = torch.empty(1 << 22, dtype=torch.float32, device=self.device)  # split-K partials

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"training kernel failed ({rc}): {self.lib.mfem_train_last_error().decode()}")

    def gemm(self, A, B, a_trans=False, b_trans=False, out=None, accumulate=False):
        """op(A) op(B): op(A) = A [M, K] or A^T (A [K, M]); op(B) = B [K, N]
        or B^T (B [N, K])."""
        import ctypes
        A = A.contiguous()
        B = B.contiguous()
        M, K = (A.shape[1], A.shape[0]) if a_trans else (A.shape[0], A.shape[1])
        N = B.shape[0] if b_trans else B.shape[1]
        if (B.shape[1] if b_trans else B.shape[0]) != K:
            raise ValueError(f"inner dimensions differ: {tuple(A.shape)} {tuple(B.shape)}")
        if out is None:
            out = torch.empty(M, N, dtype=torch.float32, device=self.device)
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        self._check(self.lib.mfem_train_gemm(M, N, K, P(A), A.shape[1], int(a_trans), P(B), B.shape[1],
                                             int(b_trans), P(out), out.shape[1], int(accumulate), P(self.ws),
                                             self.ws.numel(), stream))
        return out

    def linear(self, x, W, b=None):
        y = self.gemm(x, W, b_trans=True)
        return y + b if b is not None else y

    def adam(self, params, grads, m, v, lr, step, beta1=0.9, beta2=0.999, eps=1e-8):
        import ctypes
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        self._check(self.lib.mfem_train_adam(P(params), P(grads), P(m), P(v), params.numel(), float(lr), beta1,
                                             beta2, eps, int(step), stream))


def net_inputs(G: Graph, Ks, d, vstatic):
    """The 16 per-vertex inputs of the net (as ``forward``)."""
    n = G.n
    Kd = Ks[G.diag]
    ld = torch.log10(torch.where(d > 0, d, torch.ones_like(d)))
    offr, offc = G.rows[G.off], G.cols[G.off]
    cnt = torch.zeros(n, device=Ks.device).index_add_(0, offr, torch.ones_like(offr, dtype=torch.float32))
    ldn = torch.zeros(n, device=Ks.device).index_add_(0, offr, ld[offc]) / cnt.clamp_min(1.0)
    x = torch.zeros(n, N_IN, device=Ks.device)
    x[:, 0] = Kd[:, 0, 0] - 1.0
    x[:, 1] = Kd[:, 1, 1] - 1.0
    x[:, 2] = Kd[:, 2, 2] - 1.0
    x[:, 3] = Kd[:, 0, 1]
    x[:, 4] = Kd[:, 0, 2]
    x[:, 5] = Kd[:, 1, 2]
    x[:, 6] = torch.where(cnt > 0, ld - ldn, torch.zeros_like(ld))
    x[:, 7:11] = vstatic
    x[:, 11] = G.deg / 15.0
    return x


def _apply_LT(G: Graph, Ld, Lo, r):
    """L~^T r for r [n, 3, k]."""
    li, lj = G.rows[G.lo], G.cols[G.lo]
    t = torch.einsum("nji,njk->nik", Ld, r)
    return t.index_add(0, lj, torch.einsum("eji,ejk->eik", Lo, r[li]))


def _apply_L(G: Graph, Ld, Lo, t):
    """L~ t for t [n, 3, k]."""
    li, lj = G.rows[G.lo], G.cols[G.lo]
    y = torch.einsum("nij,njk->nik", Ld, t)
    return y.index_add(0, li, torch.einsum("eij,ejk->eik", Lo, t[lj]))


class HandGrad:
    """Loss and gradient of the factor net written out by hand: the forward
    pass keeps what the backward pass needs, every dense product (forward,
    input gradient, weight gradient) runs on the library's BF16 tensor-core
    GEMM, and the graph operations (gathers, scatter-adds, block products of
    the loss) are explicit adjoints.  No autograd is involved."""

    def __init__(self, kernels: TrainKernels):
        self.tk = kernels

    def forward(self, P: dict, G: Graph, values, vstatic):
        tk = self.tk
        s, d, Ks = scaled_system(G, values)
        x = net_inputs(G, Ks, d, vstatic)
        offr, offc = G.rows[G.off], G.cols[G.off]
        w = torch.linalg.vector_norm(Ks[G.off].reshape(-1, 9), dim=1)
        wsum = torch.zeros(G.n, device=values.device).index_add_(0, offr, w)
        winv = torch.where(wsum > 0, 1.0 / wsum.clamp_min(1e-30), torch.zeros_like(wsum))
        u = tk.linear(x, P["inp.weight"], P["inp.bias"])
        h = torch.relu(u)
        c = dict(x=x, m_in=u > 0, w=w, winv=winv, cats=[], masks=[])
        for layer in range(3):
            a = torch.zeros_like(h).index_add_(0, offr, w[:, None] * h[offc]) * winv[:, None]
            cat = torch.cat([h, a], 1)
            u = tk.linear(cat, P[f"mp.{layer}.weight"], P[f"mp.{layer}.bias"])
            h = h + torch.relu(u)
            c["cats"].append(cat)
            c["masks"].append(u > 0)
        o = tk.linear(h, P["diag.weight"], P["diag.bias"])
        sp = nn.functional.softplus
        z0 = torch.zeros(G.n, device=values.device)
        Ld = torch.stack([torch.stack([sp(o[:, 0]), z0, z0], 1),
                          torch.stack([o[:, 3], sp(o[:, 1]), z0], 1),
                          torch.stack([o[:, 4], o[:, 5], sp(o[:, 2])], 1)], 1)
        li, lj = G.rows[G.lo], G.cols[G.lo]
        e = Ks[G.lo].reshape(-1, 9)
        v = (tk.linear(h, P["P.weight"], P["P.bias"])[li] + tk.linear(h, P["Q.weight"])[lj] +
             tk.linear(e, P["R.weight"]))
        z = torch.relu(v)
        Lo = tk.linear(z, P["out.weight"], P["out.bias"]).reshape(-1, 3, 3)
        c.update(h=h, o=o, e=e, z=z, m_z=v > 0)
        return s, Ks, Ld, Lo, c

    def loss_and_grad(self, flat, grad, G: Graph, values, vstatic, r, smooth=None, smooth_weight: float = 0.0):
        """The loss of ``loss`` (same r, same smooth fields) and its gradient
        by the packed parameters, written into ``grad`` [N_PARAMS]."""
        tk = self.tk
        P, dP = param_views(flat), param_views(grad)
        s, Ks, Ld, Lo, c = self.forward(P, G, values, vstatic)
        li, lj = G.rows[G.lo], G.cols[G.lo]
        dLd = torch.zeros_like(Ld)
        dLo = torch.zeros_like(Lo)

        # residual form: res = r - K L~ L~^T r
        k = r.shape[2]
        t = _apply_LT(G, Ld, Lo, r)
        y = _apply_L(G, Ld, Lo, t)
        res = r - apply_blocks(G, Ks, y)
        total = (torch.linalg.vector_norm(res.reshape(-1, k), dim=0) ** 2).mean()
        dy = -apply_blocks(G, Ks, (2.0 / k) * res)  # K is symmetric
        pairs = [(dy, t, r)]
        if smooth is not None and smooth_weight > 0.0:
            zf = smooth / s[:, None, None]
            kz = zf.shape[2]
            zf = zf / torch.linalg.vector_norm(zf.reshape(-1, kz), dim=0).clamp_min(1e-30)
            q = apply_blocks(G, Ks, zf)
            t2 = _apply_LT(G, Ld, Lo, q)
            err = zf - _apply_L(G, Ld, Lo, t2)
            total = total + smooth_weight * (torch.linalg.vector_norm(err.reshape(-1, kz), dim=0) ** 2).mean()
            pairs.append((-(2.0 * smooth_weight / kz) * err, t2, q))
        # y = L~ t with t = L~^T q: dL~ = dy t^T + q (L~^T dy)^T on the pattern
        for dyy, tt, qq in pairs:
            dt = _apply_LT(G, Ld, Lo, dyy)
            dLd += torch.einsum("nik,njk->nij", dyy, tt) + torch.einsum("nik,njk->nij", qq, dt)
            dLo += torch.einsum("eik,ejk->eij", dyy[li], tt[lj]) + torch.einsum("eik,ejk->eij", qq[li], dt[lj])
        # diagonal blocks from o (softplus on the diagonal)
        o = c["o"]
        do = torch.stack([dLd[:, 0, 0] * torch.sigmoid(o[:, 0]), dLd[:, 1, 1] * torch.sigmoid(o[:, 1]),
                          dLd[:, 2, 2] * torch.sigmoid(o[:, 2]), dLd[:, 1, 0], dLd[:, 2, 0], dLd[:, 2, 1]], 1)
        h = c["h"]
        # off-diagonal blocks: Lo = W_o z + b_o, z = relu(P h_i + b_p + Q h_j + R e)
        dLo9 = dLo.reshape(-1, 9)
        dP["out.bias"].copy_(dLo9.sum(0))
        tk.gemm(dLo9, c["z"], a_trans=True, out=dP["out.weight"])
        dv = tk.gemm(dLo9, P["out.weight"]) * c["m_z"]
        dPh = torch.zeros(G.n, WIDTH, device=h.device).index_add_(0, li, dv)
        dQh = torch.zeros(G.n, WIDTH, device=h.device).index_add_(0, lj, dv)
        tk.gemm(dv, c["e"], a_trans=True, out=dP["R.weight"])
        dP["P.bias"].copy_(dPh.sum(0))
        tk.gemm(dPh, h, a_trans=True, out=dP["P.weight"])
        tk.gemm(dQh, h, a_trans=True, out=dP["Q.weight"])
        dP["diag.bias"].copy_(do.sum(0))
        tk.gemm(do, h, a_trans=True, out=dP["diag.weight"])
        dh = tk.gemm(dPh, P["P.weight"])
        tk.gemm(dQh, P["Q.weight"], out=dh, accumulate=True)
        tk.gemm(do, P["diag.weight"], out=dh, accumulate=True)
        # message-passing layers, last first: h' = h + relu(W [h, a] + b), a = A h
        offr, offc = G.rows[G.off], G.cols[G.off]
        w, winv = c["w"], c["winv"]
        for layer in reversed(range(3)):
            du = dh * c["masks"][layer]
            dP[f"mp.{layer}.bias"].copy_(du.sum(0))
            tk.gemm(du, c["cats"][layer], a_trans=True, out=dP[f"mp.{layer}.weight"])
            dcat = tk.gemm(du, P[f"mp.{layer}.weight"])
            da = dcat[:, WIDTH:] * winv[:, None]
            dh = dh + dcat[:, :WIDTH]
            dh = dh.index_add(0, offc, w[:, None] * da[offr])
        du = dh * c["m_in"]
        dP["inp.bias"].copy_(du.sum(0))
        tk.gemm(du, c["x"], a_trans=True, out=dP["inp.weight"])
        return float(total)


def train(meshes, pairs: int = 2000, r_per_system: int = 8, epochs: int = 12, seed: int = 5,
          device: str = "cuda:0", log=print, smooth_weight: float = 0.0, lr: float = 2e-3,
          init: Optional[np.ndarray] = None) -> FactorNet:
    """Trains on about ``pairs`` (K, r) pairs: pairs / r_per_system systems
    drawn along trajectories of ``meshes``; smooth_weight > 0 adds the
    smooth-field term of ``loss`` (8 fields a system).  The gradient is
    ``HandGrad``'s and the update the library's Adam kernel, with a cosine
    learning-rate schedule over the epochs; ``init`` starts from packed
    parameters (default: FactorNet's block-Jacobi-like start)."""
    torch.manual_seed(seed)
    systems = []
    per_mesh = max(1, pairs // r_per_system // len(meshes))
    for m_i, mesh in enumerate(meshes):
        its = mesh.spec.iterations
        steps = max(1, (per_mesh + its - 1) // its)
        rp, ci, sysl, vs = solver_systems(mesh, steps, seed + 17 * m_i, device)
        G = Graph(rp, ci, device)
        vst = torch.as_tensor(vs, device=device)
        frng = np.random.default_rng(seed + 31 * m_i)
        for vals, rhs in sysl[:per_mesh]:
            sm = (torch.as_tensor(smooth_fields(mesh.rest_q, 8, frng), device=device)
                  if smooth_weight > 0 else None)
            systems.append((G, vals, vst, rhs, sm))
        log(f"mesh {mesh.spec.name} {mesh.spec.cells}: {min(per_mesh, len(sysl))} systems")
    start = FactorNet().pack() if init is None else np.asarray(init, dtype=np.float32)
    flat = torch.as_tensor(start, device=device).clone()
    grad = torch.zeros_like(flat)
    m1 = torch.zeros_like(flat)
    m2 = torch.zeros_like(flat)
    hg = HandGrad(TrainKernels(device))
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    step = 0
    with torch.no_grad():
        for ep in range(epochs):
            lr_ep = 0.5 * lr * (1.0 + math.cos(math.pi * ep / epochs))
            perm = np.random.default_rng(seed + ep).permutation(len(systems))
            tot = 0.0
            for i in perm:
                G, vals, vst, rhs, sm = systems[i]
                s, _, _ = scaled_system(G, vals)
                r = probe_vectors(G, s, rhs, r_per_system, gen)
                tot += hg.loss_and_grad(flat, grad, G, vals, vst, r, sm, smooth_weight)
                step += 1
                hg.tk.adam(flat, grad, m1, m2, lr_ep, step)
            log(f"epoch {ep}: loss {tot / len(systems):.4f}")
    return FactorNet().unpack(flat.cpu().numpy())


def main(argv=None):
    import argparse
    from . import beams
    ap = argparse.ArgumentParser(description="train the learned factor preconditioner")
    ap.add_argument("--out", default=str(WEIGHTS_FILE))
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--device", default="cuda:0")
    ap.add_argument("--smooth-weight", type=float, default=0.0,
                    help="weight of the smooth-field term of the loss (0: the residual form only)")
    ap.add_argument("--lr", type=float, default=2e-3, help="peak Adam learning rate (cosine schedule)")
    ap.add_argument("--init", default=None,
                    help="start from these packed weights (.npz, 'shipped' for the package's) instead of "
                         "the block-Jacobi-like start")
    ap.add_argument("--seed", type=int, default=5)
    args = ap.parse_args(argv)
    meshes = [beams.build_beam("nh_beam"), beams.build_beam("stiff_beam")]
    init = None
    if args.init:
        init = load_weights(None if args.init == "shipped" else Path(args.init))
    net = train(meshes, pairs=args.pairs, epochs=args.epochs, device=args.device, smooth_weight=args.smooth_weight,
                lr=args.lr, init=init, seed=args.seed)
    np.savez(args.out, params=net.pack())
    print(f"wrote {args.out} ({N_PARAMS} parameters)")


if __name__ == "__main__":
    main()
