"""Host side of the learned factor preconditioner: the packed parameter
layout agrees with the C header, packing round-trips, and the float32
reference factor has the structure the PCG relies on (lower block-triangular
on H's lower pattern, positive diagonal), on CPU."""
import re

import numpy as np
import torch

from mfem_gb300 import _lib, beams, factor_net as F


def test_param_count_matches_header():
    text = _lib.HEADER.read_text()
    m = re.search(r"#define\s+MFEM_FACTOR_NET_PARAMS\s+(\d+)", text)
    assert m and int(m.group(1)) == F.N_PARAMS == _lib.FACTOR_NET_PARAMS


def test_pack_unpack_round_trip():
    torch.manual_seed(1)
    net = F.FactorNet()
    for p in net.parameters():
        torch.nn.init.normal_(p, std=0.1)
    flat = net.pack()
    assert flat.shape == (F.N_PARAMS,)
    net2 = F.FactorNet().unpack(flat)
    np.testing.assert_array_equal(net2.pack(), flat)


def _system(cells=(4, 2, 2)):
    mesh = beams.build_beam("nh_beam", cells=cells)
    rp, ci = (np.asarray(a) for a in _host_sparsity(mesh))
    rng = np.random.default_rng(3)
    n = mesh.n
    rows = np.repeat(np.arange(n), np.diff(rp))
    # a symmetric positive definite block matrix on the pattern
    A = rng.normal(size=(ci.size, 3, 3))
    vals = np.zeros_like(A)
    for k in range(ci.size):
        r, c = rows[k], ci[k]
        if r == c:
            vals[k] = 20.0 * np.eye(3) + 0.5 * (A[k] + A[k].T)
        elif r < c:
            vals[k] = 0.3 * A[k]
    for k in range(ci.size):
        r, c = rows[k], ci[k]
        if r > c:
            kk = rp[c] + np.searchsorted(ci[rp[c]:rp[c + 1]], r)
            vals[k] = vals[kk].T
    return mesh, rp, ci, vals


def _host_sparsity(mesh):
    import ctypes
    lib = _lib.load()
    n, T = mesh.n, mesh.T
    tets = np.ascontiguousarray(mesh.tet_indices, dtype=np.int32)
    nnzb = ctypes.c_int64()
    rp = np.zeros(n + 1, dtype=np.int32)
    lib.mfem_bsr_sparsity(n, T, tets.ctypes.data_as(ctypes.c_void_p), rp.ctypes.data_as(ctypes.c_void_p),
                          None, ctypes.byref(nnzb))
    ci = np.zeros(nnzb.value, dtype=np.int32)
    lib.mfem_bsr_sparsity(n, T, tets.ctypes.data_as(ctypes.c_void_p), rp.ctypes.data_as(ctypes.c_void_p),
                          ci.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nnzb))
    return rp, ci


def test_reference_factor_structure(built_lib):
    mesh, rp, ci, vals = _system()
    torch.manual_seed(2)
    net = F.FactorNet()
    for p in net.parameters():
        torch.nn.init.normal_(p, std=0.05)
    vs = F.static_features(mesh.rest_q, mesh.tet_indices, mesh.tet_materials)
    assert vs.shape == (mesh.n, 4) and np.allclose(vs[:, 1:].mean(0), 0.0, atol=1e-6)
    L = F.reference_factor(net, rp, ci, vals, vs)
    G = F.Graph(rp, ci)
    assert L.shape == (G.nnzl, 3, 3)
    Ld = L[G.l_of_diag.numpy()]
    assert np.all(Ld[:, [0, 0, 1], [1, 2, 2]] == 0.0)      # lower-triangular diagonal blocks
    assert np.all(np.diagonal(Ld, axis1=1, axis2=2) > 0.0)  # positive diagonal
    # M = L L^T is symmetric positive definite
    n3 = 3 * mesh.n
    lrow = np.zeros(mesh.n + 1, dtype=np.int64)
    rows = np.repeat(np.arange(mesh.n), np.diff(rp))
    lmask = rows >= ci
    np.add.at(lrow, rows[lmask] + 1, 1)
    lrow = np.cumsum(lrow)
    import scipy.sparse as sp
    Ls = sp.bsr_matrix((L, ci[lmask], lrow), shape=(n3, n3)).toarray()
    M = Ls @ Ls.T
    assert np.linalg.eigvalsh(M).min() > 0.0
    # emulating BF16 changes the factor only at BF16 resolution
    L32 = F.reference_factor(net, rp, ci, vals, vs, emulate_bf16=False)
    assert np.abs(L - L32).max() <= 3e-2 * np.abs(L32).max()


def test_smooth_field_loss_term(built_lib):
    """The opt-in smooth-field term: off by default (the residual form
    alone, bit for bit), finite, larger and differentiable when on."""
    mesh, rp, ci, vals = _system()
    G = F.Graph(rp, ci)
    v = torch.as_tensor(vals, dtype=torch.float32)
    vs = torch.as_tensor(F.static_features(mesh.rest_q, mesh.tet_indices, mesh.tet_materials))
    rhs = torch.ones(mesh.n, 3)
    sm = torch.as_tensor(F.smooth_fields(mesh.rest_q, 4, np.random.default_rng(0)))
    assert sm.shape == (mesh.n, 3, 4) and torch.isfinite(sm).all() and sm.abs().max() > 0
    torch.manual_seed(4)
    net = F.FactorNet()
    g0 = torch.Generator().manual_seed(0)
    base = F.loss(net, G, v, vs, rhs, 8, g0)
    g1 = torch.Generator().manual_seed(0)
    off = F.loss(net, G, v, vs, rhs, 8, g1, sm, 0.0)
    assert torch.equal(base, off)
    g2 = torch.Generator().manual_seed(0)
    on = F.loss(net, G, v, vs, rhs, 8, g2, sm, 2.0)
    assert torch.isfinite(on) and on > base
    on.backward()
    assert all(p.grad is None or torch.isfinite(p.grad).all() for p in net.parameters())
    assert any(p.grad is not None and p.grad.abs().sum() > 0 for p in net.parameters())
