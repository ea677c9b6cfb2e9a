"""The learned factor's hand-written training kernels.

* mfem_train_gemm (BF16 operands staged from float32, FP32 accumulation on the
  tensor cores) against torch's float64 product of the BF16-rounded operands,
  in all four operand layouts, ragged sizes and a split K: within 1e-5 of the
  product's scale (the fp32 accumulation order is the only difference).
* mfem_train_adam against the textbook update in float64: 1e-6.
* HandGrad's loss and gradient against torch float32 autograd of the same
  loss (same probe vectors and smooth fields) on a 6x3x3 beam: the loss
  within 2e-2 and the gradient within 5e-2 relative in norm, cosine >= 0.998
  (the hand-written pass rounds every GEMM operand to BF16, autograd does not).
"""
import numpy as np
import pytest
import torch

from mfem_gb300 import beams, factor_net as F

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def bf16(t):
    return t.to(torch.bfloat16).to(torch.float64)


@pytest.mark.parametrize("M,N,K", [(64, 64, 32), (1000, 9, 64), (70, 130, 100), (64, 128, 20000), (6, 64, 5001)])
@pytest.mark.parametrize("a_trans,b_trans", [(False, False), (False, True), (True, False), (True, True)])
def test_train_gemm_matches_bf16_product(M, N, K, a_trans, b_trans):
    g = torch.Generator(device=DEV).manual_seed(M * 7 + N * 3 + K)
    A = torch.randn((K, M) if a_trans else (M, K), device=DEV, generator=g)
    B = torch.randn((N, K) if b_trans else (K, N), device=DEV, generator=g)
    tk = F.TrainKernels(DEV)
    C = tk.gemm(A, B, a_trans=a_trans, b_trans=b_trans)
    opA = bf16(A).t() if a_trans else bf16(A)
    opB = bf16(B).t() if b_trans else bf16(B)
    ref = opA @ opB
    err = (C.double() - ref).abs().max().item()
    assert err <= 1e-5 * ref.abs().max().item() * max(1.0, K / 1000.0), err
    # accumulate
    C2 = C.clone()
    tk.gemm(A, B, a_trans=a_trans, b_trans=b_trans, out=C2, accumulate=True)
    assert (C2.double() - 2 * ref).abs().max().item() <= 2e-5 * ref.abs().max().item() * max(1.0, K / 1000.0)


def test_train_adam_matches_formula():
    tk = F.TrainKernels(DEV)
    g = torch.Generator(device=DEV).manual_seed(3)
    p = torch.randn(5000, device=DEV, generator=g)
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    P, M, V = p.double().clone(), m.double().clone(), v.double().clone()
    for step in range(1, 6):
        grad = torch.randn(5000, device=DEV, generator=g)
        tk.adam(p, grad, m, v, 1e-2, step)
        G = grad.double()
        M = 0.9 * M + 0.1 * G
        V = 0.999 * V + 0.001 * G * G
        P = P - 1e-2 * (M / (1 - 0.9 ** step)) / ((V / (1 - 0.999 ** step)).sqrt() + 1e-8)
    torch.cuda.synchronize()
    assert (p.double() - P).abs().max().item() <= 1e-6


def test_hand_gradient_matches_autograd():
    mesh = beams.build_beam("nh_beam", cells=(6, 3, 3))
    rp, ci, sysl, vs = F.solver_systems(mesh, 1, seed=9, device=DEV)
    G = F.Graph(rp, ci, DEV)
    vals, rhs = sysl[3]
    vst = torch.as_tensor(vs, device=DEV)
    torch.manual_seed(0)
    net = F.FactorNet()
    with torch.no_grad():  # a trained-looking net: non-zero output layers
        for p in net.parameters():
            p.add_(0.05 * torch.randn_like(p))
    net = net.to(DEV)
    s, _, _ = F.scaled_system(G, vals)
    gen = torch.Generator(device=DEV).manual_seed(1)
    r = F.probe_vectors(G, s, rhs, 8, gen)
    smooth = torch.as_tensor(F.smooth_fields(mesh.rest_q, 4, np.random.default_rng(2)), device=DEV)
    # reference: torch float32 autograd
    lv = F.loss(net, G, vals, vst, rhs, r=r, smooth=smooth, smooth_weight=2.0)
    net.zero_grad()
    lv.backward()
    ref = torch.cat([dict(net.named_parameters())[k].grad.reshape(-1) for k, _ in F.LAYOUT])
    # hand-written
    flat = torch.as_tensor(net.pack(), device=DEV)
    grad = torch.zeros_like(flat)
    with torch.no_grad():
        hl = F.HandGrad(F.TrainKernels(DEV)).loss_and_grad(flat, grad, G, vals, vst, r, smooth, 2.0)
    assert abs(hl - float(lv)) <= 2e-2 * abs(float(lv)), (hl, float(lv))
    rel = ((grad - ref).norm() / ref.norm()).item()
    cos = (torch.dot(grad, ref) / (grad.norm() * ref.norm())).item()
    print(f"loss {hl:.5f} vs {float(lv):.5f}; gradient relative error {rel:.3e}, cosine {cos:.6f}")
    assert rel <= 5e-2 and cos >= 0.998
    # every parameter group gets a gradient
    dv = F.param_views(grad)
    for k, _ in F.LAYOUT:
        assert dv[k].abs().max().item() > 0, k
