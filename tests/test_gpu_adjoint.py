"""Differentiable batched QR on the GPU: forward against the oracle's tile QR,
adjoint against the CPU FP64 reference adjoint and central differences.

Forward: Q, R and the packed factor of every problem match the oracle's
flat-tree tile QR (NextLA's geqrt!/tsqrt!, same Householder signs) within
1e-12 n relative.  Backward: Abar matches the reference pullback
(Walter & Lehmann) evaluated in FP64 on the CPU, and the directional
derivative <Abar, E> matches central differences (h = 1e-6) of
f(A) = 1/2 ||R^-1 Q^T b - y||^2 + <dQ, Q> + <dR, R> evaluated with the
GPU forward.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(2048, 256), (600, 100), (256, 256), (300, 17), (40, 40), (1, 1), (513, 255)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def batch_inputs(batch, m, n, seed, torch):
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn((batch, m, n), generator=g, dtype=torch.float64, device="cuda")
    b = torch.randn((batch, m), generator=g, dtype=torch.float64, device="cuda")
    y = torch.randn((batch, n), generator=g, dtype=torch.float64, device="cuda")
    dQ = torch.randn((batch, m, n), generator=g, dtype=torch.float64, device="cuda")
    dR = torch.randn((batch, n, n), generator=g, dtype=torch.float64, device="cuda")
    return A, b, y, dQ, dR


def loss_torch(Q, R, b, y, dQ, dR, torch):
    c = torch.einsum("bmn,bm->bn", Q, b)
    x = torch.linalg.solve_triangular(R, c.unsqueeze(-1), upper=True).squeeze(-1)
    return 0.5 * ((x - y) ** 2).sum() + (dQ * Q).sum() + (dR * torch.triu(R)).sum()


@pytest.mark.parametrize("m,n", SHAPES)
def test_forward_matches_oracle(tq, oracle, m, n):
    import torch
    from tileqr import autodiff as AD
    batch = 3
    A, *_ = batch_inputs(batch, m, n, 1, torch)
    Q, R, F, tau = AD.qr_forward(A, 32)
    torch.cuda.synchronize()
    for p in range(batch):
        Qo, Ro, Fo = oracle.qr_explicit(A[p].cpu().numpy(), 256, 32)
        assert rel(R[p].cpu().numpy(), Ro) <= 1e-12 * n
        assert rel(Q[p].cpu().numpy(), Qo) <= 1e-12 * n
        assert rel(F[p].cpu().numpy(), Fo) <= 1e-12 * n
    # A is left untouched
    A2, *_ = batch_inputs(batch, m, n, 1, torch)
    assert torch.equal(A, A2)


@pytest.mark.parametrize("m,n", SHAPES)
def test_backward_matches_reference_adjoint(tq, oracle, m, n):
    import torch
    from tileqr import autodiff as AD
    batch = 3
    A, b, y, dQ, dR = batch_inputs(batch, m, n, 2, torch)
    Q, R, F, tau = AD.qr_forward(A, 32)
    Qh, Rh = Q.cpu().numpy(), R.cpu().numpy()
    Qb = np.empty((batch, m, n))
    Rb = np.empty((batch, n, n))
    for p in range(batch):
        _, Qb[p], Rb[p] = oracle.ls_loss_cotangents(Qh[p], Rh[p], b[p].cpu().numpy(), y[p].cpu().numpy(),
                                                    dQ[p].cpu().numpy(), dR[p].cpu().numpy())
    Abar = AD.qr_backward(F, tau, torch.from_numpy(Qb).cuda(), torch.from_numpy(Rb).cuda(), 32)
    Ah = Abar.cpu().numpy()
    for p in range(batch):
        Qo, Ro, _ = oracle.qr_explicit(A[p].cpu().numpy(), 256, 32)
        ref = oracle.qr_adjoint(Qo, Ro, Qb[p], Rb[p])
        kappa = np.linalg.cond(Ro)
        assert rel(Ah[p], ref) <= 1e-13 * n * kappa, (p, rel(Ah[p], ref), kappa)


def test_autograd_rule_and_central_differences(tq, oracle):
    import torch
    from tileqr import autodiff as AD
    batch, m, n = 4, 2048, 256
    A, b, y, dQ, dR = batch_inputs(batch, m, n, 3, torch)
    Ar = A.clone().requires_grad_(True)
    Q, R = AD.qr(Ar)
    f = loss_torch(Q, R, b, y, dQ, dR, torch)
    f.backward()
    G = Ar.grad.detach()
    # autograd's cotangents through the rule equal the oracle's hand-derived ones
    Qh, Rh = Q.detach().cpu().numpy(), R.detach().cpu().numpy()
    for p in range(batch):
        _, Qb, Rb = oracle.ls_loss_cotangents(Qh[p], Rh[p], b[p].cpu().numpy(), y[p].cpu().numpy(),
                                              dQ[p].cpu().numpy(), dR[p].cpu().numpy())
        Qo, Ro, _ = oracle.qr_explicit(A[p].cpu().numpy(), 256, 32)
        ref = oracle.qr_adjoint(Qo, Ro, Qb, Rb)
        assert rel(G[p].cpu().numpy(), ref) <= 1e-10
    # central differences of the GPU forward along random directions
    g = torch.Generator(device="cuda").manual_seed(11)
    h = 1e-6
    with torch.no_grad():
        for _ in range(3):
            E = torch.randn(A.shape, generator=g, dtype=torch.float64, device="cuda")
            Qp, Rp, _, _ = AD.qr_forward(A + h * E)
            Qm, Rm, _, _ = AD.qr_forward(A - h * E)
            fd = (loss_torch(Qp, Rp, b, y, dQ, dR, torch) - loss_torch(Qm, Rm, b, y, dQ, dR, torch)).item() / (2 * h)
            an = (G * E).sum().item()
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


def test_single_matrix_and_none_cotangents(tq, oracle):
    """A 2-D input returns 2-D factors; a loss on R alone gives Qbar = None."""
    import torch
    from tileqr import autodiff as AD
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn((700, 64), generator=g, dtype=torch.float64, device="cuda").requires_grad_(True)
    Q, R = AD.qr(A)
    assert Q.shape == (700, 64) and R.shape == (64, 64)
    W = torch.randn((64, 64), generator=g, dtype=torch.float64, device="cuda")
    (W * R).sum().backward()
    Qo, Ro, _ = oracle.qr_explicit(A.detach().cpu().numpy(), 256, 32)
    ref = oracle.qr_adjoint(Qo, Ro, np.zeros((700, 64)), W.cpu().numpy())
    assert rel(A.grad.cpu().numpy(), ref) <= 1e-11


def test_full_configuration_256_x_2048x256(tq, oracle):
    """256 problems 2048x256 (N(0,1)): a sample of problems against the
    reference adjoint and one central difference over the whole batch."""
    import torch
    from tileqr import autodiff as AD
    batch, m, n = 256, 2048, 256
    A, b, y, dQ, dR = batch_inputs(batch, m, n, 4, torch)
    Ar = A.clone().requires_grad_(True)
    Q, R = AD.qr(Ar)
    loss_torch(Q, R, b, y, dQ, dR, torch).backward()
    G = Ar.grad.detach()
    assert torch.isfinite(G).all()
    Qh, Rh = Q.detach(), R.detach()
    for p in (0, 97, 255):
        _, Qb, Rb = oracle.ls_loss_cotangents(Qh[p].cpu().numpy(), Rh[p].cpu().numpy(), b[p].cpu().numpy(),
                                              y[p].cpu().numpy(), dQ[p].cpu().numpy(), dR[p].cpu().numpy())
        Qo, Ro, _ = oracle.qr_explicit(A[p].cpu().numpy(), 256, 32)
        assert rel(Rh[p].cpu().numpy(), Ro) <= 1e-12 * n
        ref = oracle.qr_adjoint(Qo, Ro, Qb, Rb)
        assert rel(G[p].cpu().numpy(), ref) <= 1e-10
    g = torch.Generator(device="cuda").manual_seed(12)
    E = torch.randn(A.shape, generator=g, dtype=torch.float64, device="cuda")
    h = 1e-6
    with torch.no_grad():
        Qp, Rp, _, _ = AD.qr_forward(A + h * E)
        Qm, Rm, _, _ = AD.qr_forward(A - h * E)
        fd = (loss_torch(Qp, Rp, b, y, dQ, dR, torch) - loss_torch(Qm, Rm, b, y, dQ, dR, torch)).item() / (2 * h)
    an = (G * E).sum().item()
    assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


def test_sharded_adjoint_one_rank():
    """The multi-rank differentiable-QR measurement with a single rank."""
    import os
    import sys
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    r = bench.adjoint_sharded_bench(torch, 1, 0, batch=8, m=512, n=64, steps=1, warmup=1)
    assert r["rank0_problems"] == 8 and r["problems_per_s"] > 0
