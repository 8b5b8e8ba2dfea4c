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


@pytest.mark.parametrize("dt", ["complex128", "complex64"])
@pytest.mark.parametrize("m,n", [(600, 100), (300, 17), (257, 256), (41, 40), (513, 255)])
def test_complex_forward_and_adjoint_match_oracle(tq, oracle, dt, m, n):
    """ComplexF64 / ComplexF32 batches: Q, R of the forward kernel against the
    complex oracle's tile QR on the same inputs, and the adjoint kernel's
    Abar against the complex reference pullback evaluated in complex128 on
    the CPU (itself checked against central differences in the oracle
    tests).  Bars: 1e-12 n (ComplexF64), 1e-5 n (ComplexF32, inputs rounded
    to complex64 for the oracle)."""
    import torch
    from tileqr import autodiff as AD
    tdt = getattr(torch, dt)
    batch = 2
    g = torch.Generator(device="cuda").manual_seed(m + n)
    cr = lambda *s: torch.complex(torch.randn(s, generator=g, dtype=torch.float64, device="cuda"),
                                  torch.randn(s, generator=g, dtype=torch.float64, device="cuda")).to(tdt)
    A, Qbar, Rbar = cr(batch, m, n), cr(batch, m, n), torch.triu(cr(batch, n, n))
    Q, R, F, tau = AD.qr_forward(A, 32)
    Abar = AD.qr_backward(F, tau, Qbar, Rbar, 32)
    torch.cuda.synchronize()
    bar = (1e-12 if dt == "complex128" else 1e-5) * max(n, 8)
    for p in range(batch):
        Ah = A[p].to(torch.complex128).cpu().numpy()
        Qo, Ro, _ = oracle.qr_explicit(Ah, 256, 32)
        assert rel(R[p].to(torch.complex128).cpu().numpy(), Ro) <= bar
        assert rel(Q[p].to(torch.complex128).cpu().numpy(), Qo) <= bar
        Qg = Q[p].to(torch.complex128).cpu().numpy()
        Rg = R[p].to(torch.complex128).cpu().numpy()
        Ab_ref = oracle.qr_adjoint(Qg, Rg, Qbar[p].to(torch.complex128).cpu().numpy(),
                                   Rbar[p].to(torch.complex128).cpu().numpy())
        cond = np.linalg.cond(Rg)
        assert rel(Abar[p].to(torch.complex128).cpu().numpy(), Ab_ref) <= bar * max(1.0, cond / 100)


def test_complex_autograd_matches_central_differences(tq):
    """torch.autograd through the complex rule: the gradient of a real loss of
    (Q, R) against central differences of the GPU forward along a random
    complex direction E (Re<Abar, E> = dL/dt at t = 0 of L(A + t E))."""
    import torch
    from tileqr import autodiff as AD
    m, n = 300, 40
    g = torch.Generator(device="cuda").manual_seed(4)
    cr = lambda *s: torch.complex(torch.randn(s, generator=g, dtype=torch.float64, device="cuda"),
                                  torch.randn(s, generator=g, dtype=torch.float64, device="cuda"))
    A, dQ, dR, E = cr(m, n), cr(m, n), torch.triu(cr(n, n)), cr(m, n)

    def L(A_):
        Q_, R_ = AD.qr(A_)
        return (torch.vdot(dQ.flatten(), Q_.flatten()).real + torch.vdot(dR.flatten(), R_.flatten()).real)

    Ag = A.clone().requires_grad_(True)
    L(Ag).backward()
    h = 1e-6
    with torch.no_grad():
        fd = (L(A + h * E) - L(A - h * E)).item() / (2 * h)
    an = torch.vdot(Ag.grad.flatten(), E.flatten()).real.item()
    assert abs(an - fd) <= 1e-6 * max(1.0, abs(fd)), (an, fd)


def test_complex_adjoint_rejects_square(tq):
    """A square complex matrix keeps a complex R_nn (the one-row last column
    gets no reflector, src/geqr2.jl:32-35), outside the complex adjoint's
    formula: the backward refuses it as an argument error; the forward runs."""
    import torch
    from tileqr import autodiff as AD
    from tileqr import ArgumentError
    A = torch.complex(torch.randn(2, 40, 40, dtype=torch.float64, device="cuda"),
                      torch.randn(2, 40, 40, dtype=torch.float64, device="cuda"))
    Q, R, F, tau = AD.qr_forward(A, 32)
    with pytest.raises(ArgumentError):
        AD.qr_backward(F, tau, torch.zeros_like(Q), torch.zeros_like(R), 32)


@pytest.mark.parametrize("dt", ["float32", "complex64", "float64"])
@pytest.mark.parametrize("m,n", [(600, 100), (300, 17), (513, 255), (97, 33)])
def test_adjoint_partial_solve_block_is_finite_and_repeatable(tq, oracle, dt, m, n):
    """n not a multiple of the triangular solve's column block: the first
    (partial) block's unused rows of the staged R must be zero, not whatever
    an earlier kernel left in shared memory.  Three backward calls on the same
    inputs give the same finite Abar, and Abar matches the FP64 reference
    pullback (bar 1e-4 n for the 4-byte-real types, 1e-12 n for FP64)."""
    import torch
    from tileqr import autodiff as AD
    tdt = getattr(torch, dt)
    g = torch.Generator(device="cuda").manual_seed(3 * m + n)
    if tdt.is_complex:
        cr = lambda *s: torch.complex(torch.randn(s, generator=g, dtype=torch.float64, device="cuda"),
                                      torch.randn(s, generator=g, dtype=torch.float64, device="cuda")).to(tdt)
    else:
        cr = lambda *s: torch.randn(s, generator=g, dtype=torch.float64, device="cuda").to(tdt)
    A, Qbar, Rbar = cr(4, m, n), cr(4, m, n), torch.triu(cr(4, n, n))
    Q, R, F, tau = AD.qr_forward(A, 32)
    outs = [AD.qr_backward(F, tau, Qbar, Rbar, 32) for _ in range(3)]
    torch.cuda.synchronize()
    for o in outs:
        assert bool(torch.isfinite(torch.view_as_real(o) if tdt.is_complex else o).all())
        assert torch.equal(o, outs[0])
    bar = (1e-12 if dt == "float64" else 1e-4) * n
    wide = torch.complex128 if tdt.is_complex else torch.float64
    for p in range(4):
        Qg, Rg = Q[p].to(wide).cpu().numpy(), R[p].to(wide).cpu().numpy()
        ref = oracle.qr_adjoint(Qg, Rg, Qbar[p].to(wide).cpu().numpy(), Rbar[p].to(wide).cpu().numpy())
        cond = np.linalg.cond(Rg)
        assert rel(outs[0][p].to(wide).cpu().numpy(), ref) <= bar * max(1.0, cond / 100)
