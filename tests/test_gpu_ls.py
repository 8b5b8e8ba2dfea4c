"""Least squares on the GPU: the plain FP64 solve and the mixed-precision solve.

The problem family is the mixed-precision configuration scaled down: a
Float32-stored A = U diag(sigma) V^T with Haar U, V (QR of Gaussians with R's
diagonal signs fixed), sigma geometric from 1 to 1e-6, b = A x_true + 1e-10
N(0,1), several right-hand sides.  Both solves must give the FP64 least-squares
solution of the FP32-valued A: they are compared with each other and with the
CPU oracle's tile-QR solution, and the mixed solve's normwise backward error
||b - A x|| / (||A||_2 ||x|| + ||b||) must not exceed the FP64 solve's by more
than rounding.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def haar(m, n, g, torch):
    Z = torch.randn(m, n, generator=g, dtype=torch.float64, device="cuda")
    Q, R = torch.linalg.qr(Z)
    return Q * torch.sign(torch.diagonal(R)).unsqueeze(0)


def make_problem(m, n, k, seed, torch):
    g = torch.Generator(device="cuda").manual_seed(seed)
    U = haar(m, n, g, torch)
    V = haar(n, n, g, torch)
    sigma = torch.logspace(0, -6, n, dtype=torch.float64, device="cuda")
    A = ((U * sigma.unsqueeze(0)) @ V.t()).float()
    x_true = torch.randn(n, k, generator=g, dtype=torch.float64, device="cuda")
    b = A.double() @ x_true + 1e-10 * torch.randn(m, k, generator=g, dtype=torch.float64, device="cuda")
    return A, b


def backward_error(A64, x, b, torch):
    r = b - A64 @ x
    return (torch.linalg.norm(r, dim=0) / (1.0 * torch.linalg.norm(x, dim=0) + torch.linalg.norm(b, dim=0))).max().item()


@pytest.mark.parametrize("m,n,k", [(4096, 1024, 4), (2048, 512, 3)])
def test_mixed_and_fp64_least_squares(tq, oracle, m, n, k):
    import torch
    A32, b = make_problem(m, n, k, 17 + n, torch)
    A64 = A32.double()
    # plain FP64 GPU solve
    Af = tq.empty(m, n)
    Af.copy_(A64)
    Bf = tq.empty(m, k)
    Bf.copy_(b)
    X64 = tq.lstsq_fp64(Af, Bf, 256, 32).clone()
    # mixed solve (A32 and b column-major)
    Ac = tq.empty(m, n, dtype=torch.float32)
    Ac.copy_(A32)
    bc = tq.empty(m, k)
    bc.copy_(b)
    Xm, iters, relres = tq.lstsq_mixed(Ac, bc, 256, 32, maxit=60, tol=1e-13)
    # the oracle's FP64 tile-QR solution of the same FP32-valued A
    Xo = oracle.tile_lstsq(A64.cpu().numpy(), b.cpu().numpy(), 256, 32)
    Xo = torch.from_numpy(Xo).cuda()
    rel = lambda a, c: (torch.linalg.norm(a - c) / torch.linalg.norm(c)).item()
    assert rel(X64, Xo) < 1e-12 * n                      # FP64 parity with the oracle
    assert rel(Xm, Xo) < 1e-8, (iters, relres)           # mixed reaches the FP64 solution
    be64 = backward_error(A64, X64, b, torch)
    bem = backward_error(A64, Xm, b, torch)
    beo = backward_error(A64, Xo, b, torch)
    assert bem <= 1.01 * beo + 1e-15 and be64 <= 1.01 * beo + 1e-15
    assert iters <= 60


def test_mixed_factor_orthogonality(tq):
    """||I - Q^T Q|| of the FP32 factor the mixed solve refines with (FP32 level),
    next to the FP64 factor's (FP64 level)."""
    import torch
    m, n = 2048, 512
    A32, _ = make_problem(m, n, 1, 5, torch)
    out = {}
    for dt in (torch.float32, torch.float64):
        A = tq.empty(m, n, dtype=dt)
        A.copy_(A32.to(dt))
        T, _ = tq.tile_geqrf(A, 256, 32)
        Q = tq.empty(m, n, dtype=dt)
        Q.copy_(torch.eye(m, n, dtype=dt, device="cuda"))
        tq.tile_unmqr("N", A, T, Q, 256, 32)
        Qd = Q.double()
        out[dt] = torch.linalg.norm(Qd.t() @ Qd - torch.eye(n, dtype=torch.float64, device="cuda")).item()
    assert out[torch.float64] < 1e-13 * n ** 0.5
    assert out[torch.float32] < 1e-4
