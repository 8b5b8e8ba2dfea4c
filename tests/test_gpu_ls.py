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


def _factor_error(tq, A32, nb, ib, f64p):
    """(||I - Q^T Q||_F, ||A - Q R||_F / ||A||_F) of the stored FP32 factor,
    with Q formed in FP64 from the FP32 V and T (widened): the factor's own
    orthogonality and backward error, not those of an FP32 Q formation."""
    import torch
    m, n = A32.shape
    A = tq.empty(m, n, dtype=torch.float32)
    A.copy_(A32)
    if f64p:
        T, _ = tq.tile_geqrf_f64p(A, nb, ib)
    else:
        T, _ = tq.tile_geqrf(A, nb, ib)
    Fd, Td = tq.empty(m, n), tq.empty(*T.shape)
    Fd.copy_(A.double())
    Td.copy_(T.double())
    Q = tq.zeros(m, n)
    Q.diagonal().fill_(1.0)
    tq.tile_unmqr("N", Fd, Td, Q, nb, ib)
    orth = torch.linalg.norm(Q.t() @ Q - torch.eye(n, dtype=torch.float64, device="cuda")).item()
    A64 = A32.double()
    berr = (torch.linalg.norm(A64 - Q @ torch.triu(Fd[:n])) / torch.linalg.norm(A64)).item()
    return orth, berr


@pytest.mark.parametrize("m,n", [(4096, 1024), (8192, 512)])
def test_fp64_panels_improve_the_mixed_factor(tq, m, n):
    """The mixed solve's factorisation keeps the larfg norm and scaling, the
    larft T build and the tsqrt diagonal triangles in FP64 (FP32 updates):
    on the mixed configuration's matrix family (condition number 1e6) its
    stored factor is closer to orthogonal than with FP32 panels, and its
    backward error stays at the FP32 level the updates set."""
    import torch
    A32, _ = make_problem(m, n, 1, 23 + n, torch)
    o32, b32 = _factor_error(tq, A32, 256, 32, False)
    o64, b64 = _factor_error(tq, A32, 256, 32, True)
    print(f"\n{m}x{n}: ||I - Q^T Q||_F FP32 panels {o32:.3e}, FP64 panels {o64:.3e}; "
          f"||A - QR|| / ||A|| {b32:.3e} -> {b64:.3e}")
    assert o64 < 0.75 * o32
    assert o64 < 1e-4 and b64 <= 1.05 * b32 and b64 < 1e-5


def test_fp64_panel_factor_matches_the_oracle(tq, oracle):
    """Parity of the FP64-panel factorisation with the FP64 oracle on the
    same FP32-valued input, at the FP32 bar (the updates are FP32)."""
    import torch
    rng = np.random.default_rng(31)
    m, n, nb, ib = 1024, 512, 256, 32
    A0 = rng.standard_normal((m, n)).astype(np.float32).astype(np.float64)
    A = tq.to_device(A0, dtype=torch.float32)
    T, tau = tq.tile_geqrf_f64p(A, nb, ib)
    Ao = np.asfortranarray(A0)
    To, tauo = oracle.tile_geqrf(Ao, nb, ib)
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    assert rel(tq.to_numpy(A).astype(np.float64), Ao) < 1e-5
    assert rel(tq.to_numpy(T).astype(np.float64), To) < 1e-5
    assert rel(tq.to_numpy(tau).astype(np.float64), tauo) < 1e-5


def test_mixed_solve_with_either_panel_precision(tq, oracle):
    """The mixed solve reaches the FP64 least-squares solution with FP64
    panels (the default) and with FP32 panels (tqr_dsgels_fp64_panels(0)) in
    about as many CGLS iterations (the stagnation stop moves the count by a
    few from one rounding pattern to another)."""
    import torch
    m, n, k = 4096, 1024, 2
    A32, b = make_problem(m, n, k, 41, torch)
    Xo = torch.from_numpy(oracle.tile_lstsq(A32.double().cpu().numpy(), b.cpu().numpy(), 256, 32)).cuda()
    Ac = tq.empty(m, n, dtype=torch.float32)
    Ac.copy_(A32)
    bc = tq.empty(m, k)
    bc.copy_(b)
    res = {}
    old = tq.dsgels_fp64_panels(True)
    try:
        for on in (True, False):
            tq.dsgels_fp64_panels(on)
            Xm, iters, relres = tq.lstsq_mixed(Ac, bc, 256, 32, maxit=60, tol=1e-13)
            res[on] = (iters, (torch.linalg.norm(Xm - Xo) / torch.linalg.norm(Xo)).item())
    finally:
        tq.dsgels_fp64_panels(old)
    print(f"\nmixed solve: FP64 panels {res[True]}, FP32 panels {res[False]} (iterations, rel. to oracle)")
    assert res[True][1] < 1e-8 and res[False][1] < 1e-8
    assert res[True][0] <= res[False][0] + 4


def test_mixed_solve_on_the_hierarchical_tree(tq, oracle):
    """tqr_dsgels with the hierarchical factorisation (tqr_dsgels_hqr_group):
    the same FP64 least-squares solution as the oracle's."""
    import torch
    m, n, k = 8192, 1024, 3
    A32, b = make_problem(m, n, k, 59, torch)
    Xo = torch.from_numpy(oracle.tile_lstsq(A32.double().cpu().numpy(), b.cpu().numpy(), 256, 32)).cuda()
    Ac = tq.empty(m, n, dtype=torch.float32)
    Ac.copy_(A32)
    bc = tq.empty(m, k)
    bc.copy_(b)
    old = tq.dsgels_hqr_group(8)
    try:
        Xm, iters, relres = tq.lstsq_mixed(Ac, bc, 256, 32, maxit=60, tol=1e-13)
    finally:
        tq.dsgels_hqr_group(old)
    rel_ = (torch.linalg.norm(Xm - Xo) / torch.linalg.norm(Xo)).item()
    print(f"\nmixed solve on the hierarchical tree: {iters} iterations, {rel_:.2e} from the oracle")
    assert rel_ < 1e-8 and iters <= 60


@pytest.mark.parametrize("m,n,k", [(4096, 1024, 4), (3000, 1000, 2), (2048, 768, 1)])
def test_pipelined_triangular_solves_match_cooperative_form(tq, m, n, k):
    """The CGLS refinement with R^-1 / R^-T applied by the pipelined task list
    (the default) against the cooperative form with grid barriers: the same
    least-squares solution to refinement accuracy and about the same
    iteration count, run twice (the products' FP64 atomics make the solve
    itself reproducible only to rounding).  n = 1000 leaves a ragged last
    block."""
    import torch
    from tileqr import _lib
    A32, b = make_problem(m, n, k, 40 + n, torch)
    Ac = tq.empty(m, n, dtype=torch.float32)
    Ac.copy_(A32)
    bc = tq.empty(m, k)
    bc.copy_(b)
    L = _lib.lib()
    old = L.tqr_dsgels_trsv_pipelined(1)
    try:
        X1, it1, _ = tq.lstsq_mixed(Ac, bc, 256, 32, maxit=60, tol=1e-13)
        X1 = X1.clone()
        X2, it2, _ = tq.lstsq_mixed(Ac, bc, 256, 32, maxit=60, tol=1e-13)
        X2 = X2.clone()
        L.tqr_dsgels_trsv_pipelined(0)
        Xc, itc, _ = tq.lstsq_mixed(Ac, bc, 256, 32, maxit=60, tol=1e-13)
        Xc = Xc.clone()
    finally:
        L.tqr_dsgels_trsv_pipelined(old)
    rel = lambda a, c: (torch.linalg.norm(a - c) / torch.linalg.norm(c)).item()
    # the stopping rule (three iterations without gain) makes the count move
    # by a few either way between runs; the solutions must agree
    assert rel(X1, X2) < 1e-9
    assert rel(X1, Xc) < 1e-9
    assert min(it1, it2) <= itc + 3
