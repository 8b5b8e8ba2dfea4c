"""Tile QR, Q application, triangular solve and least squares on the GPU.

Small and medium sizes compare with the oracle's flat-tree tile QR on the same
seeded inputs: R, V and T relative differences must stay within 1e-12 * n
(the parity bar for the plain FP64 form).  At the full benchmark sizes, where
the scalar oracle would take minutes, size-independent properties stand in:
orthogonal invariance ||A x|| = ||R x||, Q^T A = R through the Q application,
and ||Q^T b|| = ||b||.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def F(a):
    return np.array(a, dtype=np.float64, order="F")


@pytest.mark.parametrize("m,n,nb,ib", [
    (1024, 1024, 256, 32),     # the CPU-runnable configuration (4 x 4 tiles)
    (300, 200, 64, 16),
    (513, 257, 128, 32),       # ragged last tiles
    (1000, 1000, 256, 32),
    (200, 300, 64, 32),        # wide
    (96, 96, 96, 32),          # single tile
    (2048, 256, 256, 32),      # tall-skinny panel
])
def test_tile_qr_vs_oracle(tq, oracle, m, n, nb, ib):
    rng = np.random.default_rng(m * 7 + n)
    A0 = F(rng.uniform(-1, 1, (m, n)))
    A = tq.to_device(A0)
    T, tau = tq.tile_geqrf(A, nb, ib)
    Ao = A0.copy(order="F")
    To, tauo = oracle.tile_geqrf(Ao, nb, ib)
    tol = 1e-12 * max(m, n)
    assert rel(tq.to_numpy(A), Ao) < tol
    assert rel(tq.to_numpy(T), To) < tol
    assert rel(tq.to_numpy(tau), tauo) < tol
    k = min(m, n)
    assert rel(np.triu(tq.to_numpy(A)[:k]), np.triu(Ao[:k])) < tol


@pytest.mark.parametrize("m,n,nb,ib", [(1024, 1024, 256, 32), (2048, 1024, 256, 32),
                                       (1024, 2048, 256, 32), (512, 512, 128, 32),
                                       (768, 512, 128, 16), (1024, 1024, 256, 64)])
def test_dag_equals_stream_driver(tq, oracle, m, n, nb, ib):
    """The persistent-kernel schedule runs the same per-strip arithmetic as the
    stream driver, so the two agree bit for bit; both match the oracle."""
    import torch
    rng = np.random.default_rng(m + 3 * n + ib)
    A0 = F(rng.standard_normal((m, n)))
    Ad, As = tq.to_device(A0), tq.to_device(A0)
    Td, taud = tq.tile_geqrf(Ad, nb, ib, dag=True)
    Ts, taus = tq.tile_geqrf(As, nb, ib, dag=False)
    torch.cuda.synchronize()
    assert torch.equal(Ad, As)
    assert torch.equal(Td, Ts)
    assert torch.equal(taud, taus)
    Ao = A0.copy(order="F")
    To, _ = oracle.tile_geqrf(Ao, nb, ib)
    assert rel(tq.to_numpy(Ad), Ao) < 1e-12 * max(m, n)
    assert rel(tq.to_numpy(Td), To) < 1e-12 * max(m, n)


def test_dag_repeated_calls_reuse_workspace(tq):
    """Back-to-back factorisations through the same cached workspace."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(7)
    A0 = tq.empty(1024, 1024)
    A0.copy_(torch.randn(1024, 1024, generator=g, dtype=torch.float64, device="cuda"))
    outs = []
    for _ in range(3):
        A = A0.clone()
        T, _ = tq.tile_geqrf(A, 256, 32)
        outs.append((A, T))
    for A, T in outs[1:]:
        assert torch.equal(A, outs[0][0]) and torch.equal(T, outs[0][1])


@pytest.mark.parametrize("trans", ["C", "N"])
def test_tile_unmqr_vs_oracle(tq, oracle, trans):
    """The 1024^2 tile QR's second half: Q applied to 16 seeded right-hand sides."""
    rng = np.random.default_rng(16)
    m = n = 1024
    nb, ib = 256, 32
    A0 = F(rng.uniform(-1, 1, (m, n)))
    A = tq.to_device(A0)
    T, _ = tq.tile_geqrf(A, nb, ib)
    Ao = A0.copy(order="F")
    To, _ = oracle.tile_geqrf(Ao, nb, ib)
    B0 = F(rng.uniform(-1, 1, (m, 16)))
    B = tq.to_device(B0)
    tq.tile_unmqr(trans, A, T, B, nb, ib)
    Bo = B0.copy(order="F")
    oracle.tile_unmqr(trans, Ao, To, Bo, nb, ib)
    assert rel(tq.to_numpy(B), Bo) < 1e-12 * n


def test_trsm_vs_oracle(tq, oracle):
    rng = np.random.default_rng(4)
    n = 700
    R0 = F(np.triu(rng.uniform(-1, 1, (n, n))) + 4 * np.eye(n))
    B0 = F(rng.standard_normal((n, 5)))
    B = tq.to_device(B0)
    tq.trsm_lun(tq.to_device(R0), B)
    Bo = B0.copy(order="F")
    oracle.trsm_lun(R0, Bo)
    assert rel(tq.to_numpy(B), Bo) < 1e-12 * n


@pytest.mark.parametrize("m,n,nrhs", [(1024, 1024, 16), (2000, 700, 4)])
def test_tile_gels(tq, oracle, m, n, nrhs):
    rng = np.random.default_rng(m + nrhs)
    A0 = F(rng.standard_normal((m, n)))
    X0 = rng.standard_normal((n, nrhs))
    B0 = F(A0 @ X0 + 1e-10 * rng.standard_normal((m, nrhs)))
    A, B = tq.to_device(A0), tq.to_device(B0)
    X, _, _ = tq.tile_gels(A, B, 256, 32)
    Xo = oracle.tile_lstsq(A0, B0, 256, 32)
    assert rel(tq.to_numpy(X), Xo) < 1e-12 * n
    x = tq.to_numpy(X)
    r = B0 - A0 @ x
    assert np.linalg.norm(A0.T @ r) / (np.linalg.norm(A0) ** 2 * np.linalg.norm(x)) < 1e-14


@pytest.mark.parametrize("m,n", [(8192, 8192), (65536, 512)])
def test_full_size_properties(tq, m, n):
    """Benchmark sizes: orthogonal invariance and Q^T A = R."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(m + n)
    A = tq.empty(m, n)
    A.copy_(torch.randn(m, n, generator=g, device="cuda", dtype=torch.float64))
    A0 = A.clone()
    nb, ib = 256, 32
    T, _ = tq.tile_geqrf(A, nb, ib)
    R = torch.triu(A[:n, :n])
    X = torch.randn(n, 8, generator=g, device="cuda", dtype=torch.float64)
    lhs = torch.linalg.norm(A0 @ X, dim=0)
    rhs = torch.linalg.norm(R @ X, dim=0)
    assert float(torch.max(torch.abs(lhs - rhs) / rhs)) < 1e-12 * n ** 0.5
    # Q^T applied to 8 columns of the original A reproduces R's columns
    cols = [0, 1, n // 3, n // 2, n - 2, n - 1, 17, n // 5]
    B = tq.empty(m, len(cols))
    B.copy_(A0[:, cols])
    tq.tile_unmqr("C", A, T, B, nb, ib)
    Bh = B.cpu().numpy()
    Rh = R[:, cols].cpu().numpy()
    assert rel(Bh[:n], Rh) < 1e-12 * n
    if m > n:
        assert np.max(np.abs(Bh[n:])) < 1e-12 * n * np.max(np.abs(Rh))


def test_dag_bounded_wait_reports_and_context_survives(tq):
    """Failure detection without a fault: task 0 of the persistent kernel also
    waits for a word nothing writes.  Every wait is bounded (100 ms here), so
    the launch ends by itself with status 1 (a wait timed out) and the CUDA
    context stays usable: a normal factorisation afterwards is correct."""
    import ctypes
    import time
    import torch
    from tileqr import _lib
    L = _lib.lib()
    m = n = 512
    nb, ib = 256, 32
    rng = np.random.default_rng(5)
    A0 = np.asfortranarray(rng.standard_normal((m, n)))
    A = tq.to_device(A0)
    ts, taus = tq.tile_shapes(m, n, nb, ib)
    T, tau = tq.zeros(*ts), tq.zeros(*taus)
    w, off, size = tq.dag_workspace(m, n, nb, ib, A.device)
    wp = w.data_ptr() + off
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    st = torch.cuda.current_stream()
    t0 = time.time()
    rc = L.tqr_tile_dag_wait_selftest(m, n, nb, ib, P(A), m, P(T), ts[0], P(tau), taus[0], ctypes.c_void_p(wp), size,
                                      100, ctypes.c_void_p(st.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert time.time() - t0 < 10
    status, task = tq.dag_status(wp)
    assert status == 1, (status, task)
    assert L.tqr_tile_dag_wait_selftest(m, n, nb, ib, P(A), m, P(T), ts[0], P(tau), taus[0], ctypes.c_void_p(wp),
                                        size, 0, None) == -13
    # the context still works: a full factorisation is right
    B = tq.to_device(A0)
    tq.tile_geqrf(B, nb, ib)
    R = np.triu(tq.to_numpy(B)[:n])
    x = rng.standard_normal((n, 2))
    ax = np.linalg.norm(A0 @ x, axis=0)
    assert np.max(np.abs(ax - np.linalg.norm(R @ x, axis=0)) / ax) < 1e-13 * n
