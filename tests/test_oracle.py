"""The CPU oracle against LAPACK golden vectors and the reference's own checks.

These pin the oracle (oracle/nextla_oracle.c) before it is used to judge the
CUDA library: the reference tests compare NextLA's kernels with LAPACK at
rtol 1e-12 (test/lapack_helpers.jl:14), and so do these, on the fixtures in
tests/golden (made by tests/golden/make_golden.py).
"""
import numpy as np
import pytest

RTOL = 1e-12


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def F(a):
    return np.array(a, dtype=np.float64, order="F")


@pytest.mark.parametrize("m,n,ib", [(20, 15, 4), (32, 32, 8), (64, 32, 16), (32, 64, 8), (256, 256, 32)])
def test_geqrt_vs_lapack(oracle, golden, m, n, ib):
    key = f"geqrt_{m}_{n}_{ib}"
    A = F(golden[key + "_A"])
    k = min(m, n)
    T = np.zeros((ib, k), order="F")
    tau = np.zeros(k)
    oracle.geqrt(m, n, ib, A, T, tau, np.zeros(ib * n))
    assert rel(A, golden[key + "_outA"]) < RTOL
    assert rel(T, golden[key + "_outT"]) < RTOL * 10


@pytest.mark.parametrize("m,n,ib", [(32, 24, 8), (48, 32, 16), (64, 48, 16), (20, 20, 10), (256, 256, 32)])
def test_tsqrt_vs_lapack(oracle, golden, m, n, ib):
    key = f"tsqrt_{m}_{n}_{ib}"
    A1, A2 = F(golden[key + "_A1"]), F(golden[key + "_A2"])
    T = np.zeros((ib, n), order="F")
    tau = np.zeros(n)
    oracle.tsqrt(m, n, ib, A1, A2, T, tau, np.zeros(ib * n))
    assert rel(A1, golden[key + "_outA1"]) < RTOL
    assert rel(A2, golden[key + "_outA2"]) < RTOL
    assert rel(T, golden[key + "_outT"]) < RTOL
    assert np.allclose(np.diag(T[:, :ib]) if ib == n else tau[:ib], tau[:ib])


@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_tsmqr_vs_lapack(oracle, golden, st):
    key = f"tsmqr_{st}"
    m1, n1, m2, n2, k, ib = (int(x) for x in golden[key + "_dims"])
    A1, A2 = F(golden[key + "_A1"]), F(golden[key + "_A2"])
    V, T = F(golden[key + "_V"]), F(golden[key + "_T"])
    oracle.tsmqr(st[0], st[1], m1, n1, m2, n2, k, ib, A1, A2, V, T, np.zeros(ib * max(m1, n1)))
    assert rel(A1, golden[key + "_outA1"]) < RTOL
    assert rel(A2, golden[key + "_outA2"]) < RTOL


def test_tsmqr_tile_size_vs_lapack(oracle, golden):
    A1, A2 = F(golden["tsmqr_big_A1"]), F(golden["tsmqr_big_A2"])
    V, T = F(golden["tsmqr_big_V"]), F(golden["tsmqr_big_T"])
    oracle.tsmqr("L", "C", 256, 128, 256, 128, 256, 32, A1, A2, V, T, np.zeros(32 * 256))
    assert rel(A1, golden["tsmqr_big_outA1"]) < RTOL
    assert rel(A2, golden["tsmqr_big_outA2"]) < RTOL


@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_unmqr_vs_lapack(oracle, golden, st):
    Aq, Tq = F(golden["unmqr_Aqr"]), F(golden["unmqr_T"])
    C = F(golden[f"unmqr_{st}_C"])
    m, k = Aq.shape
    ib = Tq.shape[0]
    mm, nn = C.shape
    work = np.zeros((nn if st[0] == "L" else mm, ib), order="F")
    oracle.unmqr(st[0], st[1], mm, nn, k, ib, Aq, m, Tq, C, work)
    assert rel(C, golden[f"unmqr_{st}_out"]) < RTOL


@pytest.mark.parametrize("n", [2, 7, 33, 256])
def test_householder_vs_dlarfg(oracle, golden, n):
    """A one-column geqr2 is NextLA's inline larfg (src/geqr2.jl:37-73)."""
    x = golden[f"larfg_{n}_x"]
    ref = golden[f"larfg_{n}_out"]
    A = F(x.reshape(n, 1))
    tau = np.zeros(1)
    oracle.geqr2(n, 1, A, tau, np.zeros(1))
    assert abs(A[0, 0] - ref[0]) <= RTOL * abs(ref[0])
    assert rel(A[1:, 0], ref[1:-1]) < RTOL
    assert abs(tau[0] - ref[-1]) <= RTOL * abs(ref[-1])


def test_geqrt_ib1_equals_geqr2(oracle):
    """test/geqrt.jl:54-71."""
    rng = np.random.default_rng(1)
    A0 = F(rng.random((16, 12)))
    A1, A2 = A0.copy(order="F"), A0.copy(order="F")
    oracle.geqrt(16, 12, 1, A1, np.zeros((1, 12), order="F"), np.zeros(12), np.zeros(12))
    oracle.geqr2(16, 12, A2, np.zeros(12), np.zeros(12))
    assert rel(A1, A2) < RTOL


@pytest.mark.parametrize("storev", ["C", "R"])
@pytest.mark.parametrize("n,k", [(1, 1), (5, 3), (10, 4), (20, 8)])
def test_larft_explicit_h(oracle, storev, n, k):
    """test/larft.jl:6-61: T upper, diag = tau, I - V T V^H = H_1 ... H_k."""
    rng = np.random.default_rng(n * 100 + k)
    if storev == "C":
        V = F(rng.standard_normal((n, k)))
        for j in range(k):
            V[:j, j] = 0.0
            V[j, j] = 1.0
    else:
        V = F(rng.standard_normal((k, n)))
        for i in range(k):
            V[i, :i] = 0.0
            V[i, i] = 1.0
    tau = rng.standard_normal(k)
    T = np.zeros((k, k), order="F")
    oracle.larft("F", storev, n, k, V, tau, T)
    assert np.allclose(T, np.triu(T))
    assert np.allclose(np.diag(T), tau)
    Hc = np.eye(n) - (V @ T @ V.T if storev == "C" else V.T @ T @ V)
    Ht = np.eye(n)
    for j in range(k):
        v = V[:, j] if storev == "C" else V[j, :]
        Ht = Ht @ (np.eye(n) - tau[j] * np.outer(v, v))
    assert np.linalg.norm(Hc - Ht) / max(1.0, np.linalg.norm(Ht)) < RTOL * n


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
@pytest.mark.parametrize("m,n", [(5, 4), (10, 8), (20, 15)])
def test_larfb_explicit_h(oracle, side, trans, m, n):
    """test/larfb.jl:6-43."""
    rng = np.random.default_rng(m * 31 + n)
    k = min(m if side == "L" else n, 4)
    rows = m if side == "L" else n
    panel = F(rng.standard_normal((rows, k)))
    tau = np.zeros(k)
    oracle.geqr2(rows, k, panel, tau, np.zeros(k))
    V = panel.copy(order="F")
    for j in range(k):
        V[:j, j] = 0.0
        V[j, j] = 1.0
    T = np.zeros((k, k), order="F")
    oracle.larft("F", "C", rows, k, V, tau, T)
    C0 = F(rng.standard_normal((m, n)))
    C = C0.copy(order="F")
    work = np.zeros((n if side == "L" else m, k), order="F")
    oracle.larfb(side, trans, "F", "C", m, n, k, V, rows, T, C, work)
    H = np.eye(rows) - V @ T @ V.T
    Ht = H if trans == "N" else H.T
    ref = Ht @ C0 if side == "L" else C0 @ Ht
    assert np.allclose(C, ref, rtol=RTOL * max(1, m, n), atol=RTOL * max(1, m, n))


def test_unmqr_orthogonality(oracle):
    """test/unmqr.jl:69-78: Q Q^H = I."""
    rng = np.random.default_rng(7)
    m, k, ib = 64, 32, 8
    A = F(rng.random((m, k)))
    T = np.zeros((ib, k), order="F")
    oracle.geqrt(m, k, ib, A, T, np.zeros(k), np.zeros(ib * k))
    C = np.eye(m, order="F")
    work = np.zeros((m, ib), order="F")
    oracle.unmqr("L", "N", m, m, k, ib, A, m, T, C, work)
    oracle.unmqr("L", "C", m, m, k, ib, A, m, T, C, work)
    assert np.allclose(C, np.eye(m), atol=1e-13)


def test_argument_errors(oracle):
    """test/geqrt.jl:76-81, test/tsqrt.jl error cases, test/tsmqr.jl:88-93."""
    z = np.zeros((5, 5), order="F")
    with pytest.raises(ValueError):
        oracle.geqrt(-1, 5, 2, z, np.zeros((2, 5), order="F"), np.zeros(5), np.zeros(10))
    with pytest.raises(ValueError):
        oracle.geqrt(5, 5, 0, z, np.zeros((2, 5), order="F"), np.zeros(5), np.zeros(10))
    with pytest.raises(ValueError):
        oracle.tsqrt(8, -1, 4, np.zeros((8, 8), order="F"), np.zeros((8, 8), order="F"),
                     np.zeros((4, 8), order="F"), np.zeros(8), np.zeros(32))
    with pytest.raises(ValueError):
        oracle.tsmqr("X", "N", 8, 8, 8, 8, 4, 2, np.zeros((8, 8), order="F"), np.zeros((8, 8), order="F"),
                     np.zeros((8, 4), order="F"), np.zeros((2, 4), order="F"), np.zeros(16))


@pytest.mark.parametrize("m,n,nb,ib", [(1024, 1024, 256, 32), (300, 200, 64, 16), (513, 257, 128, 32)])
def test_tile_qr_oracle_backward_error(oracle, m, n, nb, ib):
    rng = np.random.default_rng(m + n)
    A0 = F(rng.uniform(-1, 1, (m, n)))
    A = A0.copy(order="F")
    T, _ = oracle.tile_geqrf(A, nb, ib)
    R = np.triu(A[:n, :n])
    Q = np.eye(m, order="F")
    oracle.tile_unmqr("N", A, T, Q, nb, ib)
    eps = np.finfo(float).eps
    assert np.linalg.norm(A0 - Q[:, :n] @ R, 1) / (np.linalg.norm(A0, 1) * n * eps) < 10
    assert np.linalg.norm(Q.T @ Q - np.eye(m), 1) / (m * eps) < 10
    # R agrees with LAPACK's up to row signs
    R_l = np.linalg.qr(A0, mode="r")
    assert np.allclose(np.abs(R), np.abs(R_l), atol=1e-10 * np.abs(R_l).max())


def test_tile_lstsq_oracle(oracle):
    rng = np.random.default_rng(3)
    A = F(rng.standard_normal((600, 300)))
    x = rng.standard_normal((300, 2))
    B = A @ x
    X = oracle.tile_lstsq(A, B, 128, 32)
    assert np.abs(X - x).max() < 1e-10
