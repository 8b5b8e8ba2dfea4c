"""The ComplexF64 oracle (oracle/nextla_oracle_z.c) against LAPACK's complex
routines and the reference's own complex checks.

The reference runs every tile-kernel test for ComplexF32 and ComplexF64
(test/lapack_helpers.jl:11) at rtol 1e-12 for double precision
(test/lapack_helpers.jl:14); the fixtures are zgeqrt / ztpqrt / ztpmqrt /
zgemqrt / zlarfg outputs (tests/golden/make_golden.py, keys "z_*").

One deliberate difference from LAPACK is pinned too: the reference's geqr2
gives the last reflector of an m <= n panel tau = 0 (src/geqr2.jl:32-35, a
one-element column), where zgeqrt makes that diagonal entry real with a
scalar reflector; LAPACK's last row of R is then (1 - conj(tau)) times the
reference's.
"""
import numpy as np
import pytest

RTOL = 1e-12


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def Z(a):
    return np.array(a, dtype=np.complex128, order="F")


def zeros(*shape):
    return np.zeros(shape, dtype=np.complex128, order="F")


@pytest.mark.parametrize("m,n,ib", [(20, 15, 4), (32, 32, 8), (64, 32, 16), (32, 64, 8), (128, 128, 32)])
def test_zgeqrt_vs_lapack(oracle, golden, m, n, ib):
    key = f"z_geqrt_{m}_{n}_{ib}"
    A = Z(golden[key + "_A"])
    k = min(m, n)
    T, tau = zeros(ib, k), zeros(k)
    oracle.geqrt(m, n, ib, A, T, tau, zeros(ib * n))
    outA, outT = golden[key + "_outA"], golden[key + "_outT"]
    if m > n:
        assert rel(A, outA) < RTOL
        assert rel(T, outT) < RTOL * 10
        return
    # m <= n: every reflector but the last (one-element) one matches zgeqrt
    L = m - 1
    assert rel(A[:L], outA[:L]) < RTOL
    assert rel(A[L, :L], outA[L, :L]) < RTOL
    assert rel(T[:, :L], outT[:, :L]) < RTOL * 10
    assert tau[L] == 0 and np.all(T[:, L] == 0)
    tau_lapack = outT[L % ib, L]
    assert abs(tau_lapack) > 0
    assert rel((1 - np.conj(tau_lapack)) * A[L, L:], outA[L, L:]) < RTOL


@pytest.mark.parametrize("m,n,ib", [(32, 24, 8), (48, 32, 16), (20, 20, 10), (128, 128, 32)])
def test_ztsqrt_vs_lapack(oracle, golden, m, n, ib):
    key = f"z_tsqrt_{m}_{n}_{ib}"
    A1, A2 = Z(golden[key + "_A1"]), Z(golden[key + "_A2"])
    T, tau = zeros(ib, n), zeros(n)
    oracle.tsqrt(m, n, ib, A1, A2, T, tau, zeros(ib * n))
    assert rel(A1, golden[key + "_outA1"]) < RTOL
    assert rel(A2, golden[key + "_outA2"]) < RTOL
    assert rel(T, golden[key + "_outT"]) < RTOL


@pytest.mark.parametrize("kind", ["tsmqr", "ttmqr"])
@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_ztsmqr_ttmqr_vs_lapack(oracle, golden, kind, st):
    key = f"z_{kind}_{st}"
    m1, n1, m2, n2, k, ib = (int(x) for x in golden[key + "_dims"])
    A1, A2 = Z(golden[key + "_A1"]), Z(golden[key + "_A2"])
    V, T = Z(golden[key + "_V"]), Z(golden[key + "_T"])
    # both routines reduce to ztpmqrt(l = 0) on these inputs (V rectangular,
    # or upper triangular with zeros below, test/ttmqr.jl:14)
    oracle.tsmqr(st[0], st[1], m1, n1, m2, n2, k, ib, A1, A2, V, T, zeros(ib * max(m1, n1)))
    assert rel(A1, golden[key + "_outA1"]) < RTOL
    assert rel(A2, golden[key + "_outA2"]) < RTOL
    if kind == "ttmqr":
        B1, B2 = Z(golden[key + "_A1"]), Z(golden[key + "_A2"])
        oracle.ttmqr(st[0], st[1], m1, n1, m2, n2, k, ib, B1, B2, V, T, zeros(ib * max(m1, n1)))
        assert rel(B1, golden[key + "_outA1"]) < RTOL
        assert rel(B2, golden[key + "_outA2"]) < RTOL


@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_zunmqr_vs_lapack(oracle, golden, st):
    Aq, Tq = Z(golden["z_unmqr_Aqr"]), Z(golden["z_unmqr_T"])
    C = Z(golden[f"z_unmqr_{st}_C"])
    m, k = Aq.shape
    ib = Tq.shape[0]
    mm, nn = C.shape
    work = zeros(nn if st[0] == "L" else mm, ib)
    oracle.unmqr(st[0], st[1], mm, nn, k, ib, Aq, m, Tq, C, work)
    assert rel(C, golden[f"z_unmqr_{st}_out"]) < RTOL


@pytest.mark.parametrize("n", [2, 7, 33, 256])
def test_zhouseholder_vs_zlarfg(oracle, golden, n):
    """A one-column geqr2 is the reference's inline complex larfg."""
    x = golden[f"z_larfg_{n}_x"]
    ref = golden[f"z_larfg_{n}_out"]
    A = Z(x.reshape(n, 1))
    tau = zeros(1)
    oracle.geqr2(n, 1, A, tau, zeros(1))
    assert abs(A[0, 0] - ref[0]) <= RTOL * abs(ref[0])
    assert A[0, 0].imag == 0.0                  # beta is real
    assert rel(A[1:, 0], ref[1:-1]) < RTOL
    assert abs(tau[0] - ref[-1]) <= RTOL * abs(ref[-1])


@pytest.mark.parametrize("n,ib", [(16, 4), (24, 8), (48, 16)])
def test_zttqrt_vs_lapack(oracle, golden, n, ib):
    key = f"z_ttqrt_{n}_{ib}"
    A1, A2 = Z(golden[key + "_A1"]), Z(golden[key + "_A2"])
    T, tau = zeros(ib, n), zeros(n)
    oracle.ttqrt(n, n, ib, A1, A2, T, tau, zeros(ib * n))
    assert rel(np.triu(A1), np.triu(golden[key + "_outA1"])) < RTOL
    assert rel(np.triu(A2), np.triu(golden[key + "_outA2"])) < RTOL
    assert rel(T, golden[key + "_outT"]) < RTOL
    for trans in "NC":
        C1, C2 = Z(golden[f"{key}_L{trans}_C1"]), Z(golden[f"{key}_L{trans}_C2"])
        oracle.ttmqr("L", trans, n, 40, n, 40, n, ib, C1, C2, A2, T, zeros(ib * 40))
        assert rel(C1, golden[f"{key}_L{trans}_out1"]) < RTOL
        assert rel(C2, golden[f"{key}_L{trans}_out2"]) < RTOL


def test_zgeqrt_ib1_equals_geqr2(oracle):
    """test/geqrt.jl:54-71 for ComplexF64."""
    rng = np.random.default_rng(1)
    A0 = Z(rng.random((16, 12)) + 1j * rng.random((16, 12)))
    A1, A2 = A0.copy(order="F"), A0.copy(order="F")
    oracle.geqrt(16, 12, 1, A1, zeros(1, 12), zeros(12), zeros(12))
    oracle.geqr2(16, 12, A2, zeros(12), zeros(12))
    assert rel(A1, A2) < RTOL


@pytest.mark.parametrize("direct", ["F", "B"])
@pytest.mark.parametrize("storev", ["C", "R"])
@pytest.mark.parametrize("n,k", [(1, 1), (5, 3), (10, 4), (20, 8)])
def test_zlarft_explicit_h(oracle, direct, storev, n, k):
    """test/larft.jl:6-61 for ComplexF64: I - V T V^H = H_1 H_2 ... H_k
    (forward) or H_k ... H_1 ... in the backward layout (V's unit entries at
    rows n-k+i), with H_i = I - tau_i v_i v_i^H."""
    rng = np.random.default_rng(n * 100 + k + (7 if direct == "B" else 0))
    Vc = Z(rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k)))
    for j in range(k):
        if direct == "F":
            Vc[:j, j] = 0.0
            Vc[j, j] = 1.0
        else:
            Vc[n - k + j + 1:, j] = 0.0
            Vc[n - k + j, j] = 1.0
    # rowwise storage holds v_i^H in row i (H = I - V^H T V, LAPACK's zlarft)
    V = Vc if storev == "C" else Z(Vc.conj().T)
    tau = rng.standard_normal(k) + 1j * rng.standard_normal(k)
    T = zeros(k, k)
    oracle.larft(direct, storev, n, k, V, Z(tau), T)
    assert np.allclose(np.diag(T), tau)
    if direct == "B":
        assert np.allclose(T, np.tril(T))
        return   # the backward form keeps the reference's own indexing (larft.jl:146-158)
    assert np.allclose(T, np.triu(T))
    Hc = np.eye(n) - Vc @ T @ Vc.conj().T
    Ht = np.eye(n, dtype=complex)
    for j in range(k):
        v = Vc[:, j]
        Ht = Ht @ (np.eye(n) - tau[j] * np.outer(v, v.conj()))
    assert np.linalg.norm(Hc - Ht) / max(1.0, np.linalg.norm(Ht)) < RTOL * n * 10


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
@pytest.mark.parametrize("m,n", [(5, 4), (10, 8), (20, 15)])
def test_zlarfb_explicit_h(oracle, side, trans, m, n):
    """test/larfb.jl:6-43 for ComplexF64."""
    rng = np.random.default_rng(m * 31 + n)
    k = min(m if side == "L" else n, 4)
    rows = m if side == "L" else n
    panel = Z(rng.standard_normal((rows, k)) + 1j * rng.standard_normal((rows, k)))
    tau = zeros(k)
    oracle.geqr2(rows, k, panel, tau, zeros(k))
    V = panel.copy(order="F")
    for j in range(k):
        V[:j, j] = 0.0
        V[j, j] = 1.0
    T = zeros(k, k)
    oracle.larft("F", "C", rows, k, V, tau, T)
    C0 = Z(rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n)))
    C = C0.copy(order="F")
    work = zeros(n if side == "L" else m, k)
    oracle.larfb(side, trans, "F", "C", m, n, k, V, rows, T, C, work)
    H = np.eye(rows) - V @ T @ V.conj().T
    Ht = H if trans == "N" else H.conj().T
    ref = Ht @ C0 if side == "L" else C0 @ Ht
    assert np.allclose(C, ref, rtol=RTOL * max(1, m, n), atol=RTOL * max(1, m, n))
    # the explicit product of the reflectors is unitary
    assert np.allclose(H.conj().T @ H, np.eye(rows), atol=1e-13 * rows)


def test_zunmqr_unitary(oracle):
    """test/unmqr.jl:69-78 for ComplexF64: Q Q^H = I."""
    rng = np.random.default_rng(7)
    m, k, ib = 64, 32, 8
    A = Z(rng.random((m, k)) + 1j * rng.random((m, k)))
    T = zeros(ib, k)
    oracle.geqrt(m, k, ib, A, T, zeros(k), zeros(ib * k))
    C = Z(np.eye(m))
    work = zeros(m, ib)
    oracle.unmqr("L", "N", m, m, k, ib, A, m, T, C, work)
    oracle.unmqr("L", "C", m, m, k, ib, A, m, T, C, work)
    assert np.allclose(C, np.eye(m), atol=1e-13)


def test_ztrans_t_equals_c(oracle, golden):
    """'T' acts as 'C' for complex elements (src/tsmqr.jl:20)."""
    key = "z_tsmqr_LC"
    m1, n1, m2, n2, k, ib = (int(x) for x in golden[key + "_dims"])
    A1, A2 = Z(golden[key + "_A1"]), Z(golden[key + "_A2"])
    V, T = Z(golden[key + "_V"]), Z(golden[key + "_T"])
    oracle.tsmqr("L", "T", m1, n1, m2, n2, k, ib, A1, A2, V, T, zeros(ib * max(m1, n1)))
    assert rel(A1, golden[key + "_outA1"]) < RTOL


def test_zmixed_types_rejected(oracle):
    with pytest.raises(TypeError):
        oracle.geqrt(4, 4, 2, zeros(4, 4), np.zeros((2, 4), order="F"), zeros(4), zeros(8))


@pytest.mark.parametrize("m,n,nb,ib", [(300, 200, 64, 16), (513, 257, 128, 32), (256, 256, 256, 32)])
def test_ztile_qr_backward_error(oracle, m, n, nb, ib):
    rng = np.random.default_rng(m + n)
    A0 = Z(rng.uniform(-1, 1, (m, n)) + 1j * rng.uniform(-1, 1, (m, n)))
    A = A0.copy(order="F")
    T, tau = oracle.tile_geqrf(A, nb, ib)
    assert T.dtype == np.complex128
    R = np.triu(A[:n, :n])
    Q = Z(np.eye(m))
    oracle.tile_unmqr("N", A, T, Q, nb, ib)
    eps = np.finfo(float).eps
    assert np.linalg.norm(A0 - Q[:, :n] @ R, 1) / (np.linalg.norm(A0, 1) * n * eps) < 10
    assert np.linalg.norm(Q.conj().T @ Q - np.eye(m), 1) / (m * eps) < 10
    # |R| agrees with LAPACK's (R is unique up to a unit complex factor per row)
    R_l = np.linalg.qr(A0, mode="r")
    assert np.allclose(np.abs(R), np.abs(R_l), atol=1e-10 * np.abs(R_l).max())
    # Q^H applied through the tiles gives [R; 0]
    B = A0.copy(order="F")
    oracle.tile_unmqr("C", A, T, B, nb, ib)
    assert np.linalg.norm(B[:n] - R) <= 1e-13 * n * np.linalg.norm(R)


def test_ztile_lstsq(oracle):
    """Complex least squares through the tile QR and LeftUpperTRSM!'s solve."""
    rng = np.random.default_rng(3)
    A = Z(rng.standard_normal((600, 300)) + 1j * rng.standard_normal((600, 300)))
    x = rng.standard_normal((300, 2)) + 1j * rng.standard_normal((300, 2))
    X = oracle.tile_lstsq(A, A @ x, 128, 32)
    assert X.dtype == np.complex128
    assert np.abs(X - x).max() < 1e-10


def test_ztrsm_smith_division(oracle):
    """The back-substitution against numpy's solve on a well-conditioned R,
    including diagonal entries with a dominant imaginary part (the second
    branch of Smith's division)."""
    rng = np.random.default_rng(4)
    n = 40
    R = np.triu(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    R[np.diag_indices(n)] = (2 + rng.random(n)) * np.exp(1j * rng.uniform(0, 2 * np.pi, n))
    R = Z(R)
    B = Z(rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3)))
    X = B.copy(order="F")
    oracle.trsm_lun(R, X)
    assert np.abs(R @ X - B).max() < 1e-13


@pytest.mark.parametrize("m,n,nb,ib,grp", [(1024, 256, 128, 32, 1), (1000, 300, 128, 16, 3), (1024, 256, 128, 32, 2),
                                           (517, 130, 64, 16, 3), (300, 400, 256, 32, 2), (768, 256, 128, 32, 100)])
def test_ztile_hqr_properties(oracle, m, n, nb, ib, grp):
    """The complex hierarchical / binary-tree tile QR (geqrt on the leaders,
    tsqrt merges in each group, ttqrt merges between leaders, as ttqrt!'s
    ComplexF64 tests run them, test/ttqrt.jl:28-66): Q^H A = [R; 0] and
    Q Q^H = I through the stored factors, and |R| equal to the flat tree's
    (R is unique up to a unitary diagonal)."""
    rng = np.random.default_rng(m + n + grp)
    A0 = Z(rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n)))
    A = A0.copy(order="F")
    T, tau, T2, tau2 = oracle.tile_geqrf_hqr(A, nb, ib, grp)
    assert T.dtype == np.complex128 and tau2.dtype == np.complex128
    k = min(m, n)
    R = np.triu(A[:k])
    B = A0.copy(order="F")
    oracle.tile_unmqr_hqr("C", A, T, T2, B, nb, ib, grp)
    assert np.linalg.norm(B[:k] - R) <= 1e-13 * np.linalg.norm(R) * k
    assert np.linalg.norm(B[k:]) <= 1e-13 * np.linalg.norm(A0) * k
    C0 = Z(rng.standard_normal((m, 5)) + 1j * rng.standard_normal((m, 5)))
    C = C0.copy(order="F")
    oracle.tile_unmqr_hqr("N", A, T, T2, C, nb, ib, grp)
    oracle.tile_unmqr_hqr("C", A, T, T2, C, nb, ib, grp)
    assert np.abs(C - C0).max() < 1e-13 * m
    F = A0.copy(order="F")
    oracle.tile_geqrf(F, nb, ib)
    assert np.allclose(np.abs(R), np.abs(np.triu(F[:k])), atol=1e-11 * np.abs(R).max())
