"""The oracle's TT kernels and tree driver, pinned to LAPACK.

ttqrt! is checked the way test/ttqrt.jl checks it (A1, A2 = triu(randn) + 2I
against dtpqrt with l = n, reference shapes n, ib = 16/4, 24/8, 32/8, 48/16)
and at the 256/32 tile size, T included; ttmqr! the way test/ttmqr.jl does
(n = 24, k = 16, ib = 8, V = triu(randn), dtpmqrt l = 0, all side x trans)
plus on a real TT factorisation against dtpmqrt with l = n.  The tree tile QR
is checked by its properties (Q R = A, Q^T Q = I, |R| = |R| of LAPACK's QR).
"""
import numpy as np
import pytest

RTOL = 1e-12


def close(a, b, rtol=RTOL):
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("n,ib", [(16, 4), (24, 8), (32, 8), (48, 16), (256, 32)])
def test_ttqrt_matches_dtpqrt(oracle, golden, n, ib):
    key = f"ttqrt_{n}_{ib}"
    A1 = np.array(golden[key + "_A1"], order="F")
    A2 = np.array(golden[key + "_A2"], order="F")
    T = np.zeros((ib, n), order="F")
    tau = np.zeros(n)
    oracle.ttqrt(n, n, ib, A1, A2, T, tau, np.zeros(ib * n))
    assert close(A1, golden[key + "_outA1"])
    assert close(A2, golden[key + "_outA2"])
    # T blocks: upper triangles of the ib x ib blocks (LAPACK leaves the rest)
    Tg = golden[key + "_outT"]
    for j in range(0, n, ib):
        sb = min(ib, n - j)
        assert close(np.triu(T[:sb, j:j + sb]), np.triu(Tg[:sb, j:j + sb]))


@pytest.mark.parametrize("n,ib", [(16, 4), (24, 8), (32, 8), (48, 16), (256, 32)])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_ttmqr_on_tt_factor_matches_dtpmqrt(oracle, golden, n, ib, trans):
    key = f"ttqrt_{n}_{ib}"
    V = golden[key + "_outA2"]
    T = np.array(golden[key + "_outT"], order="F")
    C1 = np.array(golden[f"{key}_L{trans}_C1"], order="F")
    C2 = np.array(golden[f"{key}_L{trans}_C2"], order="F")
    oracle.ttmqr("L", trans, n, 40, n, 40, n, ib, C1, C2, np.array(V, order="F"), T, np.zeros(ib * 40))
    assert close(C1, golden[f"{key}_L{trans}_out1"])
    assert close(C2, golden[f"{key}_L{trans}_out2"])


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_ttmqr_matches_reference_test_form(oracle, golden, side, trans):
    key = f"ttmqr_{side}{trans}"
    n, k, ib = 24, 16, 8
    A1 = np.array(golden[key + "_A1"], order="F")
    A2 = np.array(golden[key + "_A2"], order="F")
    oracle.ttmqr(side, trans, n, n, n, n, k, ib, A1, A2, np.array(golden[key + "_V"], order="F"),
                 np.array(golden[key + "_T"], order="F"), np.zeros(ib * n))
    assert close(A1, golden[key + "_outA1"])
    assert close(A2, golden[key + "_outA2"])


def test_ttqrt_reads_only_the_upper_triangle(oracle):
    """Entries below A2's diagonal (geqrt's reflectors in a tree) change nothing."""
    rng = np.random.default_rng(3)
    n, ib = 40, 8
    A1 = np.asfortranarray(np.triu(rng.standard_normal((n, n))) + 2 * np.eye(n))
    A2 = np.asfortranarray(np.triu(rng.standard_normal((n, n))) + 2 * np.eye(n))
    junk = np.asfortranarray(np.tril(rng.standard_normal((n, n)), -1))
    outs = []
    for B in (A2, A2 + junk):
        a1, a2 = A1.copy(order="F"), B.copy(order="F")
        T = np.zeros((ib, n), order="F")
        oracle.ttqrt(n, n, ib, a1, a2, T, np.zeros(n), np.zeros(ib * n))
        C1 = np.asfortranarray(rng.standard_normal((n, 9)))
        C2 = np.asfortranarray(rng.standard_normal((n, 9)))
        C1c, C2c = C1.copy(order="F"), C2.copy(order="F")
        outs.append((a1, np.triu(a2), T, C1c, C2c, a2))
    (a, b, t, _, _, v0), (a_, b_, t_, _, _, v1) = outs
    assert np.array_equal(a, a_) and np.array_equal(b, b_) and np.array_equal(t, t_)
    assert np.array_equal(np.tril(v1, -1), junk)          # the lower part is left as it was
    rng2 = np.random.default_rng(4)
    C1 = np.asfortranarray(rng2.standard_normal((n, 9)))
    C2 = np.asfortranarray(rng2.standard_normal((n, 9)))
    res = []
    for V in (v0, v1):
        c1, c2 = C1.copy(order="F"), C2.copy(order="F")
        oracle.ttmqr("L", "C", n, 9, n, 9, n, ib, c1, c2, V, t, np.zeros(ib * 9))
        res.append((c1, c2))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("m,n,ib", [(32, 16, 4), (48, 24, 8), (64, 32, 16), (16, 32, 4), (24, 48, 8)])
def test_ttqrt_rectangular_tiles(oracle, m, n, ib):
    """test/ttqrt.jl:76-150: finite results and A1's strictly lower part untouched."""
    rng = np.random.default_rng(m + n)
    k = min(m, n)
    A1 = np.asfortranarray(np.triu(rng.standard_normal((m, n))))
    A2 = np.asfortranarray(np.triu(rng.standard_normal((m, n))))
    A1[np.arange(k), np.arange(k)] += 2
    A2[np.arange(k), np.arange(k)] += 2
    T = np.zeros((ib, k), order="F")
    oracle.ttqrt(m, n, ib, A1, A2, T, np.zeros(k), np.zeros(ib * n))
    assert np.isfinite(A1).all() and np.isfinite(A2).all() and np.isfinite(T).all()
    assert np.abs(np.tril(A1[:k, :k], -1)).max() < 1e-10


def test_tt_argument_errors(oracle):
    z = np.zeros((8, 8), order="F")
    with pytest.raises(ValueError):
        oracle.ttmqr("X", "N", 8, 8, 8, 8, 4, 2, z, z.copy(order="F"), z[:, :4], z[:2, :4], np.zeros(16))
    with pytest.raises(ValueError):
        oracle.ttmqr("L", "X", 8, 8, 8, 8, 4, 2, z, z.copy(order="F"), z[:, :4], z[:2, :4], np.zeros(16))
    with pytest.raises(ValueError):
        oracle.ttqrt(-1, 8, 2, z, z.copy(order="F"), z[:2], np.zeros(8), np.zeros(16))
    with pytest.raises(ValueError):
        oracle.parfb_l("L", "C", 4, 8, 8, 8, 4, 5, z, z.copy(order="F"), z[:, :4], z[:4, :4], z)
    # k = 0 is a no-op (test/ttmqr.jl:169-179)
    A1 = np.asfortranarray(np.random.default_rng(0).random((8, 8)))
    A2 = A1.copy(order="F")
    oracle.ttmqr("L", "N", 8, 8, 8, 8, 0, 0, A1, A2, z[:, :1], z[:1, :1], np.zeros(1))
    assert np.array_equal(A1, A2)


@pytest.mark.parametrize("m,n,nb,ib", [(1024, 256, 128, 32), (1000, 300, 128, 16), (1024, 64, 32, 8),
                                       (300, 300, 128, 32), (517, 130, 64, 16), (130, 130, 64, 16),
                                       (260, 129, 64, 16), (64, 200, 32, 8)])
def test_tree_tile_qr_properties(oracle, m, n, nb, ib):
    rng = np.random.default_rng(m * 7 + n)
    A0 = np.asfortranarray(rng.standard_normal((m, n)))
    A = A0.copy(order="F")
    T, tau, T2, tau2 = oracle.tile_geqrf_tree(A, nb, ib)
    k = min(m, n)
    R = np.triu(A[:k, :])
    Q = np.asfortranarray(np.eye(m, k))
    oracle.tile_unmqr_tree("N", A, T, T2, Q, nb, ib)
    assert np.linalg.norm(Q @ R - A0) <= 1e-14 * np.linalg.norm(A0) * k
    assert np.linalg.norm(Q.T @ Q - np.eye(k)) <= 1e-14 * k
    QtA = A0.copy(order="F")
    oracle.tile_unmqr_tree("C", A, T, T2, QtA, nb, ib)
    assert np.linalg.norm(QtA[:k] - R) <= 1e-14 * np.linalg.norm(R) * k
    assert np.linalg.norm(QtA[k:]) <= 1e-14 * np.linalg.norm(A0) * k
    # R is unique up to the signs of its rows
    Rl = np.linalg.qr(A0, mode="r")
    assert np.linalg.norm(np.abs(R) - np.abs(Rl)) <= 1e-12 * np.linalg.norm(Rl) * k


# ---- hierarchical tree (groups reduced flat, leaders by the binary tree) ----
@pytest.mark.parametrize("m,n,nb,ib,grp", [(1024, 256, 128, 32, 2), (1000, 300, 128, 16, 3), (2048, 256, 128, 32, 4),
                                           (1800, 512, 256, 32, 2), (517, 130, 64, 16, 3), (300, 400, 256, 32, 2),
                                           (1024, 256, 128, 32, 8), (1024, 256, 128, 32, 100)])
def test_hqr_properties(oracle, m, n, nb, ib, grp):
    """Q^T A = [R; 0], Q Q^T = I through the stored factors, |R| equal to the
    flat tree's, and grp = 1 identical to the binary tree."""
    rng = np.random.default_rng(m + n + grp)
    A0 = np.asfortranarray(rng.standard_normal((m, n)))
    A = A0.copy(order="F")
    T, tau, T2, tau2 = oracle.tile_geqrf_hqr(A, nb, ib, grp)
    k = min(m, n)
    R = np.triu(A[:k])
    B = A0.copy(order="F")
    oracle.tile_unmqr_hqr("C", A, T, T2, B, nb, ib, grp)
    assert np.linalg.norm(B[:k] - R) <= 1e-13 * np.linalg.norm(R) * k
    assert np.linalg.norm(B[k:]) <= 1e-13 * np.linalg.norm(A0) * k
    C0 = np.asfortranarray(rng.standard_normal((m, 5)))
    C = C0.copy(order="F")
    oracle.tile_unmqr_hqr("N", A, T, T2, C, nb, ib, grp)
    oracle.tile_unmqr_hqr("C", A, T, T2, C, nb, ib, grp)
    assert np.abs(C - C0).max() < 1e-13 * m
    F = A0.copy(order="F")
    oracle.tile_geqrf(F, nb, ib)
    assert np.allclose(np.abs(R), np.abs(np.triu(F[:k])), atol=1e-11 * np.abs(R).max())


def test_hqr_group_one_is_the_binary_tree(oracle):
    rng = np.random.default_rng(9)
    A0 = np.asfortranarray(rng.standard_normal((1000, 300)))
    A1, A2 = A0.copy(order="F"), A0.copy(order="F")
    r1 = oracle.tile_geqrf_tree(A1, 128, 16)
    r2 = oracle.tile_geqrf_hqr(A2, 128, 16, 1)
    assert np.array_equal(A1, A2)
    for a, b in zip(r1, r2):
        assert np.array_equal(a, b)
