"""The oracle's pamm! (every op / side / storev / direct form, real and
complex) against its definition written with numpy, and, for the columnwise
forward forms parfb! uses, the W / T / A1 / A sequence against the oracle's
parfb!, which the LAPACK golden vectors pin (src/pamm.jl:49-473,
src/parfb.jl:121-137)."""
import itertools

import numpy as np
import pytest

FORMS = list(itertools.product("WA", "LR", "CR", "FB"))


def F(a, dt):
    return np.array(a, dtype=dt, order="F")


def masked_ve(V, storev, direct, mv, k, l):
    Ve = np.array(V if storev == "C" else V.T, dtype=V.dtype)[:mv, :k].copy()
    for r in range(mv):
        for p in range(k):
            if direct == "F":
                bad = p < l and r >= mv - l and r - (mv - l) > p
            else:
                bad = p >= k - l and r < l and r < p - (k - l)
            if bad:
                Ve[r, p] = 0
    return Ve


def reference(op, side, storev, direct, m, n, k, l, A1, A2, V, W):
    L = side == "L"
    mv = m if L else n
    Ve = masked_ve(V, storev, direct, mv, k, l)
    cjw = (L and storev == "C") or (not L and storev == "R")
    cja = (L and storev == "R") or (not L and storev == "C")
    A2, W = A2.copy(), W.copy()
    if op == "W":
        f = Ve.conj() if cjw else Ve
        if L:
            W[:k, :n] = A1[:k, :n] + f.T @ A2[:m, :n]
        else:
            W[:m, :k] = A1[:m, :k] + A2[:m, :n] @ f
        return A2, W
    g = Ve.conj() if cja else Ve
    if L:
        A2[:m, :n] -= g @ W[:k, :n]
    else:
        A2[:m, :n] -= W[:m, :k] @ g.T
    b0 = 0 if direct == "F" else k - l
    rows = [(mv - l + t) if direct == "F" else t for t in range(l)]
    tri = g[rows, b0:b0 + l] if l else np.zeros((0, 0), dtype=g.dtype)
    if L:
        W[b0:b0 + l, :n] = tri @ W[b0:b0 + l, :n]
    else:
        W[:m, b0:b0 + l] = W[:m, b0:b0 + l] @ tri.T
    return A2, W


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("op,side,storev,direct", FORMS)
@pytest.mark.parametrize("l", [0, 3, 8])
def test_pamm_matches_definition(oracle, dt, op, side, storev, direct, l):
    rng = np.random.default_rng(hash((op, side, storev, direct, l)) % 2**32)
    m, n, k = 13, 11, 8
    mv = m if side == "L" else n
    cplx = np.iscomplexobj(np.zeros(1, dt))
    R = lambda *s: F(rng.standard_normal(s) + (1j * rng.standard_normal(s) if cplx else 0), dt)
    A1 = R(k, n) if side == "L" else R(m, k)
    A2 = R(m, n)
    V = R(mv, k) if storev == "C" else R(k, mv)
    W = R(k, n) if side == "L" else R(m, k)
    A2r, Wr = reference(op, side, storev, direct, m, n, k, l, A1, A2, V, W)
    A2o, Wo = A2.copy(order="F"), W.copy(order="F")
    oracle.pamm(op, side, storev, direct, m, n, k, l, A1, A2o, V, Wo)
    assert np.abs(A2o - A2r).max() <= 1e-13 * max(1.0, np.abs(A2r).max())
    assert np.abs(Wo - Wr).max() <= 1e-13 * max(1.0, np.abs(Wr).max())


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("side", "LR")
@pytest.mark.parametrize("trans", "NC")
@pytest.mark.parametrize("l", [0, 4, 6])
def test_pamm_sequence_is_parfb(oracle, dt, side, trans, l):
    """parfb! = pamm 'W', W := op(T) W (or W op(T)), A1 -= W, pamm 'A'."""
    rng = np.random.default_rng(11 + l)
    cplx = np.iscomplexobj(np.zeros(1, dt))
    R = lambda *s: F(rng.standard_normal(s) + (1j * rng.standard_normal(s) if cplx else 0), dt)
    k = 6
    if side == "L":
        m1, n1, m2, n2 = 9, 7, 10, 7
    else:
        m1, n1, m2, n2 = 8, 9, 8, 10
    A1, A2 = R(m1, n1), R(m2, n2)
    V = R(m2 if side == "L" else n2, k)
    T = F(np.triu(R(k, k)), dt)
    B1, B2 = A1.copy(order="F"), A2.copy(order="F")
    oracle.parfb_l(side, trans, m1, n1, m2, n2, k, l, B1, B2, V, T, np.zeros((max(m1, m2), max(n1, n2)), dt, order="F"))
    W = np.zeros((k, n2) if side == "L" else (m2, k), dt, order="F")
    oracle.pamm("W", side, "C", "F", m2, n2, k, l, A1, A2, V, W)
    if side == "L":
        opT = T if trans == "N" else T.conj().T
        W = F(opT @ W, dt)
        A1[:k] -= W
    else:
        opT = T if trans == "N" else T.conj().T
        W = F(W @ opT, dt)
        A1[:, :k] -= W
    oracle.pamm("A", side, "C", "F", m2, n2, k, l, None, A2, V, W)
    assert np.abs(A1 - B1).max() <= 1e-13 * np.abs(B1).max()
    assert np.abs(A2 - B2).max() <= 1e-13 * np.abs(B2).max()


def test_pamm_quick_return_and_errors(oracle):
    """test/pamm.jl: zero dimensions leave W untouched; bad flags and
    negative sizes are argument errors."""
    rng = np.random.default_rng(1)
    A1, A2 = F(rng.random((5, 5)), np.complex128), F(rng.random((10, 5)), np.complex128)
    V, W = F(rng.random((10, 5)), np.complex128), F(rng.random((5, 5)), np.complex128)
    W0 = W.copy()
    for (m, n, k) in [(0, 5, 5), (10, 0, 5), (10, 5, 0)]:
        oracle.pamm("W", "L", "C", "F", m, n, k, 3, A1, A2, V, W)
        assert np.array_equal(W, W0)
    for args in [("X", "L", "C", "F", 10, 5, 5, 3), ("W", "X", "C", "F", 10, 5, 5, 3),
                 ("W", "L", "X", "F", 10, 5, 5, 3), ("W", "L", "C", "X", 10, 5, 5, 3),
                 ("W", "L", "C", "F", -1, 5, 5, 3), ("W", "L", "C", "F", 10, 5, 5, -1),
                 ("W", "L", "C", "F", 10, 5, 5, 6)]:
        with pytest.raises(ValueError):
            oracle.pamm(*args, A1, A2, V, W)


def explicit_tprfb(side, trans, direct, storev, k, l, V, T, A1, A2):
    """[A1; A2] := op(H) [A1; A2] (side L) or [A1 A2] op(H) (R) with the
    pentagonal block reflector H = I - Vf T Vf^H (columnwise: Vf = [I; Ve]) or
    I - Vf^H T Vf (rowwise: Vf = [I Ve^T]), T's upper ('F') or lower ('B')
    triangle, V's trapezoid of order l -- LAPACK's tprfb, which the reference
    tests parfb! against (test/parfb.jl:44-51)."""
    L = side == "L"
    mv = A2.shape[0] if L else A2.shape[1]
    Ve = masked_ve(V, storev, direct, mv, k, l)
    Tt = np.triu(T[:k, :k]) if direct == "F" else np.tril(T[:k, :k])
    Vc = np.vstack([np.eye(k, dtype=Ve.dtype), Ve])           # columnwise reflectors
    if storev == "C":
        H = np.eye(k + mv, dtype=Ve.dtype) - Vc @ Tt @ Vc.conj().T
    else:
        Vr = Vc.T                                               # rows [I V]: V is stored rowwise
        H = np.eye(k + mv, dtype=Ve.dtype) - Vr.conj().T @ Tt @ Vr
    op = H if trans == "N" else H.conj().T
    if L:
        X = op @ np.vstack([A1[:k], A2])
        return X[:k], X[k:]
    X = np.hstack([A1[:, :k], A2]) @ op
    return X[:, :k], X[:, k:]


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("side", "LR")
@pytest.mark.parametrize("trans", "NC")
@pytest.mark.parametrize("direct", "FB")
@pytest.mark.parametrize("storev", "CR")
def test_parfb_every_form_vs_explicit_reflector(oracle, dt, side, trans, direct, storev):
    """test/parfb.jl's shapes (m2, n2, k, l = 20, 24, 8, 4, T = rand(k, k))."""
    rng = np.random.default_rng(hash((side, trans, direct, storev)) % 2**32)
    cplx = np.iscomplexobj(np.zeros(1, dt))
    R = lambda *s: F(rng.random(s) + (1j * rng.random(s) if cplx else 0), dt)
    m2, n2, k, l = 20, 24, 8, 4
    m1, n1 = (k, n2) if side == "L" else (m2, k)
    A1, A2 = R(m1, n1), R(m2, n2)
    mv = m2 if side == "L" else n2
    V = R(mv, k) if storev == "C" else R(k, mv)
    T = R(k, k)
    W = np.zeros((k, n2) if side == "L" else (m2, k), dt, order="F")
    X1, X2 = explicit_tprfb(side, trans, direct, storev, k, l, V, T, A1, A2)
    oracle.parfb_full(side, trans, direct, storev, m1, n1, m2, n2, k, l, A1, A2, V, T, W)
    assert np.abs(A1 - X1).max() <= 1e-12 * np.abs(X1).max()
    assert np.abs(A2 - X2).max() <= 1e-12 * np.abs(X2).max()
