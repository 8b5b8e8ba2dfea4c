"""The CPU FP64 reference adjoint of the thin QR, pinned by central differences.

The reference forward is the oracle's flat-tree tile QR (NextLA's geqrt!/
tsqrt!/unmqr! restated in C) with the explicit Q formed by the tile Q
application; the reference adjoint is the published thin-QR pullback.  The
scalar checked is f(A) = 1/2 ||R^-1 Q^T b - y||^2 + <dQ, Q> + <dR, R> with
seeded b, y, dQ, dR, along random directions E with h = 1e-6.
"""
import numpy as np
import pytest


def loss(oracle, A, b, y, dQ, dR, nb, ib):
    Q, R, _ = oracle.qr_explicit(A, nb, ib)
    return oracle.ls_loss_cotangents(Q, R, b, y, dQ, dR)[0]


@pytest.mark.parametrize("m,n,nb,ib", [(40, 12, 16, 4), (64, 32, 32, 8), (37, 37, 16, 4), (300, 64, 256, 32),
                                       (520, 96, 256, 32)])
def test_reference_adjoint_matches_central_differences(oracle, m, n, nb, ib):
    rng = np.random.default_rng(m * 1000 + n)
    A = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    y = rng.standard_normal(n)
    dQ = rng.standard_normal((m, n))
    dR = rng.standard_normal((n, n))
    Q, R, _ = oracle.qr_explicit(A, nb, ib)
    assert np.linalg.norm(Q @ R - A) <= 1e-13 * np.linalg.norm(A) * n
    assert np.linalg.norm(Q.T @ Q - np.eye(n)) <= 1e-13 * n
    _, Qb, Rb = oracle.ls_loss_cotangents(Q, R, b, y, dQ, dR)
    Ab = oracle.qr_adjoint(Q, R, Qb, Rb)
    h = 1e-6
    for _ in range(3):
        E = rng.standard_normal((m, n))
        fd = (loss(oracle, A + h * E, b, y, dQ, dR, nb, ib) - loss(oracle, A - h * E, b, y, dQ, dR, nb, ib)) / (2 * h)
        an = float(np.sum(Ab * E))
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


def test_reference_adjoint_of_q_and_r_separately(oracle):
    """Cotangents on Q alone and on R alone (the loss-free pullbacks)."""
    rng = np.random.default_rng(7)
    m, n, nb, ib = 90, 20, 32, 8
    A = rng.standard_normal((m, n))
    dQ = rng.standard_normal((m, n))
    dR = np.triu(rng.standard_normal((n, n)))
    E = rng.standard_normal((m, n))
    h = 1e-6
    Q, R, _ = oracle.qr_explicit(A, nb, ib)
    for Qb, Rb, fn in ((dQ, np.zeros((n, n)), lambda Q_, R_: np.sum(dQ * Q_)),
                       (np.zeros((m, n)), dR, lambda Q_, R_: np.sum(dR * R_))):
        Ab = oracle.qr_adjoint(Q, R, Qb, Rb)
        fp = fn(*oracle.qr_explicit(A + h * E, nb, ib)[:2])
        fm = fn(*oracle.qr_explicit(A - h * E, nb, ib)[:2])
        fd = (fp - fm) / (2 * h)
        an = float(np.sum(Ab * E))
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


@pytest.mark.parametrize("m,n,nb,ib", [(48, 20, 16, 4), (31, 30, 32, 8), (70, 9, 32, 4)])
def test_complex_reference_adjoint_matches_central_differences(oracle, m, n, nb, ib):
    """The complex pullback (R's diagonal real): Abar = (Qbar + Q X) R^-H with
    X = tril(M,-1) + tril(M,-1)^H + Re diag(M), M = R Rbar^H - Qbar^H Q, the
    gradient of a real loss as dL/dRe(A) + i dL/dIm(A), against central
    differences in the real and the imaginary direction of every entry of A
    for L = Re<dQ, Q> + Re<dR, R> through the complex tile QR; m > n, so every
    column has a reflector and R's diagonal is real."""
    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    dQ = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    dR = np.triu(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))

    def L(A_):
        Q_, R_, _ = oracle.qr_explicit(A_, nb, ib)
        return float(np.real(np.vdot(dQ, Q_)) + np.real(np.vdot(dR, R_)))

    Q, R, _ = oracle.qr_explicit(A, nb, ib)
    assert np.abs(R.diagonal().imag).max() == 0.0
    Ab = oracle.qr_adjoint(Q, R, dQ, dR)
    h = 1e-6
    G = np.zeros_like(A)
    for i in range(m):
        for j in range(n):
            E = np.zeros_like(A)
            E[i, j] = h
            G[i, j] = (L(A + E) - L(A - E)) / (2 * h) + 1j * (L(A + 1j * E) - L(A - 1j * E)) / (2 * h)
    assert np.abs(G - Ab).max() <= 1e-6 * np.abs(G).max()


def test_complex_reference_adjoint_refuses_square(oracle):
    """A square complex matrix: the one-row last column keeps tau = 0
    (src/geqr2.jl:32-35), so R[n-1, n-1] stays complex and the Re-diagonal
    gauge term does not describe it; the reference pullback refuses, as the
    GPU backward does (argument error -2)."""
    rng = np.random.default_rng(9)
    A = rng.standard_normal((12, 12)) + 1j * rng.standard_normal((12, 12))
    Q, R, _ = oracle.qr_explicit(A, 32, 4)
    assert abs(R[-1, -1].imag) > 0.0
    assert np.abs(R.diagonal()[:-1].imag).max() == 0.0
    with pytest.raises(ValueError):
        oracle.qr_adjoint(Q, R, np.zeros_like(Q), np.zeros_like(R))
