"""Parity of the triangle-on-triangle kernels (ttqrt!, ttmqr!, parfb! with
l > 0) with the oracle and the LAPACK golden vectors.

Bars as for the other kernels: FP64 relative max-abs difference <= 1e-12
(test/lapack_helpers.jl:14), FP32 1e-5.  Shapes follow test/ttqrt.jl and
test/ttmqr.jl, plus the 256/32 tile the tree factorisation uses.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def F(a):
    return np.array(a, dtype=np.float64, order="F")


def dev(tq, a, dtype=None):
    import torch
    return tq.to_device(a, dtype=dtype or torch.float64)


def host(tq, t):
    return tq.to_numpy(t).astype(np.float64)


@pytest.mark.parametrize("n,ib", [(16, 4), (24, 8), (32, 8), (48, 16), (256, 32)])
def test_ttqrt_golden_and_oracle(tq, oracle, golden, n, ib):
    key = f"ttqrt_{n}_{ib}"
    A1h, A2h = F(golden[key + "_A1"]), F(golden[key + "_A2"])
    A1, A2, T, tau = dev(tq, A1h), dev(tq, A2h), tq.zeros(ib, n), dev(tq, np.zeros(n))
    tq.ttqrt(n, n, ib, A1, A2, T, tau, None)
    o1, o2, To, tauo = A1h.copy(order="F"), A2h.copy(order="F"), np.zeros((ib, n), order="F"), np.zeros(n)
    oracle.ttqrt(n, n, ib, o1, o2, To, tauo, np.zeros(ib * n))
    assert rel(host(tq, A1), o1) < RTOL and rel(host(tq, A2), o2) < RTOL
    assert rel(host(tq, T), To) < RTOL and rel(host(tq, tau), tauo) < RTOL
    assert rel(host(tq, A1), golden[key + "_outA1"]) < RTOL
    assert rel(host(tq, A2), golden[key + "_outA2"]) < RTOL


@pytest.mark.parametrize("n,ib", [(24, 8), (256, 32)])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_ttmqr_on_tt_factor_golden(tq, golden, n, ib, trans):
    key = f"ttqrt_{n}_{ib}"
    V, T = dev(tq, golden[key + "_outA2"]), dev(tq, golden[key + "_outT"])
    C1, C2 = dev(tq, golden[f"{key}_L{trans}_C1"]), dev(tq, golden[f"{key}_L{trans}_C2"])
    tq.ttmqr("L", trans, n, 40, n, 40, n, ib, C1, C2, V, T, None)
    assert rel(host(tq, C1), golden[f"{key}_L{trans}_out1"]) < RTOL
    assert rel(host(tq, C2), golden[f"{key}_L{trans}_out2"]) < RTOL


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_ttmqr_reference_form_golden(tq, oracle, golden, side, trans):
    key = f"ttmqr_{side}{trans}"
    n, k, ib = 24, 16, 8
    A1, A2 = dev(tq, golden[key + "_A1"]), dev(tq, golden[key + "_A2"])
    tq.ttmqr(side, trans, n, n, n, n, k, ib, A1, A2, dev(tq, golden[key + "_V"]), dev(tq, golden[key + "_T"]),
             None)
    assert rel(host(tq, A1), golden[key + "_outA1"]) < RTOL
    assert rel(host(tq, A2), golden[key + "_outA2"]) < RTOL


@pytest.mark.parametrize("m,n,ib", [(32, 16, 4), (48, 24, 8), (64, 32, 16), (16, 32, 4), (24, 48, 8),
                                    (300, 256, 32), (256, 100, 32)])
def test_ttqrt_rectangular_and_lower_part_untouched(tq, oracle, m, n, ib):
    """test/ttqrt.jl:76-150 shapes against the oracle, with junk below A2's
    diagonal (geqrt's reflectors in a tree) that must be neither read nor
    written."""
    rng = np.random.default_rng(m * 100 + n)
    k = min(m, n)
    A1h = F(np.triu(rng.standard_normal((m, n))))
    A2h = F(np.triu(rng.standard_normal((m, n))))
    A1h[np.arange(k), np.arange(k)] += 2
    A2h[np.arange(k), np.arange(k)] += 2
    junk = F(np.tril(rng.standard_normal((m, n)), -1))
    A1, A2, T, tau = dev(tq, A1h), dev(tq, A2h + junk), tq.zeros(ib, k), dev(tq, np.zeros(k))
    tq.ttqrt(m, n, ib, A1, A2, T, tau, None)
    o1, o2, To, tauo = A1h.copy(order="F"), A2h.copy(order="F"), np.zeros((ib, k), order="F"), np.zeros(k)
    oracle.ttqrt(m, n, ib, o1, o2, To, tauo, np.zeros(ib * n))
    g2 = host(tq, A2)
    assert np.array_equal(np.tril(g2, -1), junk)
    assert rel(host(tq, A1), o1) < RTOL and rel(np.triu(g2), o2) < RTOL
    assert rel(host(tq, T), To) < RTOL and rel(host(tq, tau), tauo) < RTOL


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
@pytest.mark.parametrize("n,k,ib", [(24, 16, 8), (256, 256, 32), (64, 50, 16)])
def test_ttmqr_vs_oracle_with_junk_below(tq, oracle, side, trans, n, k, ib):
    rng = np.random.default_rng(n + k)
    A1h, A2h = F(rng.standard_normal((n, n))), F(rng.standard_normal((n, n)))
    Vh = F(np.triu(rng.standard_normal((n, k))))
    junk = F(np.tril(rng.standard_normal((n, k)), -1))
    Th = F(np.triu(rng.random((ib, k))) / 4)
    A1, A2 = dev(tq, A1h), dev(tq, A2h)
    tq.ttmqr(side, trans, n, n, n, n, k, ib, A1, A2, dev(tq, Vh + junk), dev(tq, Th), None)
    o1, o2 = A1h.copy(order="F"), A2h.copy(order="F")
    oracle.ttmqr(side, trans, n, n, n, n, k, ib, o1, o2, Vh, Th, np.zeros(ib * n))
    assert rel(host(tq, A1), o1) < RTOL and rel(host(tq, A2), o2) < RTOL


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("l", [0, 3, 8])
def test_parfb_triangular_part(tq, oracle, side, l):
    rng = np.random.default_rng(l + (side == "L"))
    m1, n1, m2, n2, k = (8, 20, 14, 20, 8) if side == "L" else (20, 8, 20, 14, 8)
    A1h, A2h = F(rng.standard_normal((m1, n1))), F(rng.standard_normal((m2, n2)))
    Vh = F(rng.standard_normal((m2 if side == "L" else n2, k)))
    Th = F(np.triu(rng.random((k, k))) / 4)
    for trans in "NC":
        A1, A2 = dev(tq, A1h), dev(tq, A2h)
        tq.parfb(side, trans, "F", "C", m1, n1, m2, n2, k, l, A1, A2, dev(tq, Vh), dev(tq, Th), None)
        o1, o2 = A1h.copy(order="F"), A2h.copy(order="F")
        oracle.parfb_l(side, trans, m1, n1, m2, n2, k, l, o1, o2, Vh, Th, np.zeros((20, 20), order="F"))
        assert rel(host(tq, A1), o1) < RTOL and rel(host(tq, A2), o2) < RTOL


def test_tt_argument_errors_and_noops(tq):
    """test/ttmqr.jl:169-187 and test/ttqrt.jl argument checks."""
    z = tq.zeros(8, 8)
    with pytest.raises(tq.ArgumentError):
        tq.ttmqr("X", "N", 8, 8, 8, 8, 4, 2, z, tq.zeros(8, 8), tq.zeros(8, 4), tq.zeros(2, 4), None)
    with pytest.raises(tq.ArgumentError):
        tq.ttmqr("L", "X", 8, 8, 8, 8, 4, 2, z, tq.zeros(8, 8), tq.zeros(8, 4), tq.zeros(2, 4), None)
    with pytest.raises(tq.ArgumentError):
        tq.ttqrt(-1, 8, 2, z, tq.zeros(8, 8), tq.zeros(2, 8), dev(tq, np.zeros(8)), None)
    with pytest.raises(tq.ArgumentError):
        tq.parfb("L", "C", "F", "C", 4, 8, 8, 8, 4, 5, tq.zeros(4, 8), tq.zeros(8, 8), tq.zeros(8, 4),
                 tq.zeros(4, 4), None)
    rng = np.random.default_rng(0)
    A1h = F(rng.random((8, 8)))
    A1, A2 = dev(tq, A1h), dev(tq, A1h)
    tq.ttmqr("L", "N", 8, 8, 8, 8, 0, 0, A1, A2, tq.zeros(8, 1), tq.zeros(1, 1), None)
    assert np.array_equal(host(tq, A1), A1h) and np.array_equal(host(tq, A2), A1h)


def test_tt_helpers_and_float(tq, oracle):
    """The allocating helpers equal the kernels; FP32 within 1e-5."""
    import torch
    rng = np.random.default_rng(9)
    n, ib = 24, 8
    A1h = F(np.triu(rng.standard_normal((n, n))) + np.eye(n))
    A2h = F(np.triu(rng.standard_normal((n, n))) + np.eye(n))
    h1, h2, hT = dev(tq, A1h), dev(tq, A2h), tq.zeros(ib, n)
    tq.ttqrt(h1, h2, hT)
    k1, k2, kT, kt = dev(tq, A1h), dev(tq, A2h), tq.zeros(ib, n), dev(tq, np.zeros(n))
    tq.ttqrt(n, n, ib, k1, k2, kT, kt, None)
    assert rel(host(tq, h1), host(tq, k1)) == 0 and rel(host(tq, h2), host(tq, k2)) == 0
    C1h, C2h = F(rng.standard_normal((n, n))), F(rng.standard_normal((n, n)))
    c1, c2 = dev(tq, C1h), dev(tq, C2h)
    tq.ttmqr("L", "N", c1, c2, k2, kT)
    d1, d2 = dev(tq, C1h), dev(tq, C2h)
    tq.ttmqr("L", "N", n, n, n, n, n, ib, d1, d2, k2, kT, None)
    assert rel(host(tq, c1), host(tq, d1)) == 0
    f1, f2 = dev(tq, A1h, torch.float32), dev(tq, A2h, torch.float32)
    fT, ft = tq.zeros(ib, n, dtype=torch.float32), dev(tq, np.zeros(n), torch.float32)
    tq.ttqrt(n, n, ib, f1, f2, fT, ft, None)
    o1, o2 = A1h.copy(order="F"), A2h.copy(order="F")
    oracle.ttqrt(n, n, ib, o1, o2, np.zeros((ib, n), order="F"), np.zeros(n), np.zeros(ib * n))
    assert rel(host(tq, f1), o1) < 1e-5 and rel(host(tq, f2), o2) < 1e-5
