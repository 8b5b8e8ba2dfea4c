"""Parity of every CUDA tile kernel with the CPU oracle and the LAPACK golden vectors.

Each test runs the kernel through the C ABI (tileqr front end -> libtileqr.so)
and the oracle on the same seeded inputs.  FP64 bar: relative difference
(max-abs, relative to the oracle's max-abs entry) <= 1e-12, the reference's own
test tolerance (test/lapack_helpers.jl:14).  FP32 variants: 1e-5 against the
float64 oracle scaled by the problem size, the reference's single-precision rtol.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RTOL32 = 1e-5


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def F(a):
    return np.array(a, dtype=np.float64, order="F")


def dev(tq, a, dtype=None):
    import torch
    return tq.to_device(a, dtype=dtype or torch.float64)


def host(tq, t):
    return tq.to_numpy(t).astype(np.float64)


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("m,n,ib", [(20, 15, 4), (32, 32, 8), (64, 32, 16), (32, 64, 8), (256, 256, 32)])
def test_geqrt(tq, oracle, golden, m, n, ib):
    key = f"geqrt_{m}_{n}_{ib}"
    A0 = F(golden[key + "_A"])
    k = min(m, n)
    A, T, tau = dev(tq, A0), tq.zeros(ib, k), dev(tq, np.zeros(k))
    tq.geqrt(m, n, ib, A, T, tau, None)
    Ao, To, tauo = A0.copy(order="F"), np.zeros((ib, k), order="F"), np.zeros(k)
    oracle.geqrt(m, n, ib, Ao, To, tauo, np.zeros(ib * n))
    assert rel(host(tq, A), Ao) < RTOL
    assert rel(host(tq, T), To) < RTOL
    assert rel(host(tq, tau), tauo) < RTOL
    assert rel(host(tq, A), golden[key + "_outA"]) < RTOL
    assert rel(host(tq, T), golden[key + "_outT"]) < 10 * RTOL


def test_geqrt_helper_and_ib1(tq, oracle):
    """test/geqrt.jl:34-71: helper equals kernel; ib = 1 equals geqr2."""
    rng = np.random.default_rng(5)
    A0 = F(rng.random((32, 24)))
    A1, T1 = dev(tq, A0), tq.zeros(8, 24)
    tq.geqrt(A1, T1)
    A2, T2, tau2 = dev(tq, A0), tq.zeros(8, 24), dev(tq, np.zeros(24))
    tq.geqrt(32, 24, 8, A2, T2, tau2, None)
    assert rel(host(tq, A1), host(tq, A2)) == 0.0
    assert rel(host(tq, T1), host(tq, T2)) == 0.0
    B0 = F(rng.random((16, 12)))
    Ab, Au = dev(tq, B0), dev(tq, B0)
    tq.geqrt(16, 12, 1, Ab, tq.zeros(1, 12), dev(tq, np.zeros(12)), None)
    tq.geqr2(16, 12, Au, dev(tq, np.zeros(12)), None)
    assert rel(host(tq, Ab), host(tq, Au)) < RTOL


@pytest.mark.parametrize("m,n", [(16, 12), (256, 32), (300, 40), (1500, 8)])
def test_geqr2(tq, oracle, m, n):
    rng = np.random.default_rng(m + n)
    A0 = F(rng.standard_normal((m, n)))
    A, tau = dev(tq, A0), dev(tq, np.zeros(min(m, n)))
    tq.geqr2(m, n, A, tau, None)
    Ao, tauo = A0.copy(order="F"), np.zeros(min(m, n))
    oracle.geqr2(m, n, Ao, tauo, np.zeros(n))
    assert rel(host(tq, A), Ao) < RTOL
    assert rel(host(tq, tau), tauo) < RTOL


@pytest.mark.parametrize("direct", ["F", "B"])
@pytest.mark.parametrize("storev", ["C", "R"])
@pytest.mark.parametrize("n,k", [(1, 1), (5, 3), (10, 4), (20, 8), (256, 32)])
def test_larft(tq, oracle, direct, storev, n, k):
    rng = np.random.default_rng(n * 7 + k)
    V0 = F(rng.standard_normal((n, k) if storev == "C" else (k, n)))
    if n > 3:
        if storev == "C":
            V0[-2:, -1] = 0.0          # trailing zeros exercise the lastv scan
        else:
            V0[-1, -2:] = 0.0
    tau0 = rng.standard_normal(k)
    tau0[k // 2] = 0.0 if k > 2 else tau0[k // 2]
    V, tau, T = dev(tq, V0), dev(tq, tau0), tq.zeros(k, k)
    tq.larft(direct, storev, n, k, V, tau, T)
    To = np.zeros((k, k), order="F")
    oracle.larft(direct, storev, n, k, V0, tau0, To)
    assert rel(host(tq, T), To) < RTOL


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
@pytest.mark.parametrize("m,n,k", [(5, 4, 4), (10, 8, 4), (20, 15, 4), (256, 224, 32), (300, 100, 70)])
def test_larfb(tq, oracle, side, trans, m, n, k):
    rng = np.random.default_rng(m * 3 + n + k)
    rows = m if side == "L" else n
    k = min(k, rows)
    panel = F(rng.standard_normal((rows, k)))
    tau = np.zeros(k)
    oracle.geqr2(rows, k, panel, tau, np.zeros(k))
    T0 = np.zeros((k, k), order="F")
    oracle.larft("F", "C", rows, k, panel, tau, T0)
    C0 = F(rng.standard_normal((m, n)))
    C = dev(tq, C0)
    tq.larfb(side, trans, "F", "C", m, n, k, dev(tq, panel), rows, dev(tq, T0), C, None)
    Co = C0.copy(order="F")
    oracle.larfb(side, trans, "F", "C", m, n, k, panel, rows, T0, Co,
                 np.zeros((n if side == "L" else m, k), order="F"))
    assert rel(host(tq, C), Co) < RTOL


@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_unmqr_golden(tq, oracle, golden, st):
    Aq, Tq = F(golden["unmqr_Aqr"]), F(golden["unmqr_T"])
    C0 = F(golden[f"unmqr_{st}_C"])
    m, k = Aq.shape
    ib = Tq.shape[0]
    mm, nn = C0.shape
    C = dev(tq, C0)
    tq.unmqr(st[0], st[1], mm, nn, k, ib, dev(tq, Aq), m, dev(tq, Tq), C, None)
    assert rel(host(tq, C), golden[f"unmqr_{st}_out"]) < RTOL
    Co = C0.copy(order="F")
    oracle.unmqr(st[0], st[1], mm, nn, k, ib, Aq, m, Tq, Co,
                 np.zeros((nn if st[0] == "L" else mm, ib), order="F"))
    assert rel(host(tq, C), Co) < RTOL


def test_unmqr_orthogonality_and_clamp(tq):
    """test/unmqr.jl:69-78 (Q Q^H = I) and :81-107 (k clamped to nq)."""
    rng = np.random.default_rng(11)
    m, k, ib = 64, 32, 8
    A, T = dev(tq, rng.random((m, k))), tq.zeros(ib, k)
    tq.geqrt(m, k, ib, A, T, dev(tq, np.zeros(k)), None)
    C = dev(tq, np.eye(m))
    tq.unmqr("L", "N", m, m, k, ib, A, m, T, C, None)
    tq.unmqr("L", "C", m, m, k, ib, A, m, T, C, None)
    assert np.allclose(host(tq, C), np.eye(m), atol=1e-13)
    Aw, Tw = dev(tq, rng.random((16, 16))), tq.zeros(4, 16)
    tq.geqrt(16, 16, 4, Aw, Tw, dev(tq, np.zeros(16)), None)
    C0 = rng.random((16, 24))
    Cw = dev(tq, C0)
    tq.unmqr("L", "N", 16, 24, 32, 4, Aw, 16, Tw, Cw, None)     # k = 32 > nq = 16
    assert abs(np.linalg.norm(host(tq, Cw)) - np.linalg.norm(C0)) < 1e-12 * np.linalg.norm(C0)


@pytest.mark.parametrize("m,n,ib", [(32, 24, 8), (48, 32, 16), (64, 48, 16), (20, 20, 10), (256, 256, 32)])
def test_tsqrt(tq, oracle, golden, m, n, ib):
    key = f"tsqrt_{m}_{n}_{ib}"
    A10, A20 = F(golden[key + "_A1"]), F(golden[key + "_A2"])
    A1, A2, T, tau = dev(tq, A10), dev(tq, A20), tq.zeros(ib, n), dev(tq, np.zeros(n))
    tq.tsqrt(m, n, ib, A1, A2, T, tau, None)
    A1o, A2o, To, tauo = A10.copy(order="F"), A20.copy(order="F"), np.zeros((ib, n), order="F"), np.zeros(n)
    oracle.tsqrt(m, n, ib, A1o, A2o, To, tauo, np.zeros(ib * n))
    for got, want in ((A1, A1o), (A2, A2o), (T, To), (tau, tauo)):
        assert rel(host(tq, got), want) < RTOL
    assert rel(host(tq, A1), golden[key + "_outA1"]) < RTOL
    assert rel(host(tq, A2), golden[key + "_outA2"]) < RTOL
    assert rel(host(tq, T), golden[key + "_outT"]) < RTOL


@pytest.mark.parametrize("m1,m2,n,ib", [(32, 48, 16, 4), (64, 32, 32, 8), (16, 32, 32, 4), (24, 48, 48, 8)])
def test_tsqrt_rectangular_a1(tq, oracle, m1, m2, n, ib):
    """test/tsqrt.jl:75-156: tall and wide A1 (k = min(m1, n))."""
    rng = np.random.default_rng(m1 * m2 + n)
    k = min(m1, n)
    A10 = F(np.triu(rng.random((m1, n))))
    for i in range(k):
        A10[i, i] += 2.0
    A20 = F(rng.random((m2, n)))
    A1, A2, T, tau = dev(tq, A10), dev(tq, A20), tq.zeros(ib, k), dev(tq, np.zeros(k))
    tq.tsqrt(m2, n, ib, A1, A2, T, tau, None)
    A1o, A2o, To, tauo = A10.copy(order="F"), A20.copy(order="F"), np.zeros((ib, k), order="F"), np.zeros(k)
    oracle.tsqrt(m2, n, ib, A1o, A2o, To, tauo, np.zeros(ib * n))
    for got, want in ((A1, A1o), (A2, A2o), (T, To)):
        assert rel(host(tq, got), want) < RTOL


def test_tsqrt_zero_column_keeps_t(tq, oracle):
    """A zero A2 column gives tau = 0 and leaves its T column as it was (src/tsqrt.jl:61-64)."""
    rng = np.random.default_rng(2)
    n, m, ib = 16, 24, 8
    A10 = F(np.triu(rng.random((n, n))) + 2 * np.eye(n))
    A20 = F(rng.random((m, n)))
    A20[:, 0] = 0.0          # column 0 is the only one no earlier reflector touches
    T0 = F(np.full((ib, n), 7.0))
    A1, A2, T, tau = dev(tq, A10), dev(tq, A20), dev(tq, T0), dev(tq, np.zeros(n))
    tq.tsqrt(m, n, ib, A1, A2, T, tau, None)
    A1o, A2o, To, tauo = A10.copy(order="F"), A20.copy(order="F"), T0.copy(order="F"), np.zeros(n)
    oracle.tsqrt(m, n, ib, A1o, A2o, To, tauo, np.zeros(ib * n))
    assert host(tq, tau)[0] == 0.0 and tauo[0] == 0.0
    assert host(tq, T)[0, 0] == 7.0
    assert rel(host(tq, T), To) < RTOL
    assert rel(host(tq, A2), A2o) < RTOL


@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_tsmqr_golden(tq, oracle, golden, st):
    key = f"tsmqr_{st}"
    m1, n1, m2, n2, k, ib = (int(x) for x in golden[key + "_dims"])
    A10, A20 = F(golden[key + "_A1"]), F(golden[key + "_A2"])
    V0, T0 = F(golden[key + "_V"]), F(golden[key + "_T"])
    A1, A2 = dev(tq, A10), dev(tq, A20)
    tq.tsmqr(st[0], st[1], m1, n1, m2, n2, k, ib, A1, A2, dev(tq, V0), dev(tq, T0), None)
    assert rel(host(tq, A1), golden[key + "_outA1"]) < RTOL
    assert rel(host(tq, A2), golden[key + "_outA2"]) < RTOL
    A1o, A2o = A10.copy(order="F"), A20.copy(order="F")
    oracle.tsmqr(st[0], st[1], m1, n1, m2, n2, k, ib, A1o, A2o, V0, T0, np.zeros(ib * max(m1, n1)))
    assert rel(host(tq, A1), A1o) < RTOL
    assert rel(host(tq, A2), A2o) < RTOL


def test_tsmqr_tile_size_golden(tq, golden):
    A1, A2 = dev(tq, golden["tsmqr_big_A1"]), dev(tq, golden["tsmqr_big_A2"])
    tq.tsmqr("L", "C", 256, 128, 256, 128, 256, 32, A1, A2, dev(tq, golden["tsmqr_big_V"]),
             dev(tq, golden["tsmqr_big_T"]), None)
    assert rel(host(tq, A1), golden["tsmqr_big_outA1"]) < RTOL
    assert rel(host(tq, A2), golden["tsmqr_big_outA2"]) < RTOL


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_tsmqr_wide_band(tq, oracle, side, trans):
    """The tile driver calls tsmqr on whole row bands (n1 = many tiles)."""
    rng = np.random.default_rng(ord(side) + ord(trans))
    if side == "L":
        m1, n1, m2, k, ib = 256, 1000, 200, 256, 32
        n2 = n1
    else:
        m1, n1, n2, k, ib = 700, 256, 256, 256, 32
        m2 = m1
    A10, A20 = F(rng.standard_normal((m1, n1))), F(rng.standard_normal((m2, n2)))
    V0 = F(rng.standard_normal((m2 if side == "L" else n2, k)) / 8)
    T0 = F(np.triu(rng.standard_normal((ib, k))) / 8)
    A1, A2 = dev(tq, A10), dev(tq, A20)
    tq.tsmqr(side, trans, m1, n1, m2, n2, k, ib, A1, A2, dev(tq, V0), dev(tq, T0), None)
    A1o, A2o = A10.copy(order="F"), A20.copy(order="F")
    oracle.tsmqr(side, trans, m1, n1, m2, n2, k, ib, A1o, A2o, V0, T0, np.zeros(ib * max(m1, n1)))
    assert rel(host(tq, A1), A1o) < RTOL
    assert rel(host(tq, A2), A2o) < RTOL


def test_tsmqr_k0_noop(tq):
    """test/tsmqr.jl:75-85."""
    rng = np.random.default_rng(0)
    A10, A20 = rng.random((8, 8)), rng.random((8, 8))
    A1, A2 = dev(tq, A10), dev(tq, A20)
    tq.tsmqr("L", "N", 8, 8, 8, 8, 0, 0, A1, A2, tq.zeros(8, 1), tq.zeros(1, 1), None)
    assert np.array_equal(host(tq, A1), A10) and np.array_equal(host(tq, A2), A20)


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_parfb(tq, oracle, side, trans):
    rng = np.random.default_rng(3 + ord(side) * 2 + ord(trans))
    if side == "L":
        m1, n1, m2, n2, k = 12, 10, 9, 10, 5
    else:
        m1, n1, m2, n2, k = 9, 12, 9, 10, 5
    A10, A20 = F(rng.standard_normal((m1, n1))), F(rng.standard_normal((m2, n2)))
    V0 = F(rng.standard_normal((m2 if side == "L" else n2, k)))
    T0 = F(np.triu(rng.standard_normal((k, k))))
    A1, A2 = dev(tq, A10), dev(tq, A20)
    tq.parfb(side, trans, "F", "C", m1, n1, m2, n2, k, 0, A1, A2, dev(tq, V0), dev(tq, T0), None)
    A1o, A2o = A10.copy(order="F"), A20.copy(order="F")
    oracle.parfb(side, trans, m1, n1, m2, n2, k, A1o, A2o, V0, T0,
                 np.zeros((max(m1, m2), max(n1, n2)), order="F"))
    assert rel(host(tq, A1), A1o) < RTOL
    assert rel(host(tq, A2), A2o) < RTOL


# ---- single precision -------------------------------------------------------
def test_float_variants(tq, oracle):
    import torch
    rng = np.random.default_rng(9)
    m, n, ib = 256, 256, 32
    A0 = F(rng.uniform(-1, 1, (m, n)))
    A, T, tau = dev(tq, A0, torch.float32), tq.zeros(ib, n, dtype=torch.float32), \
        torch.zeros(n, dtype=torch.float32, device="cuda")
    tq.geqrt(m, n, ib, A, T, tau, None)
    Ao, To = A0.copy(order="F"), np.zeros((ib, n), order="F")
    oracle.geqrt(m, n, ib, Ao, To, np.zeros(n), np.zeros(ib * n))
    assert rel(host(tq, A), Ao) < RTOL32 * 100
    # backward error of the float factorisation, as test/geqrt.jl:27-31 measures it
    Af = host(tq, A)
    C = dev(tq, np.eye(m), torch.float32)
    tq.unmqr("L", "N", m, m, n, ib, A, m, T, C, None)
    Q = host(tq, C)
    eps = np.finfo(np.float32).eps
    assert np.linalg.norm(A0 - Q @ np.triu(Af), 1) / (np.linalg.norm(A0, 1) * n * eps) < 10
    assert np.linalg.norm(Q.T @ Q - np.eye(m), 1) / (m * eps) < 10
