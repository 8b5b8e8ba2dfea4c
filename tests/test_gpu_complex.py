"""ComplexF64 / ComplexF32 tile kernels on the GPU against the ComplexF64
oracle and the zgeqrt / ztpqrt / ztpmqrt / zgemqrt golden vectors.

Every reference kernel test runs ComplexF32 and ComplexF64
(test/lapack_helpers.jl:11).  Bars: ComplexF64 relative max-abs difference
<= 1e-12 against the oracle (the reference's double-precision rtol,
test/lapack_helpers.jl:14); ComplexF32 <= 1e-5 times a small size factor
against the oracle run on the same complex64-rounded inputs (the reference's
single-precision rtol).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RTOL32 = 1e-5
DTYPES = ["complex128", "complex64"]


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def Z(a):
    return np.array(a, dtype=np.complex128, order="F")


def tdt(name):
    import torch
    return getattr(torch, name)


def rnd(a, dt):
    """The inputs the device sees, widened back to complex128 for the oracle."""
    return Z(np.asarray(a).astype(np.complex64)) if dt == "complex64" else Z(a)


def tol(dt, scale=1):
    return RTOL * scale if dt == "complex128" else RTOL32 * scale


def crand(rng, shape):
    return Z(rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def dev(tq, a, dt):
    return tq.to_device(a, dtype=tdt(dt))


def host(tq, t):
    return tq.to_numpy(t).astype(np.complex128)


def zeros(tq, m, n, dt):
    return tq.zeros(m, n, dtype=tdt(dt))


def zvec(n, dt):
    import torch
    return torch.zeros(n, dtype=tdt(dt), device="cuda")


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("m,n,ib", [(20, 15, 4), (32, 32, 8), (64, 32, 16), (32, 64, 8), (128, 128, 32),
                                    (300, 64, 32)])
def test_zgeqrt_vs_oracle(tq, oracle, dt, m, n, ib):
    rng = np.random.default_rng(m * 7 + n + ib)
    A0 = rnd(crand(rng, (m, n)), dt)
    k = min(m, n)
    A, T, tau = dev(tq, A0, dt), zeros(tq, ib, k, dt), zvec(k, dt)
    tq.geqrt(m, n, ib, A, T, tau, None)
    Ao, To, tauo = A0.copy(order="F"), np.zeros((ib, k), complex, order="F"), np.zeros(k, complex)
    oracle.geqrt(m, n, ib, Ao, To, tauo, np.zeros(ib * n, complex))
    s = 1 if dt == "complex128" else 10
    assert rel(host(tq, A), Ao) < tol(dt, s)
    assert rel(host(tq, T), To) < tol(dt, s * 10)
    assert rel(host(tq, tau), tauo) < tol(dt, s)
    # beta is real on the diagonal of R (but for the reference's one-row last column)
    d = np.diag(host(tq, A))[: (k if m > n else k - 1)]
    assert np.max(np.abs(d.imag)) == 0.0


@pytest.mark.parametrize("m,n,ib", [(20, 15, 4), (64, 32, 16), (128, 128, 32)])
def test_zgeqrt_golden(tq, golden, m, n, ib):
    """Straight against zgeqrt (for m > n every entry; for m <= n all but the
    reference's one-row last reflector, which the oracle tests pin)."""
    key = f"z_geqrt_{m}_{n}_{ib}"
    A0 = Z(golden[key + "_A"])
    k = min(m, n)
    A, T, tau = dev(tq, A0, "complex128"), zeros(tq, ib, k, "complex128"), zvec(k, "complex128")
    tq.geqrt(m, n, ib, A, T, tau, None)
    outA, outT = golden[key + "_outA"], golden[key + "_outT"]
    L = k if m > n else m - 1
    assert rel(host(tq, A)[:L], outA[:L]) < RTOL
    assert rel(host(tq, T)[:, :L], outT[:, :L]) < 10 * RTOL


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("m,n", [(16, 12), (256, 32), (300, 40), (1500, 8)])
def test_zgeqr2(tq, oracle, dt, m, n):
    rng = np.random.default_rng(m + n)
    A0 = rnd(crand(rng, (m, n)), dt)
    A, tau = dev(tq, A0, dt), zvec(min(m, n), dt)
    tq.geqr2(m, n, A, tau, None)
    Ao, tauo = A0.copy(order="F"), np.zeros(min(m, n), complex)
    oracle.geqr2(m, n, Ao, tauo, np.zeros(n, complex))
    s = 1 if dt == "complex128" else 10
    assert rel(host(tq, A), Ao) < tol(dt, s)
    assert rel(host(tq, tau), tauo) < tol(dt, s)


def test_zgeqr2_real_alpha_zero_x_keeps_reflector(tq, oracle):
    """A column with x = 0 but a complex alpha still gets a reflector
    (tau != 0, src/geqr2.jl:48); x = 0 with a real alpha gets tau = 0."""
    A0 = Z(np.zeros((6, 2)))
    A0[0, 0] = 1.0 + 2.0j
    A0[1, 1] = 3.0
    A0[3, 1] = 1.0j
    A, tau = dev(tq, A0, "complex128"), zvec(2, "complex128")
    tq.geqr2(6, 2, A, tau, None)
    Ao, tauo = A0.copy(order="F"), np.zeros(2, complex)
    oracle.geqr2(6, 2, Ao, tauo, np.zeros(2, complex))
    assert abs(tauo[0]) > 0
    assert rel(host(tq, A), Ao) < RTOL and rel(host(tq, tau), tauo) < RTOL
    B0 = Z(np.zeros((4, 1)))
    B0[0, 0] = 2.0
    B, tb = dev(tq, B0, "complex128"), zvec(1, "complex128")
    tq.geqr2(4, 1, B, tb, None)
    assert host(tq, tb)[0] == 0 and np.array_equal(host(tq, B), B0)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("direct", ["F", "B"])
@pytest.mark.parametrize("storev", ["C", "R"])
@pytest.mark.parametrize("n,k", [(1, 1), (5, 3), (20, 8), (256, 32)])
def test_zlarft(tq, oracle, dt, direct, storev, n, k):
    rng = np.random.default_rng(n * 7 + k)
    # entries ~ 1/sqrt(n) keep the V^H v products O(1): with unit-variance
    # entries the T recursion grows like n^(k/2) and leaves float range
    V0 = rnd(crand(rng, (n, k) if storev == "C" else (k, n)) / np.sqrt(n), dt)
    if n > 3:
        if storev == "C":
            V0[-2:, -1] = 0.0
        else:
            V0[-1, -2:] = 0.0
    tau0 = rnd(rng.standard_normal(k) + 1j * rng.standard_normal(k), dt).ravel()
    V, tau, T = dev(tq, V0, dt), dev(tq, tau0, dt), zeros(tq, k, k, dt)
    tq.larft(direct, storev, n, k, V, tau, T)
    To = np.zeros((k, k), complex, order="F")
    oracle.larft(direct, storev, n, k, V0, tau0, To)
    assert rel(host(tq, T), To) < tol(dt, 10)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
@pytest.mark.parametrize("m,n,k", [(5, 4, 4), (20, 15, 4), (256, 224, 32), (300, 100, 70)])
def test_zlarfb(tq, oracle, dt, side, trans, m, n, k):
    rng = np.random.default_rng(m * 3 + n + k)
    rows = m if side == "L" else n
    k = min(k, rows)
    panel = crand(rng, (rows, k))
    tau = np.zeros(k, complex)
    oracle.geqr2(rows, k, panel, tau, np.zeros(k, complex))
    T0 = np.zeros((k, k), complex, order="F")
    oracle.larft("F", "C", rows, k, panel, tau, T0)
    panel, T0 = rnd(panel, dt), rnd(T0, dt)
    C0 = rnd(crand(rng, (m, n)), dt)
    C = dev(tq, C0, dt)
    tq.larfb(side, trans, "F", "C", m, n, k, dev(tq, panel, dt), rows, dev(tq, T0, dt), C, None)
    Co = C0.copy(order="F")
    oracle.larfb(side, trans, "F", "C", m, n, k, panel, rows, T0, Co,
                 np.zeros((n if side == "L" else m, k), complex, order="F"))
    assert rel(host(tq, C), Co) < tol(dt, 10)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_zunmqr(tq, oracle, golden, dt, st):
    Aq, Tq = rnd(golden["z_unmqr_Aqr"], dt), rnd(golden["z_unmqr_T"], dt)
    C0 = rnd(golden[f"z_unmqr_{st}_C"], dt)
    m, k = Aq.shape
    ib = Tq.shape[0]
    mm, nn = C0.shape
    C = dev(tq, C0, dt)
    tq.unmqr(st[0], st[1], mm, nn, k, ib, dev(tq, Aq, dt), m, dev(tq, Tq, dt), C, None)
    Co = C0.copy(order="F")
    oracle.unmqr(st[0], st[1], mm, nn, k, ib, Aq, m, Tq, Co,
                 np.zeros((nn if st[0] == "L" else mm, ib), complex, order="F"))
    assert rel(host(tq, C), Co) < tol(dt, 10)
    if dt == "complex128":
        assert rel(host(tq, C), golden[f"z_unmqr_{st}_out"]) < RTOL


def test_zunmqr_unitary(tq):
    """test/unmqr.jl:69-78: Q Q^H = I, for both complex types."""
    import torch
    for dt, bar in (("complex128", 1e-13), ("complex64", 1e-5)):
        rng = np.random.default_rng(7)
        m, k, ib = 64, 32, 8
        A = dev(tq, crand(rng, (m, k)), dt)
        T = zeros(tq, ib, k, dt)
        tq.geqrt(m, k, ib, A, T, zvec(k, dt), None)
        C = dev(tq, np.eye(m), dt)
        tq.unmqr("L", "N", m, m, k, ib, A, m, T, C, None)
        tq.unmqr("L", "C", m, m, k, ib, A, m, T, C, None)
        assert np.max(np.abs(host(tq, C) - np.eye(m))) < bar
        assert C.dtype == tdt(dt) and torch.is_complex(C)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("m,n,ib", [(32, 24, 8), (48, 32, 16), (20, 20, 10), (128, 128, 32), (256, 256, 32)])
def test_ztsqrt(tq, oracle, golden, dt, m, n, ib):
    rng = np.random.default_rng(m + 3 * n)
    key = f"z_tsqrt_{m}_{n}_{ib}"
    if key + "_A1" in golden.files:
        A10, A20 = rnd(golden[key + "_A1"], dt), rnd(golden[key + "_A2"], dt)
    else:
        A10 = rnd(np.triu(crand(rng, (n, n))) + 2 * np.eye(n), dt)
        A20 = rnd(crand(rng, (m, n)), dt)
    A1, A2, T, tau = dev(tq, A10, dt), dev(tq, A20, dt), zeros(tq, ib, n, dt), zvec(n, dt)
    tq.tsqrt(m, n, ib, A1, A2, T, tau, None)
    A1o, A2o, To = A10.copy(order="F"), A20.copy(order="F"), np.zeros((ib, n), complex, order="F")
    oracle.tsqrt(m, n, ib, A1o, A2o, To, np.zeros(n, complex), np.zeros(ib * n, complex))
    s = 1 if dt == "complex128" else 10
    assert rel(np.triu(host(tq, A1)), np.triu(A1o)) < tol(dt, s)
    assert rel(host(tq, A2), A2o) < tol(dt, s)
    assert rel(host(tq, T), To) < tol(dt, 10 * s)
    if dt == "complex128" and key + "_outA2" in golden.files:
        assert rel(host(tq, A2), golden[key + "_outA2"]) < RTOL
        assert rel(host(tq, T), golden[key + "_outT"]) < RTOL


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("kind", ["tsmqr", "ttmqr"])
@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_ztsmqr_ttmqr(tq, oracle, golden, dt, kind, st):
    key = f"z_{kind}_{st}"
    m1, n1, m2, n2, k, ib = (int(x) for x in golden[key + "_dims"])
    A10, A20 = rnd(golden[key + "_A1"], dt), rnd(golden[key + "_A2"], dt)
    V0, T0 = rnd(golden[key + "_V"], dt), rnd(golden[key + "_T"], dt)
    A1, A2 = dev(tq, A10, dt), dev(tq, A20, dt)
    getattr(tq, kind)(st[0], st[1], m1, n1, m2, n2, k, ib, A1, A2, dev(tq, V0, dt), dev(tq, T0, dt), None)
    A1o, A2o = A10.copy(order="F"), A20.copy(order="F")
    getattr(oracle, kind)(st[0], st[1], m1, n1, m2, n2, k, ib, A1o, A2o, V0, T0,
                          np.zeros(ib * max(m1, n1), complex))
    assert rel(host(tq, A1), A1o) < tol(dt, 10)
    assert rel(host(tq, A2), A2o) < tol(dt, 10)
    if dt == "complex128":
        assert rel(host(tq, A1), golden[key + "_outA1"]) < RTOL
        assert rel(host(tq, A2), golden[key + "_outA2"]) < RTOL


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_ztsmqr_wide_band(tq, oracle, dt, side, trans):
    """One call over a 256-row tile pair and a wide band (the tile driver's form)."""
    rng = np.random.default_rng(11 + ord(side) + 3 * ord(trans))
    k, ib = 64, 32
    if side == "L":
        m1, n1, m2, n2 = 64, 300, 256, 300
    else:
        m1, n1, m2, n2 = 300, 64, 300, 256
    R = Z(np.triu(crand(rng, (k, k))) + 4 * np.eye(k))
    V = crand(rng, (m2 if side == "L" else n2, k))
    T = np.zeros((ib, k), complex, order="F")
    oracle.tsqrt(V.shape[0], k, ib, R, V, T, np.zeros(k, complex), np.zeros(ib * k, complex))
    V, T = rnd(V, dt), rnd(T, dt)
    A10, A20 = rnd(crand(rng, (m1, n1)), dt), rnd(crand(rng, (m2, n2)), dt)
    A1, A2 = dev(tq, A10, dt), dev(tq, A20, dt)
    tq.tsmqr(side, trans, m1, n1, m2, n2, k, ib, A1, A2, dev(tq, V, dt), dev(tq, T, dt), None)
    A1o, A2o = A10.copy(order="F"), A20.copy(order="F")
    oracle.tsmqr(side, trans, m1, n1, m2, n2, k, ib, A1o, A2o, V, T, np.zeros(ib * 300, complex))
    assert rel(host(tq, A1), A1o) < tol(dt, 10)
    assert rel(host(tq, A2), A2o) < tol(dt, 10)


def test_ztrans_t_is_c(tq):
    """'T' acts as 'C' for complex elements (src/tsmqr.jl:20)."""
    rng = np.random.default_rng(2)
    V = crand(rng, (20, 8))
    T = Z(np.triu(crand(rng, (4, 8))))
    A10, A20 = crand(rng, (8, 12)), crand(rng, (20, 12))
    out = []
    for tr in "TC":
        A1, A2 = dev(tq, A10, "complex128"), dev(tq, A20, "complex128")
        tq.tsmqr("L", tr, 8, 12, 20, 12, 8, 4, A1, A2, dev(tq, V, "complex128"), dev(tq, T, "complex128"), None)
        out.append((host(tq, A1), host(tq, A2)))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n,ib", [(16, 4), (24, 8), (48, 16)])
def test_zttqrt(tq, oracle, golden, dt, n, ib):
    key = f"z_ttqrt_{n}_{ib}"
    A10, A20 = rnd(golden[key + "_A1"], dt), rnd(golden[key + "_A2"], dt)
    A1, A2, T, tau = dev(tq, A10, dt), dev(tq, A20, dt), zeros(tq, ib, n, dt), zvec(n, dt)
    tq.ttqrt(n, n, ib, A1, A2, T, tau, None)
    A1o, A2o, To = A10.copy(order="F"), A20.copy(order="F"), np.zeros((ib, n), complex, order="F")
    oracle.ttqrt(n, n, ib, A1o, A2o, To, np.zeros(n, complex), np.zeros(ib * n, complex))
    s = 1 if dt == "complex128" else 10
    assert rel(np.triu(host(tq, A1)), np.triu(A1o)) < tol(dt, s)
    assert rel(np.triu(host(tq, A2)), np.triu(A2o)) < tol(dt, s)
    assert rel(host(tq, T), To) < tol(dt, 10 * s)
    if dt == "complex128":
        assert rel(np.triu(host(tq, A2)), np.triu(golden[key + "_outA2"])) < RTOL
        for trans in "NC":
            C1, C2 = dev(tq, golden[f"{key}_L{trans}_C1"], dt), dev(tq, golden[f"{key}_L{trans}_C2"], dt)
            tq.ttmqr("L", trans, n, 40, n, 40, n, ib, C1, C2, A2, T, None)
            assert rel(host(tq, C1), golden[f"{key}_L{trans}_out1"]) < RTOL
            assert rel(host(tq, C2), golden[f"{key}_L{trans}_out2"]) < RTOL


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("l", [0, 3, 5])
def test_zparfb(tq, oracle, dt, side, l):
    rng = np.random.default_rng(5 + l + ord(side))
    k = 5
    if side == "L":
        m1, n1, m2, n2 = 12, 10, 9, 10
    else:
        m1, n1, m2, n2 = 9, 12, 9, 10
    for trans in "NC":
        A10, A20 = rnd(crand(rng, (m1, n1)), dt), rnd(crand(rng, (m2, n2)), dt)
        V0 = rnd(crand(rng, (m2 if side == "L" else n2, k)), dt)
        T0 = rnd(np.triu(crand(rng, (k, k))), dt)
        A1, A2 = dev(tq, A10, dt), dev(tq, A20, dt)
        tq.parfb(side, trans, "F", "C", m1, n1, m2, n2, k, l, A1, A2, dev(tq, V0, dt), dev(tq, T0, dt), None)
        A1o, A2o = A10.copy(order="F"), A20.copy(order="F")
        oracle.parfb_l(side, trans, m1, n1, m2, n2, k, l, A1o, A2o, V0, T0,
                       np.zeros((max(m1, m2), max(n1, n2)), complex, order="F"))
        assert rel(host(tq, A1), A1o) < tol(dt, 10)
        assert rel(host(tq, A2), A2o) < tol(dt, 10)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("m,n,nb,ib", [(1024, 512, 256, 32), (300, 200, 64, 16), (513, 257, 128, 32),
                                       (256, 640, 128, 32)])
def test_ztile_qr(tq, oracle, dt, m, n, nb, ib):
    """Flat-tree tile QR (geqrt, unmqr, tsqrt, tsmqr in PLASMA order) on
    complex tiles against the oracle's driver, then Q^H A = [R; 0] and the
    Q application both ways."""
    rng = np.random.default_rng(m + 2 * n)
    A0 = rnd(crand(rng, (m, n)), dt)
    A = dev(tq, A0, dt)
    T, tau = tq.tile_geqrf(A, nb, ib)
    assert T.dtype == tdt(dt)
    Ao = A0.copy(order="F")
    To, tauo = oracle.tile_geqrf(Ao, nb, ib)
    s = max(n, 16) * (1 if dt == "complex128" else 10)
    assert rel(host(tq, A), Ao) < tol(dt, s)
    assert rel(host(tq, T), To) < tol(dt, s)
    assert rel(host(tq, tau), tauo) < tol(dt, s)
    k = min(m, n)
    for trans in "NC":
        C0 = rnd(crand(rng, (m, 7)), dt)
        C = dev(tq, C0, dt)
        tq.tile_unmqr(trans, A, T, C, nb, ib)
        Co = C0.copy(order="F")
        oracle.tile_unmqr(trans, Ao, To, Co, nb, ib)
        assert rel(host(tq, C), Co) < tol(dt, s)
    QhA = dev(tq, A0, dt)
    tq.tile_unmqr("C", A, T, QhA, nb, ib)
    R = np.triu(host(tq, A)[:k])
    bar = 1e-13 if dt == "complex128" else 1e-5
    assert np.linalg.norm(host(tq, QhA)[:k] - R) <= bar * np.linalg.norm(R) * k


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("m,n,nb,ib", [(1024, 512, 256, 32), (512, 1024, 256, 32), (768, 768, 128, 16),
                                       (1024, 1024, 256, 32)])
def test_ztile_qr_task_graph_equals_stream_driver(tq, dt, m, n, nb, ib):
    """The persistent task-graph kernel runs the same per-task arithmetic as
    the stream driver on complex tiles too: bit-identical A, T, tau."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(m + n)
    re = torch.randn(m, n, generator=g, dtype=torch.float64, device="cuda")
    im = torch.randn(m, n, generator=g, dtype=torch.float64, device="cuda")
    A0 = torch.complex(re, im).to(tdt(dt))
    outs = []
    for dag in (False, True):
        A = tq.empty(m, n, dtype=tdt(dt))
        A.copy_(A0)
        T, tau = tq.tile_geqrf(A, nb, ib, dag=dag)
        outs.append((A, T, tau))
    for a, b in zip(*outs):
        assert torch.equal(a, b)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n,nrhs", [(40, 3), (300, 5), (600, 1)])
def test_ztrsm_lun(tq, oracle, dt, n, nrhs):
    """LeftUpperTRSM!'s arithmetic on complex R (diagonal scaling, then
    b[r] -= (R[r,i]/R[r,r]) b[i]), blocked beyond 256 rows."""
    rng = np.random.default_rng(n + nrhs)
    R0 = np.triu(crand(rng, (n, n))) / np.sqrt(n)
    R0[np.diag_indices(n)] = (2 + rng.random(n)) * np.exp(1j * rng.uniform(0, 2 * np.pi, n))
    R0, B0 = rnd(R0, dt), rnd(crand(rng, (n, nrhs)), dt)
    B = dev(tq, B0, dt)
    tq.trsm_lun(dev(tq, R0, dt), B)
    Xo = B0.copy(order="F")
    oracle.trsm_lun(R0, Xo)
    assert rel(host(tq, B), Xo) < tol(dt, 10 * n)


@pytest.mark.parametrize("dt", DTYPES)
def test_ztile_gels(tq, oracle, dt):
    """Complex least squares (tile QR, Q^H B, back-substitution) against the
    oracle's and against the planted solution."""
    rng = np.random.default_rng(12)
    m, n, k = 600, 300, 2
    A0 = rnd(crand(rng, (m, n)), dt)
    x = crand(rng, (n, k))
    B0 = rnd(A0 @ x, dt)
    A, B = dev(tq, A0, dt), dev(tq, B0, dt)
    X, T, tau = tq.tile_gels(A, B, 128, 32)
    Xo = oracle.tile_lstsq(A0, B0, 128, 32)
    assert rel(host(tq, X), Xo) < tol(dt, 1000)
    bar = 1e-9 if dt == "complex128" else 1e-3
    assert np.abs(host(tq, X) - x).max() < bar


def test_zcomplex_real_only_paths_refuse(tq):
    """The mixed-precision solve is real-only: it says so instead of running
    on reinterpreted complex data, as do the tree driver's mixed arguments
    (mismatched element types, the FP64-panel form)."""
    A = tq.to_device(crand(np.random.default_rng(0), (512, 256)), dtype=tdt("complex128"))
    T, tau = tq.tile_geqrf(A, 256, 32, dag=True)
    assert T.dtype == tdt("complex128")
    with pytest.raises(TypeError):
        tq.tile_unmqr_tree("C", A, T, T, tq.zeros(512, 1, dtype=tdt("complex64")), 256, 32)
    with pytest.raises(TypeError):
        tq.lstsq_mixed(A, tq.zeros(512, 1, dtype=tdt("complex128")))
    with pytest.raises(TypeError):
        tq.tile_geqrf_tree(A, 256, 32, grp=2, f64p=True)


ZHQR_SHAPES = [(1024, 256, 128, 32, 1), (1000, 300, 128, 16, 3), (1024, 256, 128, 32, 2), (517, 130, 64, 16, 3),
               (300, 400, 256, 32, 2), (768, 256, 128, 32, 100), (2048, 512, 256, 32, 4)]


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("m,n,nb,ib,grp", ZHQR_SHAPES)
def test_ztree_hqr_matches_oracle(tq, oracle, dt, m, n, nb, ib, grp):
    """The tree / hierarchical tile QR on complex elements (grp 1: every
    merge a ttqrt!, as ttqrt!'s ComplexF64 tests run it, test/ttqrt.jl:28-66)
    against the complex oracle's driver in the same order, B carried along
    as Q^H B; then Q^H and Q through the stored factors."""
    rng = np.random.default_rng(m + 3 * n + grp)
    A0, B0 = rnd(crand(rng, (m, n)), dt), rnd(crand(rng, (m, 3)), dt)
    A, B = dev(tq, A0, dt), dev(tq, B0, dt)
    T, tau, T2, tau2 = tq.tile_geqrf_tree(A, nb, ib, B=B, grp=grp)
    Ao = A0.copy(order="F")
    To, tauo, T2o, tau2o = oracle.tile_geqrf_hqr(Ao, nb, ib, grp)
    Bo = B0.copy(order="F")
    oracle.tile_unmqr_hqr("C", Ao, To, T2o, Bo, nb, ib, grp)
    bar = tol(dt, max(n, 16))
    for x, y in ((A, Ao), (T, To), (tau, tauo), (T2, T2o), (tau2, tau2o), (B, Bo)):
        assert rel(host(tq, x), y) < bar
    # the stored factors: Q^H A0 = R, and Q (Q^H C) = C
    k = min(m, n)
    QhA = dev(tq, A0, dt)
    tq.tile_unmqr_tree("C", A, T, T2, QhA, nb, ib, grp=grp)
    R = np.triu(host(tq, A)[:k])
    assert np.linalg.norm(host(tq, QhA)[:k] - R) <= bar * np.linalg.norm(R)
    C0 = rnd(crand(rng, (m, 2)), dt)
    C = dev(tq, C0, dt)
    tq.tile_unmqr_tree("C", A, T, T2, C, nb, ib, grp=grp)
    tq.tile_unmqr_tree("N", A, T, T2, C, nb, ib, grp=grp)
    assert rel(host(tq, C), C0) < bar


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("m,n,nb,ib,grp,nrhs", [(1024, 512, 128, 32, 2, 3), (1000, 300, 128, 16, 1, 0),
                                                (2048, 256, 256, 32, 4, 5)])
def test_ztree_task_graph_equals_stream_driver(tq, dt, m, n, nb, ib, grp, nrhs):
    """The persistent task graph on complex elements (8-column strips for
    ComplexF64) runs the stream driver's per-task arithmetic: bit-identical."""
    import torch
    rng = np.random.default_rng(m + n + nrhs)
    A0, B0 = rnd(crand(rng, (m, n)), dt), rnd(crand(rng, (m, max(nrhs, 1))), dt)
    outs = []
    for dag in (False, True):
        A = dev(tq, A0, dt)
        B = dev(tq, B0[:, :nrhs], dt) if nrhs else None
        res = tq.tile_geqrf_tree(A, nb, ib, B=B, dag=dag, grp=grp)
        outs.append((A,) + tuple(res) + ((B,) if nrhs else ()))
    for a, b in zip(*outs):
        assert torch.equal(a, b)
