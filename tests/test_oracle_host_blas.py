"""The oracle with its products in the host BLAS, pinned like the plain one.

NextLA's larfb! forms its products with LinearAlgebra.mul! (src/larfb.jl:66-98),
the host BLAS on CPU arrays; the oracle can do the same (oracle.host_blas()),
which is what makes it fast enough to check the CUDA library at the benchmark
sizes and to serve as the timed CPU baseline.  Only the order of the sums
inside each product changes, so this path must meet the same LAPACK golden
vectors at the reference's rtol 1e-12 (test/lapack_helpers.jl:14) and agree
with the plain-loop oracle to rounding, on the tile kernels and on the flat
tile driver (whose host-BLAS form applies each panel to the whole trailing
row block in one call).
"""
import numpy as np
import pytest

RTOL = 1e-12


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def F(a):
    return np.array(a, dtype=np.float64, order="F")


@pytest.fixture
def blas(oracle):
    pytest.importorskip("scipy")
    with oracle.host_blas():
        assert oracle.lib().ora_host_blas_on() == 1
        yield oracle
    assert oracle.lib().ora_host_blas_on() == 0


@pytest.mark.parametrize("m,n,ib", [(20, 15, 4), (32, 32, 8), (64, 32, 16), (32, 64, 8), (256, 256, 32)])
def test_geqrt_vs_lapack(blas, golden, m, n, ib):
    key = f"geqrt_{m}_{n}_{ib}"
    A = F(golden[key + "_A"])
    k = min(m, n)
    T = np.zeros((ib, k), order="F")
    tau = np.zeros(k)
    blas.geqrt(m, n, ib, A, T, tau, np.zeros(ib * n))
    assert rel(A, golden[key + "_outA"]) < RTOL
    assert rel(T, golden[key + "_outT"]) < RTOL * 10


@pytest.mark.parametrize("m,n,ib", [(32, 24, 8), (48, 32, 16), (64, 48, 16), (20, 20, 10), (256, 256, 32)])
def test_tsqrt_vs_lapack(blas, golden, m, n, ib):
    key = f"tsqrt_{m}_{n}_{ib}"
    A1, A2 = F(golden[key + "_A1"]), F(golden[key + "_A2"])
    T = np.zeros((ib, n), order="F")
    tau = np.zeros(n)
    blas.tsqrt(m, n, ib, A1, A2, T, tau, np.zeros(ib * n))
    assert rel(A1, golden[key + "_outA1"]) < RTOL
    assert rel(A2, golden[key + "_outA2"]) < RTOL
    assert rel(T, golden[key + "_outT"]) < RTOL


@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_tsmqr_vs_lapack(blas, golden, st):
    key = f"tsmqr_{st}"
    m1, n1, m2, n2, k, ib = (int(x) for x in golden[key + "_dims"])
    A1, A2 = F(golden[key + "_A1"]), F(golden[key + "_A2"])
    V, T = F(golden[key + "_V"]), F(golden[key + "_T"])
    blas.tsmqr(st[0], st[1], m1, n1, m2, n2, k, ib, A1, A2, V, T, np.zeros(ib * max(m1, n1)))
    assert rel(A1, golden[key + "_outA1"]) < RTOL
    assert rel(A2, golden[key + "_outA2"]) < RTOL


@pytest.mark.parametrize("st", ["LN", "LC", "RN", "RC"])
def test_unmqr_vs_lapack(blas, golden, st):
    Aq, Tq = F(golden["unmqr_Aqr"]), F(golden["unmqr_T"])
    C = F(golden[f"unmqr_{st}_C"])
    m, k = Aq.shape
    ib = Tq.shape[0]
    mm, nn = C.shape
    work = np.zeros((nn if st[0] == "L" else mm, ib), order="F")
    blas.unmqr(st[0], st[1], mm, nn, k, ib, Aq, m, Tq, C, work)
    assert rel(C, golden[f"unmqr_{st}_out"]) < RTOL


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_larfb_matches_plain_loops(oracle, side, trans):
    """larfb! (all side x trans) with BLAS products against the plain loops."""
    pytest.importorskip("scipy")
    rng = np.random.default_rng(7)
    m, n, k = 70, 45, 12
    V = F(np.tril(rng.standard_normal((m if side == "L" else n, k)), -1))
    T = F(np.triu(rng.standard_normal((k, k))))
    C0 = F(rng.standard_normal((m, n)))
    outs = []
    for on in (False, True):
        old = oracle.set_host_blas(on)
        try:
            C = C0.copy(order="F")
            W = np.zeros((n if side == "L" else m, k), order="F")
            oracle.larfb(side, trans, "F", "C", m, n, k, V, V.shape[0], T, C, W)
            outs.append(C)
        finally:
            oracle.set_host_blas(old)
    assert rel(outs[1], outs[0]) < 1e-14


@pytest.mark.parametrize("m,n", [(1024, 1024), (1000, 700), (2048, 512), (512, 1024), (300, 300)])
def test_tile_driver_matches_plain_loops(oracle, m, n):
    """The flat tile QR with wide host-BLAS calls against the per-tile plain
    loops: R, V, T and tau to rounding, then Q^T applied both ways."""
    pytest.importorskip("scipy")
    rng = np.random.default_rng(m * 7 + n)
    A0 = F(rng.standard_normal((m, n)))
    B0 = F(rng.standard_normal((m, 5)))
    res = []
    for on in (False, True):
        old = oracle.set_host_blas(on)
        try:
            A = A0.copy(order="F")
            T, tau = oracle.tile_geqrf(A, 256, 32)
            B = B0.copy(order="F")
            oracle.tile_unmqr("C", A, T, B, 256, 32)
            res.append((A, T, tau, B))
        finally:
            oracle.set_host_blas(old)
    for x, y in zip(res[1], res[0]):
        assert rel(x, y) < 1e-13 * max(m, n) ** 0.5


def test_host_blas_switch_validates(oracle):
    pytest.importorskip("scipy")
    assert oracle.lib().ora_set_host_blas(None, None) == 0
    assert oracle.lib().ora_set_host_blas(1, None) == -1
    assert oracle.lib().ora_host_blas_on() == 0
