"""pamm! on the GPU (every op / side / storev / direct form, FP64, FP32,
ComplexF64, ComplexF32) against the oracle's pamm, which the CPU suite checks
against its definition and, through the parfb! sequence, against LAPACK
(src/pamm.jl:49-473; the reference tests ComplexF32 / ComplexF64, test/pamm.jl)."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORMS = list(itertools.product("WA", "LR", "CR", "FB"))
DTYPES = {"float64": (np.float64, 1e-13), "float32": (np.float32, 1e-5), "complex128": (np.complex128, 1e-13),
          "complex64": (np.complex64, 1e-5)}


@pytest.mark.parametrize("dt", list(DTYPES))
@pytest.mark.parametrize("op,side,storev,direct", FORMS)
@pytest.mark.parametrize("l", [0, 10])
def test_pamm_vs_oracle(tq, oracle, dt, op, side, storev, direct, l):
    import torch
    npdt, bar = DTYPES[dt]
    cplx = np.iscomplexobj(np.zeros(1, npdt))
    rng = np.random.default_rng(hash((op, side, storev, direct, l)) % 2**32)
    m, n, k = 40, 30, 20                                   # test/pamm.jl:6
    mv = m if side == "L" else n

    def R(*s):
        a = rng.standard_normal(s) + (1j * rng.standard_normal(s) if cplx else 0)
        return np.asfortranarray(a.astype(npdt).astype(np.complex128 if cplx else np.float64))
    A1 = R(k, n) if side == "L" else R(m, k)
    A2 = R(m, n)
    V = R(mv, k) if storev == "C" else R(k, mv)
    W = R(k, n) if side == "L" else R(m, k)
    A2o, Wo = A2.copy(order="F"), W.copy(order="F")
    oracle.pamm(op, side, storev, direct, m, n, k, l, A1, A2o, V, Wo)
    td = getattr(torch, dt)
    dA1, dA2, dV, dW = (tq.to_device(x, dtype=td) for x in (A1, A2, V, W))
    tq.pamm(op, side, storev, direct, m, n, k, l, dA1, dA2, dV, dW)
    g2, gw = tq.to_numpy(dA2).astype(A2o.dtype), tq.to_numpy(dW).astype(Wo.dtype)
    assert np.abs(g2 - A2o).max() <= bar * 10 * np.abs(A2o).max()
    assert np.abs(gw - Wo).max() <= bar * 10 * np.abs(Wo).max()


def test_pamm_quick_return_and_errors(tq):
    import torch
    from tileqr import ArgumentError
    rng = np.random.default_rng(1)
    A1, A2 = tq.to_device(rng.random((5, 5))), tq.to_device(rng.random((10, 5)))
    V, W = tq.to_device(rng.random((10, 5))), tq.to_device(rng.random((5, 5)))
    W0 = W.clone()
    for (m, n, k) in [(0, 5, 5), (10, 0, 5), (10, 5, 0)]:
        tq.pamm("W", "L", "C", "F", m, n, k, 3, A1, A2, V, W)
        assert torch.equal(W, W0)
    for args in [("X", "L", "C", "F", 10, 5, 5, 3), ("W", "L", "C", "F", 10, 5, 5, 6)]:
        with pytest.raises(ArgumentError):
            tq.pamm(*args, A1, A2, V, W)


@pytest.mark.parametrize("dt", list(DTYPES))
@pytest.mark.parametrize("side", "LR")
@pytest.mark.parametrize("trans", "NC")
@pytest.mark.parametrize("direct", "FB")
@pytest.mark.parametrize("storev", "CR")
def test_parfb_every_form(tq, oracle, dt, side, trans, direct, storev):
    """parfb! in every side x trans x direct x storev form at the reference's
    test shapes (test/parfb.jl:6-39: m2, n2, k, l = 20, 24, 8, 4, T = rand(k, k))
    against the oracle, which the CPU suite checks against LAPACK's tprfb
    definition."""
    import torch
    npdt, bar = DTYPES[dt]
    cplx = np.iscomplexobj(np.zeros(1, npdt))
    rng = np.random.default_rng(hash((side, trans, direct, storev)) % 2**32)

    def R(*s):
        a = rng.random(s) + (1j * rng.random(s) if cplx else 0)
        return np.asfortranarray(a.astype(npdt).astype(np.complex128 if cplx else np.float64))
    m2, n2, k, l = 20, 24, 8, 4
    m1, n1 = (k, n2) if side == "L" else (m2, k)
    A1, A2 = R(m1, n1), R(m2, n2)
    mv = m2 if side == "L" else n2
    V = R(mv, k) if storev == "C" else R(k, mv)
    T = R(k, k)
    A1o, A2o = A1.copy(order="F"), A2.copy(order="F")
    Wo = np.zeros((k, n2) if side == "L" else (m2, k), A1.dtype, order="F")
    oracle.parfb_full(side, trans, direct, storev, m1, n1, m2, n2, k, l, A1o, A2o, V, T, Wo)
    td = getattr(torch, dt)
    d1, d2, dv, dT = (tq.to_device(x, dtype=td) for x in (A1, A2, V, T))
    tq.parfb(side, trans, direct, storev, m1, n1, m2, n2, k, l, d1, d2, dv, dT, None)
    g1, g2 = tq.to_numpy(d1).astype(A1o.dtype), tq.to_numpy(d2).astype(A2o.dtype)
    assert np.abs(g1 - A1o).max() <= bar * 100 * np.abs(A1o).max()
    assert np.abs(g2 - A2o).max() <= bar * 100 * np.abs(A2o).max()


def test_parfb_general_form_needs_work(tq):
    from tileqr import _lib
    L = _lib.lib()
    # direct 'B' without a work block: the position of work is reported
    assert L.tqr_dparfb(b"L", b"N", b"B", b"C", 8, 24, 20, 24, 8, 4, 16, 8, 16, 20, 16, 20, 16, 8,
                        None, 8, None) == -20
