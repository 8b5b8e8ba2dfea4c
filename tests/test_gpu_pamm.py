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
