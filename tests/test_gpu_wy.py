"""The compact-WY tensor-core update (tqr_swy_build / tqr_swy_apply) against
the FP64 oracle's tsmqr!, unmqr! and ttmqr! and the blocked tensor-core
kernel, on the same FP32 inputs.

The WY form applies Q = I - V T V^T with the k x k T of all ib-blocks in three
large products instead of the reference's chain of ib-blocks
(src/tsmqr.jl:47-146, src/unmqr.jl:99-148, src/ttmqr.jl:1-95); only the
grouping of the sums changes.  Bar: the reference's single-precision
tolerance, relative max-abs difference <= 1e-5 to the FP64 oracle, and the
device error flag stays clear.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

IB = 32


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def f32(a):
    return np.asfortranarray(np.asarray(a).astype(np.float32).astype(np.float64))


def P(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def run_wy(tq, m1, n, m2, k, A1, A2, V, T, vmode):
    """Build the slot from (V, T) and apply it to [A1; A2] (A1 None: unmqr)."""
    import torch
    from tileqr import _lib
    L = _lib.lib()
    nbytes = L.tqr_swy_slot_bytes()
    slot = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    dv, dt = tq.to_device(V, torch.float32), tq.to_device(T, torch.float32)
    d1 = tq.to_device(A1, torch.float32) if A1 is not None else None
    d2 = tq.to_device(A2, torch.float32)
    rc = L.tqr_swy_build(m2, k, P(dv), V.shape[0], P(dt), T.shape[0], vmode, P(slot), nbytes, P(err),
                         ctypes.c_void_p(st.cuda_stream))
    assert rc == 0
    rc = L.tqr_swy_apply(m1, n, m2, k, P(d1), m1 if A1 is not None else 1, P(d2), m2, P(slot), P(err),
                         ctypes.c_void_p(st.cuda_stream))
    assert rc == 0
    st.synchronize()
    assert err.item() == 0
    o1 = tq.to_numpy(d1).astype(np.float64) if d1 is not None else None
    return o1, tq.to_numpy(d2).astype(np.float64)


@pytest.mark.parametrize("m2,k,n", [(256, 256, 256), (256, 32, 128), (128, 64, 384), (256, 96, 512),
                                    (256, 256, 1024), (128, 128, 256), (256, 160, 128), (256, 192, 256)])
def test_wy_tsmqr(tq, oracle, m2, k, n):
    rng = np.random.default_rng(3 * m2 + k + n)
    m1 = k
    A1 = f32(rng.standard_normal((m1, n)))
    A2 = f32(rng.standard_normal((m2, n)))
    R = np.asfortranarray(np.triu(rng.standard_normal((k, k))) + 4 * np.eye(k))
    V = np.asfortranarray(rng.standard_normal((m2, k)))
    T = np.zeros((IB, k), order="F")
    oracle.tsqrt(m2, k, IB, R, V, T, np.zeros(k), np.zeros(IB * k))
    V, T = f32(V), f32(T)
    o1, o2 = A1.copy(order="F"), A2.copy(order="F")
    oracle.tsmqr("L", "C", m1, n, m2, n, k, IB, o1, o2, V, T, np.zeros(IB * n))
    w1, w2 = run_wy(tq, m1, n, m2, k, A1, A2, V, T, 0)
    assert rel(w1, o1) < 1e-5
    assert rel(w2, o2) < 1e-5


@pytest.mark.parametrize("m2,n", [(256, 256), (256, 768), (128, 128)])
def test_wy_unmqr(tq, oracle, m2, n):
    """Q^T C with geqrt!'s factor of a tile (V unit lower triangular, no A1)."""
    rng = np.random.default_rng(m2 + 7 * n)
    k = m2
    A = np.asfortranarray(rng.standard_normal((m2, k)))
    T = np.zeros((IB, k), order="F")
    oracle.geqrt(m2, k, IB, A, T, np.zeros(k), np.zeros(IB * k))
    A, T = f32(A), f32(T)
    C = f32(rng.standard_normal((m2, n)))
    oc = C.copy(order="F")
    oracle.unmqr("L", "C", m2, n, k, IB, A, m2, T, oc, np.zeros((n, IB), order="F"))
    _, w2 = run_wy(tq, 0, n, m2, k, None, C, A, T, 1)
    assert rel(w2, oc) < 1e-5


@pytest.mark.parametrize("k,n", [(256, 256), (128, 384)])
def test_wy_ttmqr(tq, oracle, k, n):
    """ttmqr! with ttqrt!'s factor of two triangles (V upper triangular; the
    rows below it hold other data, which the mask must hide)."""
    rng = np.random.default_rng(k + 11 * n)
    R1 = np.asfortranarray(np.triu(rng.standard_normal((k, k))) + 4 * np.eye(k))
    R2 = np.asfortranarray(np.triu(rng.standard_normal((k, k))))
    T = np.zeros((IB, k), order="F")
    oracle.ttqrt(k, k, IB, R1, R2, T, np.zeros(k), np.zeros(IB * k))
    V = np.asfortranarray(np.triu(R2) + np.tril(rng.standard_normal((k, k)), -1))   # junk below the triangle
    V, T = f32(V), f32(T)
    A1 = f32(rng.standard_normal((k, n)))
    A2 = f32(rng.standard_normal((k, n)))
    o1, o2 = A1.copy(order="F"), A2.copy(order="F")
    oracle.ttmqr("L", "C", k, n, k, n, k, IB, o1, o2, np.asfortranarray(np.triu(V)), T, np.zeros(IB * n))
    w1, w2 = run_wy(tq, k, n, k, k, A1, A2, V, T, 2)
    assert rel(w1, o1) < 1e-5
    assert rel(w2, o2) < 1e-5


def test_wy_matches_the_blocked_tensor_core_kernel(tq, oracle):
    """Same tsmqr! inputs through the blocked (ib-chain) and the WY form: both
    meet the oracle, and they agree with each other to FP32 accuracy."""
    import torch
    from tileqr import _lib
    rng = np.random.default_rng(5)
    m1, m2, k, n = 256, 256, 256, 512
    A1 = f32(rng.standard_normal((m1, n)))
    A2 = f32(rng.standard_normal((m2, n)))
    R = np.asfortranarray(np.triu(rng.standard_normal((k, k))) + 4 * np.eye(k))
    V = np.asfortranarray(rng.standard_normal((m2, k)))
    T = np.zeros((IB, k), order="F")
    oracle.tsqrt(m2, k, IB, R, V, T, np.zeros(k), np.zeros(IB * k))
    V, T = f32(V), f32(T)
    w1, w2 = run_wy(tq, m1, n, m2, k, A1, A2, V, T, 0)
    d1, d2 = tq.to_device(A1, torch.float32), tq.to_device(A2, torch.float32)
    dv, dt = tq.to_device(V, torch.float32), tq.to_device(T, torch.float32)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    assert _lib.lib().tqr_stsmqr_tc(m1, n, m2, k, P(d1), m1, P(d2), m2, P(dv), m2, P(dt), IB, P(err),
                                    ctypes.c_void_p(st.cuda_stream)) == 0
    st.synchronize()
    assert err.item() == 0
    b1, b2 = tq.to_numpy(d1).astype(np.float64), tq.to_numpy(d2).astype(np.float64)
    assert rel(w1, b1) < 1e-5 and rel(w2, b2) < 1e-5


def test_wy_argument_errors(tq):
    from tileqr import _lib
    L = _lib.lib()
    assert L.tqr_swy_slot_bytes() == 6 * 256 * 256 * 4
    assert L.tqr_swy_build(200, 32, None, 256, None, 32, 0, None, 0, None, None) == -1
    assert L.tqr_swy_build(256, 48, None, 256, None, 32, 0, None, 0, None, None) == -2
    assert L.tqr_swy_build(256, 32, 16, 256, 16, 32, 3, None, 0, None, None) == -7
    assert L.tqr_swy_build(256, 32, 16, 256, 16, 32, 0, 256, 10, None, None) == -9
    assert L.tqr_swy_apply(32, 100, 256, 32, None, 32, None, 256, None, None, None) == -2
    assert L.tqr_swy_apply(32, 128, 200, 32, None, 32, None, 256, None, None, None) == -3
    assert L.tqr_swy_apply(32, 128, 256, 64, 16, 32, None, 256, None, None, None) == -4
