"""Tensor-core (tcgen05, TF32 split three ways) FP32 tsmqr!('L','C') against
the SIMT FP32 kernel and the FP64 oracle on the same inputs.

Bar: the reference's single-precision tolerance, relative max-abs difference
<= 1e-5 to the FP64 oracle (both FP32 kernels land near 2e-6 on these
inputs), and the device error flag stays clear.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("m2,k,n", [(256, 256, 256), (256, 32, 128), (128, 64, 384), (256, 96, 512)])
def test_tsmqr_tensor_core(tq, oracle, m2, k, n):
    import torch
    from tileqr import _lib
    rng = np.random.default_rng(m2 + k + n)
    m1 = k
    A1 = np.asfortranarray(rng.standard_normal((m1, n)))
    A2 = np.asfortranarray(rng.standard_normal((m2, n)))
    # a genuine tsqrt! factor, so V and T are the well-scaled ones a QR produces
    R = np.asfortranarray(np.triu(rng.standard_normal((k, k))) + 4 * np.eye(k))
    V = np.asfortranarray(rng.standard_normal((m2, k)))
    T = np.zeros((32, k), order="F")
    oracle.tsqrt(m2, k, 32, R, V, T, np.zeros(k), np.zeros(32 * k))
    f32 = lambda a: np.asfortranarray(a.astype(np.float32).astype(np.float64))
    A1, A2, V, T = f32(A1), f32(A2), f32(V), f32(T)
    # FP64 oracle on the FP32-rounded inputs
    o1, o2 = A1.copy(order="F"), A2.copy(order="F")
    oracle.tsmqr("L", "C", m1, n, m2, n, k, 32, o1, o2, V, T, np.zeros(32 * n))
    # tensor-core kernel
    d1, d2 = tq.to_device(A1, torch.float32), tq.to_device(A2, torch.float32)
    dv, dt = tq.to_device(V, torch.float32), tq.to_device(T, torch.float32)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    rc = _lib.lib().tqr_stsmqr_tc(m1, n, m2, k, ctypes.c_void_p(d1.data_ptr()), m1, ctypes.c_void_p(d2.data_ptr()),
                                  m2, ctypes.c_void_p(dv.data_ptr()), m2, ctypes.c_void_p(dt.data_ptr()), 32,
                                  ctypes.c_void_p(err.data_ptr()), ctypes.c_void_p(st.cuda_stream))
    assert rc == 0
    st.synchronize()
    assert err.item() == 0
    assert rel(tq.to_numpy(d1).astype(np.float64), o1) < 1e-5
    assert rel(tq.to_numpy(d2).astype(np.float64), o2) < 1e-5
    # the SIMT FP32 kernel on the same inputs agrees to FP32 accuracy as well
    s1, s2 = tq.to_device(A1, torch.float32), tq.to_device(A2, torch.float32)
    tq.tsmqr("L", "C", m1, n, m2, n, k, 32, s1, s2, dv, dt, None)
    assert rel(tq.to_numpy(s1).astype(np.float64), o1) < 1e-5
    assert rel(tq.to_numpy(s2).astype(np.float64), o2) < 1e-5


def test_tsmqr_tensor_core_argument_errors(tq):
    from tileqr import _lib
    L = _lib.lib()
    assert L.tqr_stsmqr_tc(32, 100, 256, 32, None, 32, None, 256, None, 256, None, 32, None, None) == -2
    assert L.tqr_stsmqr_tc(32, 128, 200, 32, None, 32, None, 256, None, 256, None, 32, None, None) == -3
    assert L.tqr_stsmqr_tc(32, 128, 256, 48, None, 32, None, 256, None, 256, None, 32, None, None) == -4


@pytest.mark.parametrize("m,n", [(2048, 1024), (1024, 1024), (4096, 512)])
def test_fp32_dag_with_tensor_cores(tq, oracle, m, n):
    """The FP32 persistent tile QR with its tsmqr updates on the tensor cores
    against the SIMT FP32 schedule and the FP64 oracle (same FP32 inputs)."""
    import torch
    from tileqr import _lib
    L = _lib.lib()
    rng = np.random.default_rng(m + n)
    A0 = np.asfortranarray(rng.standard_normal((m, n)).astype(np.float32).astype(np.float64))
    Ao = A0.copy(order="F")
    oracle.tile_geqrf(Ao, 256, 32)
    R_o = np.triu(Ao[:n])
    errs = {}
    for on in (1, 0):
        L.tqr_tile_dag_tensor_cores(on)
        try:
            A = tq.to_device(A0, torch.float32)
            tq.tile_geqrf(A, 256, 32)
            R = np.triu(tq.to_numpy(A).astype(np.float64)[:n])
        finally:
            L.tqr_tile_dag_tensor_cores(1)
        errs[on] = np.linalg.norm(R - R_o) / np.linalg.norm(R_o)
        # ||A x|| = ||R x||
        x = rng.standard_normal((n, 3))
        assert np.max(np.abs(np.linalg.norm(A0 @ x, axis=0) - np.linalg.norm(R @ x, axis=0)) /
                      np.linalg.norm(A0 @ x, axis=0)) < 1e-5
    assert errs[1] < 2e-5 and errs[1] < 3 * errs[0] + 1e-6, errs


def _with_tma(tq, on, fn):
    from tileqr import _lib
    old = _lib.lib().tqr_tile_tc_tma(1 if on else 0)
    try:
        return fn()
    finally:
        _lib.lib().tqr_tile_tc_tma(old)


def test_tma_and_cp_async_loads_agree_bit_for_bit(tq):
    """The tensor-core updates load their operands with TMA (128-byte-swizzled
    boxes) or, switched off, with 16-byte cp.async copies into the same
    layout: the same values reach the same arithmetic, so the stand-alone
    tsmqr, the flat FP32 tile QR and the hierarchical tree (plain and mixed
    forms, every masked-V mode) give identical bits both ways."""
    import torch
    from tileqr import _lib
    g = torch.Generator(device="cuda").manual_seed(77)
    # stand-alone tsmqr on a 256 x 1024 band
    m2, k, n = 256, 256, 1024
    A1 = tq.empty(k, n, dtype=torch.float32)
    A2 = tq.empty(m2, n, dtype=torch.float32)
    V = tq.empty(m2, k, dtype=torch.float32)
    T = tq.empty(32, k, dtype=torch.float32)
    for t, s in ((A1, 1), (A2, 1), (V, 16), (T, 16)):
        t.copy_(torch.randn(*t.shape, generator=g, device="cuda") / s)
    T.copy_(torch.triu(T))
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    st = torch.cuda.current_stream()

    def band():
        a1, a2 = A1.clone(), A2.clone()
        assert _lib.lib().tqr_stsmqr_tc(k, n, m2, k, P(a1), k, P(a2), m2, P(V), m2, P(T), 32, P(err),
                                        ctypes.c_void_p(st.cuda_stream)) == 0
        torch.cuda.synchronize()
        return a1, a2
    for x, y in zip(_with_tma(tq, True, band), _with_tma(tq, False, band)):
        assert torch.equal(x, y)
    assert int(err.item()) == 0
    # flat persistent FP32 tile QR and the hierarchical tree, plain and mixed
    m, n = 4096, 1024
    A0 = tq.empty(m, n, dtype=torch.float32)
    A0.copy_(torch.randn(m, n, generator=g, device="cuda"))

    def flat():
        A = A0.clone()
        T_, tau = tq.tile_geqrf(A, 256, 32)
        return A, T_, tau

    def tree(f64p):
        def run():
            A = A0.clone()
            return (A,) + tuple(tq.tile_geqrf_tree(A, 256, 32, grp=4, f64p=f64p))
        return run
    for fn in (flat, tree(False), tree(True)):
        for x, y in zip(_with_tma(tq, True, fn), _with_tma(tq, False, fn)):
            assert torch.equal(x, y)
