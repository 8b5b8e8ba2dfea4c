"""The allocation-free tile QR entry point, tqr_dtile_geqrf_noalloc.

Some callers cannot give the library device memory for its task schedule:
a framework whose caching allocator already owns the device, host code that
must not take the device-wide synchronisation cudaMalloc/cudaFree can imply,
or a binding with nowhere to keep a scratch buffer alive between calls.  For
them the schedule lives in a fixed array inside the library.  These tests call
that entry point through the C ABI and compare it bit for bit with the
workspace entry point (tile_geqrf on the persistent kernel), and read its
error word through tqr_tile_noalloc_status, twice in a row, because the
array keeps the previous call's contents and every call must clear what it
needs.  This file is collected last so a failure here comes after every other
test has run; it also passes on its own in a fresh process.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

TQR_ERR_SCRATCH_TOO_SMALL = -1000


def _noalloc(tq, A, T, tau, nb, ib):
    import torch
    m, n = A.shape
    pa, lda = tq._mat(A)
    pt, ldt = tq._mat(T)
    pu, ldu = tq._mat(tau)
    st = torch.cuda.current_stream()
    rc = tq._lib.lib().tqr_dtile_geqrf_noalloc(m, n, nb, ib, pa, lda, pt, ldt, pu, ldu,
                                               ctypes.c_void_p(st.cuda_stream))
    st.synchronize()
    return rc


def _noalloc_status(tq):
    """Error word of the last allocation-free launch (0 = every task ran)."""
    import torch
    status, task = ctypes.c_int(-1), ctypes.c_int(-1)
    st = torch.cuda.current_stream()
    rc = tq._lib.lib().tqr_tile_noalloc_status(ctypes.byref(status), ctypes.byref(task),
                                               ctypes.c_void_p(st.cuda_stream))
    assert rc == 0
    return status.value, task.value


@pytest.mark.parametrize("m,n,nb,ib", [(1024, 1024, 256, 32), (2048, 1024, 256, 32), (4096, 4096, 256, 32),
                                      (8192, 2048, 256, 32)])
def test_noalloc_matches_workspace_entry_point_twice(tq, m, n, nb, ib):
    import torch
    for call, seed in enumerate((11, 12)):
        g = torch.Generator(device="cuda").manual_seed(seed + m)
        A0 = tq.empty(m, n)
        A0.copy_(torch.randn(m, n, generator=g, dtype=torch.float64, device="cuda"))
        ts, taus = tq.tile_shapes(m, n, nb, ib)
        # the existing entry point (caller-provided workspace)
        A1 = A0.clone()
        T1, tau1 = tq.tile_geqrf(A1, nb, ib, dag=True)
        # the allocation-free entry point
        A2 = A0.clone()
        T2, tau2 = tq.zeros(*ts), tq.zeros(*taus)
        assert _noalloc(tq, A2, T2, tau2, nb, ib) == 0, f"call {call}"
        assert _noalloc_status(tq) == (0, 0), f"call {call}"
        # every strip sees the same operations in the same order on both
        # paths (only the order in which CTAs take tasks differs), so the
        # results agree bit for bit
        for x, y in ((A2, A1), (T2, T1), (tau2, tau1)):
            assert torch.equal(x, y), f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_array(tq):
    """16384^2 needs more schedule than the fixed array holds: a clear error,
    and nothing is launched (the null matrix pointers are never touched)."""
    n = 16384
    rc = tq._lib.lib().tqr_dtile_geqrf_noalloc(n, n, 256, 32, None, n, None, (n // 256) * 32, None, n,
                                               None)
    assert rc == TQR_ERR_SCRATCH_TOO_SMALL
