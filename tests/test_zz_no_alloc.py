"""The allocation-free tile QR entry point, tqr_dtile_geqrf_noalloc.

Some callers cannot give the library device memory for its task schedule:
a framework whose caching allocator already owns the device, host code that
must not take the device-wide synchronisation cudaMalloc/cudaFree can imply,
or a binding with nowhere to keep a scratch buffer alive between calls.  For
them the schedule lives in a fixed array inside the library.  These tests call
that entry point through the C ABI and compare it with the workspace entry
point (tile_geqrf on the persistent kernel), twice in a row, because the
array keeps the previous call's contents and every call must clear what it
needs.  This file is collected last so a failure here comes after every other
test has run; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
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


@pytest.mark.parametrize("m,n,nb,ib", [(1024, 1024, 256, 32), (2048, 1024, 256, 32)])
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
        tol = 1e-12 * max(m, n)
        for x, y in ((A2, A1), (T2, T1), (tau2, tau1)):
            a, b = x.cpu().numpy(), y.cpu().numpy()
            assert np.max(np.abs(a - b)) <= tol * max(np.max(np.abs(b)), 1e-300), f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_array(tq):
    """16384^2 needs more schedule than the fixed array holds: a clear error,
    and nothing is launched (the null matrix pointers are never touched)."""
    n = 16384
    rc = tq._lib.lib().tqr_dtile_geqrf_noalloc(n, n, 256, 32, None, n, None, (n // 256) * 32, None, n,
                                               None)
    assert rc == TQR_ERR_SCRATCH_TOO_SMALL
