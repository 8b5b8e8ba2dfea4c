"""The (nb, ib) autotuner of the tile QR (tqr_tile_autotune).

It must return one of its candidate tilings, cache it per (element type, m,
n), and the tuned factorisation must be the tile QR of that tiling: equal to
the oracle's flat-tree tile QR with the same (nb, ib) within the FP64 parity
bar 1e-12 * n (FP32: 1e-5 * n on the float32-rounded input).
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

CANDIDATES = {(256, 32), (256, 16), (256, 64), (128, 32), (128, 16), (64, 16), (64, 32)}


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("m,n", [(1024, 1024), (768, 512), (300, 200)])
def test_autotuned_tile_qr_matches_oracle(tq, oracle, m, n):
    from tileqr import _lib
    nb, ib = tq.autotune_tiling(m, n, torch.float64)
    assert (nb, ib) in CANDIDATES
    # cached: the table holds the pair and a second call returns it
    cb, ci = ctypes.c_int(0), ctypes.c_int(0)
    assert _lib.lib().tqr_tile_tuning(8, m, n, ctypes.byref(cb), ctypes.byref(ci)) == 0
    assert (cb.value, ci.value) == (nb, ib)
    assert tq.autotune_tiling(m, n, torch.float64) == (nb, ib)
    rng = np.random.default_rng(m + 3 * n)
    A0 = np.asfortranarray(rng.standard_normal((m, n)))
    A = tq.to_device(A0)
    T, tau, nb2, ib2 = tq.tile_geqrf_tuned(A)
    assert (nb2, ib2) == (nb, ib)
    Ao = A0.copy(order="F")
    To, _ = oracle.tile_geqrf(Ao, nb, ib)
    tol = 1e-12 * max(m, n)
    assert rel(tq.to_numpy(A), Ao) < tol
    assert rel(tq.to_numpy(T), To) < tol


def test_autotuned_tile_qr_float32(tq, oracle):
    m, n = 512, 512
    nb, ib = tq.autotune_tiling(m, n, torch.float32)
    assert (nb, ib) in CANDIDATES
    rng = np.random.default_rng(11)
    A0 = np.asfortranarray(rng.standard_normal((m, n)).astype(np.float32))
    A = tq.to_device(A0, dtype=torch.float32)
    T, tau, _, _ = tq.tile_geqrf_tuned(A)
    Ao = np.asfortranarray(A0.astype(np.float64))
    oracle.tile_geqrf(Ao, nb, ib)
    assert rel(tq.to_numpy(A).astype(np.float64), Ao) < 1e-5 * n


def test_autotune_force_retimes(tq):
    a = tq.autotune_tiling(256, 256, torch.float64)
    b = tq.autotune_tiling(256, 256, torch.float64, force=True)
    assert a in CANDIDATES and b in CANDIDATES
