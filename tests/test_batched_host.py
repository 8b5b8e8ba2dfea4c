"""Host-side checks of the batched planner (tqr_batched_plan, no GPU needed).

The planner packs problem q's A and B at 32-element-aligned offsets, takes the
inner block size and strip width from the tuning table, orders the problems by
decreasing flops and rejects out-of-range sizes with -(1000 + q).
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def B():
    import tileqr_build
    tileqr_build.build()
    from tileqr import batched
    return batched


def test_descriptor_layout(B):
    from tileqr import _lib
    assert _lib.lib().tqr_batched_problem_bytes() == B.PROBLEM_DTYPE.itemsize == 40


def test_plan_offsets_order_and_tuning(B):
    import torch
    ms, ns, ks = B.random_sizes(257, seed=3)
    for dt in (torch.float64, torch.float32):
        desc, order, ae, be = B.plan(ms, ns, ks, dt)
        assert (desc["m"] == ms).all() and (desc["n"] == ns).all() and (desc["k"] == ks).all()
        # packed, aligned, non-overlapping
        a_end = desc["a_off"] + desc["m"].astype(np.int64) * desc["n"]
        b_end = desc["b_off"] + desc["m"].astype(np.int64) * desc["k"]
        assert (desc["a_off"] % 32 == 0).all() and (desc["b_off"] % 32 == 0).all()
        assert (desc["a_off"][1:] >= a_end[:-1]).all() and (desc["b_off"][1:] >= b_end[:-1]).all()
        assert a_end[-1] <= ae and b_end[-1] <= be
        # order: a permutation by non-increasing flops
        assert sorted(order.tolist()) == list(range(len(ms)))
        m = desc["m"].astype(float)[order]
        n = desc["n"].astype(float)[order]
        k = desc["k"].astype(float)[order]
        cost = 2 * m * n * n - 2 * n ** 3 / 3 + 4 * m * n * k
        assert (np.diff(cost) <= 1e-6 * cost[:-1]).all()
        for q in range(len(ms)):
            ib, nw = B.tuning(dt, int(ns[q]))
            assert desc["ib"][q] == min(ib, ns[q]) and desc["nw"][q] == nw
            assert 1 <= desc["ib"][q] <= 32 and desc["nw"][q] in (8, 16)


@pytest.mark.parametrize("bad", [(600, 16, 1), (32, 40, 1), (32, 0, 1), (64, 16, 9), (64, 16, -1), (0, 0, 0)])
def test_plan_rejects_out_of_range(B, bad):
    import torch
    ms = np.array([100, bad[0], 50], dtype=np.int32)
    ns = np.array([20, bad[1], 50], dtype=np.int32)
    ks = np.array([2, bad[2], 8], dtype=np.int32)
    with pytest.raises(B.ArgumentError, match="problem 1"):
        B.plan(ms, ns, ks, torch.float64)


def test_plan_empty_and_qr_only(B):
    import torch
    desc, order, ae, be = B.plan([], [], [], torch.float64)
    assert len(desc) == 0 and len(order) == 0 and ae >= 1 and be >= 1
    desc, order, ae, be = B.plan([64, 32], [64, 16], [0, 0], torch.float32)
    assert (desc["k"] == 0).all() and ae >= 64 * 64 + 32 * 16


def test_tuning_argument_errors(B):
    import ctypes
    from tileqr import _lib
    L = _lib.lib()
    ib, nw = ctypes.c_int(0), ctypes.c_int(0)
    assert L.tqr_batched_tuning(3, 10, ctypes.byref(ib), ctypes.byref(nw)) == -1
    assert L.tqr_batched_tuning(8, 0, ctypes.byref(ib), ctypes.byref(nw)) == -2
    assert L.tqr_batched_tuning(8, 513, ctypes.byref(ib), ctypes.byref(nw)) == -2
    assert L.tqr_dbatched_gels(-1, None, None, None, None, None, 0, None) == -1
    assert L.tqr_dbatched_residual(0, None, None, None, None, None, None) == 0
