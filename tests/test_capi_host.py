"""Host-side checks of libtileqr.so that need no GPU.

The library must load, export every entry point include/tileqr.h declares,
and reject illegal arguments the way the reference throws ArgumentError
(test/geqrt.jl:76-81, test/tsqrt.jl error set, test/tsmqr.jl:88-93,
test/unmqr.jl:181-192) -- all before any CUDA call, so these run on a CPU host.
Quick returns on empty sizes also return 0 without touching the device.
"""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    import tileqr_build
    tileqr_build.build()
    from tileqr import _lib
    return _lib.lib()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "tileqr.h")).read()
    return sorted(set(re.findall(r"\b(tqr_[a-z_0-9]+)\s*\(", text)))


def test_exports_every_header_symbol(L):
    syms = header_symbols()
    assert len(syms) >= 24
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from tileqr import _lib
    declared = {f"tqr_{p}{n}" for n in _lib.SIGNATURES for p in _lib.prefixes(n)} | set(_lib.DIAG)
    assert set(header_symbols()) <= declared


NULL = None


def test_geqrt_argument_errors(L):
    assert L.tqr_dgeqrt(-1, 5, 2, NULL, 5, NULL, 2, NULL, NULL, NULL) == -1
    assert L.tqr_dgeqrt(5, -1, 2, NULL, 5, NULL, 2, NULL, NULL, NULL) == -2
    assert L.tqr_dgeqrt(5, 5, -1, NULL, 5, NULL, 2, NULL, NULL, NULL) == -3
    assert L.tqr_dgeqrt(5, 5, 0, NULL, 5, NULL, 2, NULL, NULL, NULL) == -3
    assert L.tqr_dgeqrt(0, 5, 0, NULL, 1, NULL, 1, NULL, NULL, NULL) == 0   # quick return
    assert L.tqr_sgeqrt(-1, 5, 2, NULL, 5, NULL, 2, NULL, NULL, NULL) == -1


def test_tsqrt_argument_errors(L):
    assert L.tqr_dtsqrt(-1, 8, 4, 8, NULL, 8, NULL, 8, NULL, 4, NULL, NULL, NULL) == -1
    assert L.tqr_dtsqrt(8, -1, 4, 8, NULL, 8, NULL, 8, NULL, 4, NULL, NULL, NULL) == -2
    assert L.tqr_dtsqrt(8, 8, -1, 8, NULL, 8, NULL, 8, NULL, 4, NULL, NULL, NULL) == -3
    assert L.tqr_dtsqrt(0, 8, 4, 8, NULL, 8, NULL, 8, NULL, 4, NULL, NULL, NULL) == 0


def test_tsmqr_argument_errors(L):
    args = (8, 8, 8, 8, 4, 2, NULL, 8, NULL, 8, NULL, 8, NULL, 2, NULL, 16, NULL)
    assert L.tqr_dtsmqr(b"X", b"N", *args) == -1
    assert L.tqr_dtsmqr(b"L", b"X", *args) == -2
    # side 'L' needs n2 == n1, side 'R' needs m2 == m1 (src/tsmqr.jl:69-83)
    assert L.tqr_dtsmqr(b"L", b"N", 8, 8, 8, 7, 4, 2, NULL, 8, NULL, 8, NULL, 8, NULL, 2, NULL, 16, NULL) == -6
    assert L.tqr_dtsmqr(b"R", b"N", 8, 8, 7, 8, 4, 2, NULL, 8, NULL, 8, NULL, 8, NULL, 2, NULL, 16, NULL) == -5
    # k = 0 is a no-op (test/tsmqr.jl:75-85)
    assert L.tqr_dtsmqr(b"L", b"N", 8, 8, 8, 8, 0, 0, NULL, 8, NULL, 8, NULL, 8, NULL, 1, NULL, 0, NULL) == 0


def test_unmqr_argument_errors(L):
    a = (32, 24, 16, 4, NULL, 32, NULL, 4, NULL, 32, NULL, 24, NULL)
    assert L.tqr_dunmqr(b"X", b"N", *a) == -1
    assert L.tqr_dunmqr(b"L", b"X", *a) == -2
    assert L.tqr_dunmqr(b"L", b"N", -1, 24, 16, 4, NULL, 32, NULL, 4, NULL, 32, NULL, 24, NULL) == -3
    assert L.tqr_dunmqr(b"L", b"N", 32, 24, 0, 4, NULL, 32, NULL, 4, NULL, 32, NULL, 24, NULL) == 0


def test_reference_argument_error_cases(L):
    """The ArgumentError cases of the reference's own tests that the tests
    above do not already hold, as negative return codes (every element type).
    Each check happens before any CUDA call."""
    for p in "dszc":
        geqr2, ttqrt, ttmqr, parfb = (getattr(L, f"tqr_{p}{n}") for n in ("geqr2", "ttqrt", "ttmqr", "parfb"))
        # test/geqr2.jl:57-58
        assert geqr2(-1, 5, NULL, 5, NULL, NULL, NULL) == -1
        assert geqr2(5, -1, NULL, 5, NULL, NULL, NULL) == -2
        # test/ttqrt.jl:173-175
        assert ttqrt(-1, 8, 4, NULL, 8, NULL, 8, NULL, 4, NULL, NULL, NULL) == -1
        assert ttqrt(8, -1, 4, NULL, 8, NULL, 8, NULL, 4, NULL, NULL, NULL) == -2
        assert ttqrt(8, 8, -1, NULL, 8, NULL, 8, NULL, 4, NULL, NULL, NULL) == -3
        # test/ttmqr.jl:163-165
        t = (8, 8, 8, 8, 4, 2, NULL, 8, NULL, 8, NULL, 8, NULL, 2, NULL, 16, NULL)
        assert ttmqr(b"X", b"N", *t) == -1
        assert ttmqr(b"L", b"X", *t) == -2
        # test/parfb.jl:58-61 (direct and storev are in test_parfb_argument_checks)
        a = (4, 4, 4, 4, 2, 0, NULL, 4, NULL, 4, NULL, 4, NULL, 2, NULL, 2, NULL)
        assert parfb(b"X", b"N", b"F", b"C", *a) == -1
        assert parfb(b"L", b"X", b"F", b"C", *a) == -2


def test_larfb_larft_edge_cases(L):
    # test/larfb.jl:191-196 and test/larft.jl:207-210: empty work is a no-op
    assert L.tqr_dlarfb(b"L", b"N", b"F", b"C", 0, 0, 0, NULL, 1, NULL, 1, NULL, 1, NULL, 1, NULL) == 0
    assert L.tqr_dlarfb(b"L", b"N", b"F", b"C", 5, 5, 0, NULL, 5, NULL, 1, NULL, 5, NULL, 5, NULL) == 0
    assert L.tqr_dlarfb(b"L", b"N", b"B", b"C", 5, 5, 2, NULL, 5, NULL, 2, NULL, 5, NULL, 5, NULL) == -3
    assert L.tqr_dlarft(b"F", b"C", 0, 2, NULL, 1, NULL, NULL, 2, NULL) == 0


def test_parfb_argument_checks(L):
    """Bad flags are argument errors; the backward and rowwise forms need the
    work block (its position, -20, when it is missing); l > k is illegal."""
    a = (4, 6, 4, 6, 3, 0, NULL, 4, NULL, 4, NULL, 4, NULL, 3, NULL, 3, NULL)
    assert L.tqr_dparfb(b"L", b"N", b"X", b"C", *a) == -3
    assert L.tqr_dparfb(b"L", b"N", b"F", b"X", *a) == -4
    assert L.tqr_dparfb(b"L", b"N", b"F", b"R", *a) == -20
    assert L.tqr_dparfb(b"L", b"N", b"B", b"C", *a) == -20
    assert L.tqr_dparfb(b"L", b"N", b"F", b"C", 4, 6, 4, 6, 3, 4, NULL, 4, NULL, 4, NULL, 4, NULL, 3,
                        NULL, 3, NULL) == -10   # l > k


def test_tile_driver_argument_errors(L):
    assert L.tqr_dtile_geqrf(-1, 4, 2, 1, NULL, 4, NULL, 2, NULL, 4, NULL) == -1
    assert L.tqr_dtile_geqrf(4, 4, 0, 1, NULL, 4, NULL, 2, NULL, 4, NULL) == -3
    assert L.tqr_dtile_geqrf(4, 4, 2, 3, NULL, 4, NULL, 2, NULL, 4, NULL) == -4
    assert L.tqr_dtile_geqrf(0, 4, 2, 1, NULL, 1, NULL, 1, NULL, 4, NULL) == 0
    assert L.tqr_dtile_unmqr(b"X", 4, 4, 1, 2, 1, NULL, 4, NULL, 2, NULL, 4, NULL) == -1
    assert L.tqr_dtrsm_lun(-1, 1, NULL, 1, NULL, 1, NULL) == -1
    assert L.tqr_dtile_gels(2, 4, 1, 2, 1, NULL, 2, NULL, 1, NULL, 4, NULL, 2, NULL) == -1


@pytest.mark.parametrize("shape", [(1024, 1024, 256, 32), (2048, 1024, 256, 32), (1024, 2048, 256, 32),
                                   (512, 512, 128, 32), (768, 512, 128, 16), (256, 256, 256, 32),
                                   (1024, 1024, 256, 64), (8192, 8192, 256, 32), (65536, 512, 256, 32)])
def test_dag_schedule_replay(L, shape):
    """The persistent kernel's closed-form wait targets equal a replay of the task
    list, every counter group completes, and the priority sort stays topological."""
    import tileqr
    rc, ntasks = tileqr.dag_check(*shape)
    assert rc == 0 and ntasks > 0


@pytest.mark.parametrize("q", [1.0, 8.0, 64.0])
@pytest.mark.parametrize("shape", [(1024, 1024, 256, 32), (4096, 2048, 256, 32), (8192, 8192, 256, 32)])
def test_dag_bucketed_order_stays_topological(L, shape, q):
    """The priority sort in rank buckets (loop order inside a bucket) keeps
    every dependency ahead of its task."""
    import tileqr
    old = L.tqr_tile_dag_order_quantum(q)
    try:
        rc, ntasks = tileqr.dag_check(*shape)
    finally:
        L.tqr_tile_dag_order_quantum(old)
    assert rc == 0 and ntasks > 0


def test_dag_shape_eligibility(L):
    import tileqr
    assert tileqr.dag_worksize(1000, 1000, 256, 32) is None      # not a multiple of nb
    assert tileqr.dag_worksize(1024, 1024, 512, 32) is None      # tile wider than one CTA holds
    assert tileqr.dag_worksize(1024, 1024, 256, 128) is None     # T/V blocks exceed shared memory
    assert tileqr.dag_worksize(8192, 8192, 256, 32) > 0


@pytest.mark.parametrize("shape", [(1024, 1024, 4, 256, 32), (32768, 4096, 4, 256, 32),
                                   (2048, 512, 3, 256, 32), (4096, 1024, 16, 256, 32),
                                   (768, 512, 1, 128, 16)])
def test_dag_schedule_replay_with_rhs_tile(L, shape):
    """Least-squares schedules: B rides along as one extra tile column."""
    nt = ctypes.c_longlong(0)
    assert L.tqr_tile_dag_check_rhs(*shape, ctypes.byref(nt)) == 0 and nt.value > 0


@pytest.mark.parametrize("m,n,nb,ib,nrhs", [(65536, 512, 256, 32, 0), (1000, 300, 128, 16, 5), (300, 400, 256, 32, 0),
                                            (64, 200, 32, 16, 3), (517, 130, 64, 16, 0), (4096, 4096, 256, 32, 4)])
def test_tree_task_graph_is_topological(L, m, n, nb, ib, nrhs):
    """The tree task graph's dependencies all point to earlier tasks (the
    persistent kernel's deadlock-freedom argument)."""
    nt = ctypes.c_longlong(0)
    assert L.tqr_tile_tree_dag_check(m, n, nb, ib, nrhs, ctypes.byref(nt)) == 0
    assert nt.value > 0


def test_tree_task_graph_shape_limits(L):
    size = ctypes.c_size_t(0)
    assert L.tqr_tile_tree_dag_worksize(100, 100, 64, 8, 0, ctypes.byref(size)) == -1      # ib not a multiple of 16
    assert L.tqr_tile_tree_dag_worksize(100, 100, 512, 32, 0, ctypes.byref(size)) == -1    # nb > 256
    assert L.tqr_tile_tree_dag_worksize(1024, 256, 256, 32, 0, ctypes.byref(size)) == 0 and size.value > 0


@pytest.mark.parametrize("m,n,nrhs", [(1024, 1024, 0), (4096, 1024, 4), (32768, 4096, 4), (512, 1024, 0)])
def test_tensor_core_dag_schedule_replays(L, m, n, nrhs):
    """The FP32 schedule with 128-column tensor-core tsmqr tasks: every wait
    target equals the number of writers before the task in program order."""
    nt = ctypes.c_longlong(0)
    assert L.tqr_tile_dag_check_tc(m, n, nrhs, 256, 32, ctypes.byref(nt)) == 0
    assert nt.value > 0


def test_complex_entry_points_exported(L):
    """ComplexF64 / ComplexF32 forms of every tile kernel and of the tile QR."""
    from tileqr import _lib
    for name in _lib.COMPLEX:
        for p in "zc":
            assert hasattr(L, f"tqr_{p}{name}"), (p, name)


def test_complex_argument_errors(L):
    """Same argument checks as the real forms, plus element alignment."""
    import ctypes
    z = ctypes.c_void_p(16)       # aligned; never dereferenced: the calls fail their checks first
    assert L.tqr_zgeqrt(-1, 4, 2, z, 4, z, 2, z, None, None) == -1
    assert L.tqr_zgeqrt(4, 4, 0, z, 4, z, 2, z, None, None) == -3
    assert L.tqr_zgeqrt(4, 4, 2, ctypes.c_void_p(8), 4, z, 2, z, None, None) == -4    # 8-byte aligned A
    assert L.tqr_cgeqrt(4, 4, 2, ctypes.c_void_p(4), 4, z, 2, z, None, None) == -4    # 4-byte aligned A
    assert L.tqr_ztsmqr(b"X", b"N", 8, 8, 8, 8, 4, 2, z, 8, z, 8, z, 8, z, 2, None, 0, None) == -1
    assert L.tqr_ztsmqr(b"L", b"Q", 8, 8, 8, 8, 4, 2, z, 8, z, 8, z, 8, z, 2, None, 0, None) == -2
    assert L.tqr_zunmqr(b"L", b"C", 8, 8, 4, 2, z, 8, z, 2, ctypes.c_void_p(24), 8, None, 0, None) == -11
    assert L.tqr_ztile_geqrf(8, 8, 4, 8, z, 8, z, 8, z, 8, None) == -4                  # ib > nb


def test_complex_adjoint_argument_errors(L):
    """The differentiable QR's checks, all made before any CUDA call: batch,
    n <= 256, m >= n, ib <= 32, element alignment, and the complex backward's
    m > n (a square complex problem keeps a complex R_nn, src/geqr2.jl:32-35)."""
    import ctypes
    z = ctypes.c_void_p(256)
    for p in "zc":
        fwd, bwd = getattr(L, f"tqr_{p}qr_batched_fwd"), getattr(L, f"tqr_{p}qr_batched_bwd")
        assert fwd(-1, 64, 32, 32, z, z, z, z, z, 1 << 20, None) == -1
        assert fwd(1, 600, 257, 32, z, z, z, z, z, 1 << 20, None) == -3
        assert fwd(1, 31, 32, 32, z, z, z, z, z, 1 << 20, None) == -2
        assert fwd(1, 64, 32, 33, z, z, z, z, z, 1 << 20, None) == -4
        assert bwd(1, 40, 40, 32, z, z, z, z, z, z, 1 << 20, None) == -2     # square: refused
        assert bwd(1, 41, 40, 33, z, z, z, z, z, z, 1 << 20, None) == -4     # m > n passes the -2 check
        assert bwd(0, 41, 40, 32, z, z, z, z, z, z, 1 << 20, None) == 0      # empty batch: nothing to do
        assert bwd(1, 41, 40, 32, None, z, z, z, z, z, 1 << 20, None) == -5
    assert L.tqr_zqr_batched_bwd(1, 41, 40, 32, ctypes.c_void_p(8), z, z, z, z, z, 1 << 20, None) == -5  # 8-byte aligned
    # the real backward keeps square problems (R's diagonal needs no gauge there)
    assert L.tqr_dqr_batched_bwd(1, 40, 40, 33, z, z, z, z, z, z, 1 << 20, None) == -4


@pytest.mark.parametrize("m,n,nb,ib,grp,nrhs", [(2048, 512, 128, 32, 4, 3), (4096, 1024, 256, 32, 8, 5),
                                                (517, 130, 64, 16, 3, 2), (32768, 4096, 256, 32, 16, 4),
                                                (65536, 512, 256, 32, 8, 0)])
def test_hqr_task_graph_is_topological(L, m, n, nb, ib, grp, nrhs):
    """The hierarchical schedule: every dependency precedes its task; more
    groups than tiles degenerates to the flat tree, grp = 1 to the binary tree."""
    import ctypes
    nt = ctypes.c_longlong(0)
    assert L.tqr_tile_hqr_dag_check(m, n, nb, ib, grp, nrhs, ctypes.byref(nt)) == 0
    assert nt.value > 0
    one, tree = ctypes.c_longlong(0), ctypes.c_longlong(0)
    assert L.tqr_tile_hqr_dag_check(m, n, nb, ib, 1, nrhs, ctypes.byref(one)) == 0
    assert L.tqr_tile_tree_dag_check(m, n, nb, ib, nrhs, ctypes.byref(tree)) == 0
    assert one.value == tree.value


@pytest.mark.parametrize("m,n,grp,nrhs", [(4096, 1024, 4, 3), (8192, 512, 8, 0), (32768, 4096, 16, 4),
                                        (2048, 2048, 2, 1)])
def test_hqr_tensor_core_task_graph_is_topological(L, m, n, grp, nrhs):
    """The FP32 hierarchical schedule with every trailing update of A (the
    leaders' unmqr!, the tsqrt merges' tsmqr!, the ttqrt merges' ttmqr!) as
    tensor-core chunk tasks: still topological, and one chunk task per 128
    trailing columns of A per geqrt and per merge."""
    import ctypes
    nt = ctypes.c_longlong(0)
    assert L.tqr_tile_hqr_dag_check_tc(m, n, 256, 32, grp, nrhs, ctypes.byref(nt)) == 0
    MT, NT = m // 256, n // 256
    expect = 0
    for k in range(min(MT, NT)):
        leaders = len(range(k, MT, grp))     # one geqrt! each
        merges = (MT - k) - 1                # every tile but tile k is merged once
        expect += (leaders + merges) * (n - (k + 1) * 256) // 128
    assert nt.value == expect
    assert L.tqr_tile_hqr_dag_check_tc(m + 100, n, 256, 32, grp, nrhs, ctypes.byref(nt)) == -1   # ragged


@pytest.mark.parametrize("m,n,grp,nrhs", [(4096, 1024, 4, 3), (8192, 512, 8, 0), (32768, 4096, 16, 4),
                                        (2048, 2048, 2, 1), (8192, 8192, 1, 0)])
def test_hqr_compact_wy_task_graph(L, m, n, grp, nrhs):
    """The same schedule in compact-WY form: one slot build per geqrt and per
    merge that has trailing columns of A, the same chunk tasks as the blocked
    form, each waiting for its own tile's build, and every rebuild of a slot
    (two panels later) waiting for all chunks that read it before."""
    import ctypes
    nbld, nch, ntc = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_longlong(0)
    assert L.tqr_tile_hqr_dag_check_wy(m, n, 256, 32, grp, nrhs, ctypes.byref(nbld), ctypes.byref(nch)) == 0
    assert L.tqr_tile_hqr_dag_check_tc(m, n, 256, 32, grp, nrhs, ctypes.byref(ntc)) == 0
    assert nch.value == ntc.value
    MT, NT = m // 256, n // 256
    expect = 0
    for k in range(min(MT, NT)):
        if n - (k + 1) * 256 > 0:
            expect += len(range(k, MT, grp)) + (MT - k) - 1
    assert nbld.value == expect
    assert L.tqr_tile_hqr_dag_check_wy(m + 100, n, 256, 32, grp, nrhs, ctypes.byref(nbld),
                                       ctypes.byref(nch)) == -1   # ragged


def test_tile_autotune_argument_errors(L):
    nb, ib = ctypes.c_int(0), ctypes.c_int(0)
    assert L.tqr_tile_autotune(3, 64, 64, 0, ctypes.byref(nb), ctypes.byref(ib), NULL) == -1
    assert L.tqr_tile_autotune(8, 0, 64, 0, ctypes.byref(nb), ctypes.byref(ib), NULL) == -2
    assert L.tqr_tile_autotune(8, 64, -1, 0, ctypes.byref(nb), ctypes.byref(ib), NULL) == -3
    assert L.tqr_tile_autotune(8, 64, 64, 0, NULL, ctypes.byref(ib), NULL) == -5
    assert L.tqr_tile_autotune(4, 64, 64, 0, ctypes.byref(nb), NULL, NULL) == -6
    # nothing tuned for this shape yet
    assert L.tqr_tile_tuning(8, 12345, 77, ctypes.byref(nb), ctypes.byref(ib)) == 1
    assert L.tqr_tile_tuning(8, 64, 64, NULL, ctypes.byref(ib)) == -4


@pytest.mark.parametrize("n", [1, 256, 300, 1024, 4096, 5000, 16384])
def test_pipelined_triangular_solve_task_list(L, n):
    """The mixed solve's pipelined R^-1 / R^-T task list: every wait is on
    work finished earlier in the list (so the first unfinished task can
    always run), each row block applies the solved blocks in order before
    its own product, and every task appears once."""
    import ctypes
    nt = ctypes.c_longlong(0)
    assert L.tqr_dsgels_trsv_pipe_check(n, ctypes.byref(nt)) == 0
    nblk = (n + 255) // 256
    assert nt.value == 32 * (nblk + nblk * (nblk - 1) // 2)
    assert L.tqr_dsgels_trsv_pipe_check(0, ctypes.byref(nt)) == -1


@pytest.mark.parametrize("m,n,nb,ib,grp,nrhs", [(1024, 512, 128, 32, 2, 3), (1000, 300, 128, 16, 1, 0),
                                                (32768, 4096, 256, 32, 16, 4), (2048, 256, 256, 32, 4, 5)])
def test_tree_task_graph_with_8_column_strips(L, m, n, nb, ib, grp, nrhs):
    """The ComplexF64 task graph (8-column strips): topological, with twice the
    strip tasks of the 16-column graph; the worksize query covers it."""
    n8, n16 = ctypes.c_longlong(0), ctypes.c_longlong(0)
    assert L.tqr_tile_hqr_dag_check_strips(m, n, nb, ib, grp, nrhs, 8, ctypes.byref(n8)) == 0
    assert L.tqr_tile_hqr_dag_check_strips(m, n, nb, ib, grp, nrhs, 16, ctypes.byref(n16)) == 0
    assert n8.value > n16.value
    assert L.tqr_tile_hqr_dag_check_strips(m, n, nb, 20, grp, nrhs, 8, ctypes.byref(n8)) == -1   # ib % 8


@pytest.mark.parametrize("shape", [(1024, 1024, 256, 32), (2048, 1024, 256, 32), (1024, 2048, 256, 32),
                                   (512, 512, 128, 32), (768, 512, 128, 16), (256, 256, 256, 32),
                                   (1024, 1024, 256, 64), (4096, 4096, 256, 32), (8192, 8192, 256, 32),
                                   (65536, 512, 256, 32), (512, 4096, 256, 32), (16384, 4096, 256, 32),
                                   (8192, 2048, 256, 32), (4096, 8192, 256, 32), (3072, 2048, 128, 16),
                                   (2560, 2560, 256, 32)])
def test_noalloc_bucket_order_replays(L, shape):
    """The allocation-free tile QR's device-written task order (buckets of
    key 4 min(column, k + 1) + row, loop order inside a bucket): every
    dependency listed before its task, every task of the loop order exactly
    once, and the generator's count pass agrees with its write pass."""
    nt = ctypes.c_longlong(0)
    assert L.tqr_tile_noalloc_check(*shape, ctypes.byref(nt)) == 0
    import tileqr
    rc, ntasks = tileqr.dag_check(*shape)
    assert rc == 0 and nt.value == ntasks
    assert L.tqr_tile_noalloc_check(1000, 1000, 256, 32, ctypes.byref(nt)) == -1


@pytest.mark.parametrize("shape,bound", [((2048, 2048, 256, 32), 1.05), ((4096, 4096, 256, 32), 1.40),
                                         ((8192, 8192, 256, 32), 1.33), ((16384, 4096, 256, 32), 1.75)])
def test_noalloc_order_simulated_makespan(L, shape, bound):
    """The allocation-free order against the workspace path's longest-path
    order in the host simulation of the persistent kernel (304 CTAs taking
    tasks in list order).  The bounds hold the simulated ratios the order was
    chosen for (1.00 / 1.35 / 1.29 / 1.70; the one-step lookahead it replaced
    simulated at 1.17 / 2.34 / 2.19 / 5.49).  Measured on a GB300: 1.13x at
    4096^2 and 1.10x at 8192^2."""
    a, b, ideal = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    assert L.tqr_tile_dag_simulate(*shape, 304, ctypes.byref(a), ctypes.byref(b), ctypes.byref(ideal)) == 0
    assert ideal.value > 0 and b.value >= ideal.value
    assert a.value >= ideal.value
    assert a.value / b.value <= bound, (a.value / b.value)
    assert L.tqr_tile_dag_simulate(1000, 1000, 256, 32, 304, None, None, None) == -1
    assert L.tqr_tile_dag_simulate(*shape, 0, None, None, None) == -5
