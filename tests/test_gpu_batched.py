"""Batched uneven QR + least squares on the GPU against the oracle.

Each problem's oracle is NextLA's single-tile path restated in C: tile QR with
one tile (geqrt!, src/geqrt.jl:22-68), Q^T B (unmqr!, src/unmqr.jl:52-149) and
LeftUpperTRSM! (src/trsm.jl:36-63).  Checked per problem: R and V of the
factored A (relative difference <= 1e-12 n in FP64), X against the oracle's X
(relative difference bounded through the condition number) and the
normal-equation residual ||A^T (B - A X)|| / (||A|| (||A|| ||X|| + ||B||)).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# edge shapes: a single element, one column, square at the maximum size,
# QR only (k = 0), ragged block sizes, the most right-hand sides
EDGE = [(1, 1, 1), (32, 16, 1), (512, 512, 8), (512, 1, 3), (300, 300, 0), (33, 17, 8), (2, 2, 2),
        (129, 65, 5), (64, 64, 0), (511, 257, 7)]


def sizes_with_edges(nrand, seed):
    from tileqr import batched as Bt
    ms, ns, ks = Bt.random_sizes(nrand, seed=seed)
    ms = np.concatenate([ms, [e[0] for e in EDGE]]).astype(np.int32)
    ns = np.concatenate([ns, [e[1] for e in EDGE]]).astype(np.int32)
    ks = np.concatenate([ks, [e[2] for e in EDGE]]).astype(np.int32)
    return ms, ns, ks


def fill(bg, seed, torch):
    g = torch.Generator(device="cuda").manual_seed(seed)
    bg.A.copy_(torch.randn(bg.A.shape, generator=g, device="cuda", dtype=torch.float64))
    bg.B.copy_(torch.randn(bg.B.shape, generator=g, device="cuda", dtype=torch.float64))


def oracle_solve(oracle, A, B, ib):
    A = np.array(A, order="F", dtype=np.float64)
    B = np.array(B, order="F", dtype=np.float64)
    m, n = A.shape
    nb = max(m, n)
    T, _ = oracle.tile_geqrf(A, nb, ib)
    X = None
    if B.shape[1] > 0:
        oracle.tile_unmqr("C", A, T, B, nb, ib)
        X = np.array(B[:n], order="F")
        oracle.trsm_lun(A[:n, :n], X)
    return A, X


def check_against_oracle(bg, A0, B0, oracle, qs, r_tol, x_tol_unit):
    import torch
    Ah = bg.A.double().cpu().numpy()
    Bh = bg.B.double().cpu().numpy()
    A0h = A0.double().cpu().numpy()
    B0h = B0.double().cpu().numpy()
    for q in qs:
        d = bg.desc[q]
        m, n, k, ib = int(d["m"]), int(d["n"]), int(d["k"]), int(d["ib"])
        ao, bo = int(d["a_off"]), int(d["b_off"])
        Aq = A0h[ao:ao + m * n].reshape(n, m).T
        Bq = B0h[bo:bo + m * k].reshape(k, m).T
        Af, X = oracle_solve(oracle, Aq, Bq, ib)
        Ag = Ah[ao:ao + m * n].reshape(n, m).T
        rd = np.linalg.norm(Ag - Af) / max(np.linalg.norm(Af), 1e-300)
        assert rd <= r_tol * n, (q, m, n, k, ib, rd)
        if k > 0:
            Xg = Bh[bo:bo + m * k].reshape(k, m).T[:n]
            kappa = np.linalg.cond(Aq)
            xd = np.linalg.norm(Xg - X) / max(np.linalg.norm(X), 1e-300)
            assert xd <= max(x_tol_unit * kappa * n, 1e3 * x_tol_unit), (q, m, n, k, xd, kappa)


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_batched_matches_oracle(tq, oracle, dtype_name):
    import torch
    from tileqr import batched as Bt
    dt = getattr(torch, dtype_name)
    ms, ns, ks = sizes_with_edges(54, seed=11)
    bg = Bt.BatchedGels(ms, ns, ks, dtype=dt, tune=False)
    fill(bg, 5, torch)
    A0, B0 = bg.A.clone(), bg.B.clone()
    bg.run()
    assert bg.status() == (0, -1)
    res = bg.residuals(A0, B0).cpu().numpy()
    if dt == torch.float64:
        check_against_oracle(bg, A0, B0, oracle, range(bg.nprob), 1e-12, 1e-15)
        assert res.max() < 1e-14, res.max()
    else:
        check_against_oracle(bg, A0, B0, oracle, range(bg.nprob), 1e-5, 1e-6)
        assert res.max() < 1e-5, res.max()
    # QR-only problems report residual 0
    assert (res[bg.desc["k"] == 0] == 0).all()


def test_batched_graph_replay_is_bitwise_repeatable(tq):
    import torch
    from tileqr import batched as Bt
    ms, ns, ks = sizes_with_edges(200, seed=2)
    bg = Bt.BatchedGels(ms, ns, ks, dtype=torch.float64, tune=False)
    fill(bg, 9, torch)
    A0, B0 = bg.A.clone(), bg.B.clone()
    bg.run()
    A1, B1 = bg.A.clone(), bg.B.clone()
    for _ in range(2):
        bg.A.copy_(A0)
        bg.B.copy_(B0)
        bg.replay()
        assert bg.status() == (0, -1)
        assert torch.equal(bg.A, A1) and torch.equal(bg.B, B1)
    bg.close()


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_batched_full_configuration(tq, oracle, dtype_name):
    """4096 problems, m ~ U[32,512], n ~ U[16,m], k ~ U[1,8], N(0,1) entries,
    one graph replay; every residual small and a sample checked in full."""
    import torch
    from tileqr import batched as Bt
    dt = getattr(torch, dtype_name)
    ms, ns, ks = Bt.random_sizes(4096, seed=0)
    bg = Bt.BatchedGels(ms, ns, ks, dtype=dt, tune=True)
    fill(bg, 1, torch)
    A0, B0 = bg.A.clone(), bg.B.clone()
    bg.replay()
    assert bg.status() == (0, -1)
    res = bg.residuals(A0, B0).cpu().numpy()
    assert np.isfinite(res).all()
    assert res.max() < (1e-14 if dt == torch.float64 else 1e-5), res.max()
    rng = np.random.default_rng(4)
    qs = rng.choice(bg.nprob, size=24, replace=False)
    if dt == torch.float64:
        check_against_oracle(bg, A0, B0, oracle, qs, 1e-12, 1e-15)
    else:
        check_against_oracle(bg, A0, B0, oracle, qs, 1e-5, 1e-6)
    bg.close()


def test_batched_autotune_table(tq):
    import torch
    from tileqr import batched as Bt
    for dt in (torch.float64, torch.float32):
        Bt.autotune(dt, force=True)
        for n in (16, 40, 100, 200, 400, 512):
            ib, nw = Bt.tuning(dt, n)
            assert 1 <= ib <= 32 and nw in (8, 16)


def test_batched_rejects_corrupt_descriptor(tq):
    """A descriptor changed on the device after planning is skipped and
    reported; every other problem is still solved."""
    import torch
    from tileqr import batched as Bt
    ms, ns, ks = Bt.random_sizes(40, seed=8)
    bg = Bt.BatchedGels(ms, ns, ks, dtype=torch.float64, tune=False)
    fill(bg, 3, torch)
    A0, B0 = bg.A.clone(), bg.B.clone()
    bad = bg.desc.copy()
    bad[17]["m"] = 4096
    bg.d_desc.copy_(torch.from_numpy(bad.view(np.uint8).copy()))
    bg.run()
    assert bg.status() == (1, 17)
    res = bg.residuals(A0, B0).cpu().numpy()
    assert res[17] == -1.0
    ok = np.arange(bg.nprob) != 17
    assert res[ok].max() < 1e-14
    # the rejected problem's data is untouched
    assert torch.equal(bg.a_view(17), bg.a_view(17, A0))


def test_sharded_batch_one_rank(tq):
    """The multi-rank batched measurement with a single rank: the whole batch,
    all of its cost, no rejected descriptors."""
    import os
    import sys
    import torch
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    r = bench.batched_sharded_bench(torch, 512, 1, 0, steps=1, warmup=1)
    assert r["rank0_problems"] == 512 and abs(r["rank0_cost_share"] - 1.0) < 1e-12
    assert r["rejected_descriptors_rank0"] == 0 and r["problems_per_s"] > 0


def zoracle_solve(oracle, A, B, ib):
    A = np.array(A, order="F", dtype=np.complex128)
    B = np.array(B, order="F", dtype=np.complex128)
    m, n = A.shape
    nb = max(m, n)
    T, _ = oracle.tile_geqrf(A, nb, ib)
    X = None
    if B.shape[1] > 0:
        oracle.tile_unmqr("C", A, T, B, nb, ib)
        X = np.array(B[:n], order="F")
        oracle.trsm_lun(A[:n, :n], X)
    return A, X


@pytest.mark.parametrize("dtype_name", ["complex128", "complex64"])
def test_complex_batched_matches_oracle(tq, oracle, dtype_name):
    """ComplexF64 / ComplexF32 batches (the reference's kernels run both,
    test/lapack_helpers.jl:11): every problem's factored A and its solution
    against the complex oracle's single-tile path (zgeqrt!, unmqr!('L','C'),
    LeftUpperTRSM! with Smith's division) on the same inputs, and the
    normal-equation residual ||A^H (B - A X)|| / (||A|| (||A|| ||X|| + ||B||))."""
    import torch
    from tileqr import batched as Bt
    dt = getattr(torch, dtype_name)
    ms, ns, ks = sizes_with_edges(30, seed=13)
    bg = Bt.BatchedGels(ms, ns, ks, dtype=dt, tune=True)
    g = torch.Generator(device="cuda").manual_seed(9)
    cre = lambda n: torch.complex(torch.randn(n, generator=g, device="cuda", dtype=torch.float64),
                                  torch.randn(n, generator=g, device="cuda", dtype=torch.float64))
    bg.A.copy_(cre(bg.A.shape[0]))
    bg.B.copy_(cre(bg.B.shape[0]))
    A0h = bg.A.to(torch.complex128).cpu().numpy()
    B0h = bg.B.to(torch.complex128).cpu().numpy()
    bg.run()
    assert bg.status() == (0, -1)
    Ah = bg.A.to(torch.complex128).cpu().numpy()
    Bh = bg.B.to(torch.complex128).cpu().numpy()
    r_tol, x_unit = (1e-12, 1e-15) if dt == torch.complex128 else (1e-5, 1e-6)
    worst = 0.0
    for q in range(bg.nprob):
        d = bg.desc[q]
        m, n, k, ib = int(d["m"]), int(d["n"]), int(d["k"]), int(d["ib"])
        ao, bo = int(d["a_off"]), int(d["b_off"])
        Aq = A0h[ao:ao + m * n].reshape(n, m).T
        Bq = B0h[bo:bo + m * k].reshape(k, m).T
        Af, X = zoracle_solve(oracle, Aq, Bq, ib)
        Ag = Ah[ao:ao + m * n].reshape(n, m).T
        rd = np.linalg.norm(Ag - Af) / max(np.linalg.norm(Af), 1e-300)
        assert rd <= r_tol * max(n, 1), (q, m, n, k, ib, rd)
        if k > 0:
            Xg = Bh[bo:bo + m * k].reshape(k, m).T[:n]
            kappa = np.linalg.cond(Aq)
            xd = np.linalg.norm(Xg - X) / max(np.linalg.norm(X), 1e-300)
            assert xd <= max(x_unit * kappa * n, 1e3 * x_unit), (q, m, n, k, xd, kappa)
            r = Bq - Aq @ Xg
            na = np.linalg.norm(Aq)
            worst = max(worst, np.linalg.norm(Aq.conj().T @ r) / (na * (na * np.linalg.norm(Xg) + np.linalg.norm(Bq))))
    assert worst < (1e-14 if dt == torch.complex128 else 1e-5), worst
