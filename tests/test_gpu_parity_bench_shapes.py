"""Parity with the oracle at the benchmark shapes themselves.

The benchmark quotes the FP64 tile QR of an 8192 x 8192 matrix and of a
65536 x 512 one (nb 256, ib 32), and the FP64 least-squares solve of the
32768 x 4096 mixed-precision configuration.  Here the GPU results on those
exact shapes are compared with the oracle's on the same seeded inputs.  The
oracle runs its products in the host BLAS (oracle.host_blas(); NextLA's
larfb! does the same through mul!), which brings the 8192^2 factorisation to
seconds on the host cores; tests/test_oracle_host_blas.py pins that form to
the LAPACK golden vectors and to the plain-loop oracle.

Bars:
* the parity bar "relative differences in R and Q <= 1e-12 n", applied per
  tile: every nb x nb tile of R, V and explicit Q, every ib x nb block of T
  and every panel's tau, relative to that tile's own Frobenius norm, so a
  wrong small-magnitude block cannot hide behind the large ones;
* the reference's elementwise check of R's diagonal (test/tsqrt.jl:44-48):
  | |R_jj| - |R_jj,ref| | < 100 rtol max(|R_jj|, |R_jj,ref|), rtol = 1e-12;
* the reference's normwise `isapprox(..., rtol=1e-12)` of the outputs
  (test/tsqrt.jl:33-34, test/tsmqr.jl:37-38) on the whole of R and V; for the
  least-squares matrix (condition number 1e6) V's bar is 10 kappa eps, the
  distance two backward-stable factorisations' reflectors may have.
The worst per-tile figure of each run is printed for the record.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NB, IB = 256, 32
RTOL = 1e-12


def F(a):
    return np.array(a, dtype=np.float64, order="F")


def tilewise(a, b, rb, cb):
    """max over rb x cb tiles of ||a - b||_F / ||b||_F (tiles where b is zero
    must match exactly); also returns the tile that reached it."""
    m, n = b.shape
    worst, where = 0.0, None
    for i in range(0, m, rb):
        for j in range(0, n, cb):
            bt = b[i:i + rb, j:j + cb]
            d = np.linalg.norm(a[i:i + rb, j:j + cb] - bt)
            nb_ = np.linalg.norm(bt)
            r = d / nb_ if nb_ > 0 else (0.0 if d == 0 else np.inf)
            if r > worst:
                worst, where = r, (i // rb, j // cb)
    return worst, where


def split_rv(A, k):
    """R (upper triangle of the first k rows) and V (everything below it)."""
    R = np.triu(A[:k])
    V = A.copy()
    V[:k] -= R
    return R, V


def check_factor(tag, m, n, Ag, Tg, taug, Ao, To, tauo, extra=(), kappa=1.0):
    """kappa: condition number of A.  R's normwise agreement does not depend
    on it; V (the reflectors) moves by O(kappa eps) between two backward-
    stable factorisations, so V's normwise bar is the reference's 1e-12 for
    the well-conditioned Gaussian matrices and 10 kappa eps beyond that."""
    k = min(m, n)
    tol = RTOL * max(m, n)
    Rg, Vg = split_rv(Ag, k)
    Ro, Vo = split_rv(Ao, k)
    report = {}
    for name, a, b, rb, cb in (("R", Rg, Ro, NB, NB), ("V", Vg, Vo, NB, NB), ("T", Tg, To, IB, NB),
                               ("tau", taug, tauo, NB, 1)) + tuple(extra):
        w, where = tilewise(a, b, rb, cb)
        report[name] = (w, where)
        assert w <= tol, f"{tag}: {name} tile {where} differs by {w:.3e} > {tol:.1e}"
    # the reference's elementwise diagonal check and normwise isapprox
    dg, do = np.abs(np.diag(Rg)), np.abs(np.diag(Ro))
    big = do > RTOL * 10
    diag = float(np.max(np.abs(dg - do)[big] / np.maximum(dg, do)[big]))
    assert diag < 100 * RTOL, f"{tag}: diagonal of R differs elementwise by {diag:.3e}"
    for name, a, b, bar in (("R", Rg, Ro, RTOL), ("V", Vg, Vo, max(RTOL, 10 * kappa * 2.0 ** -52))):
        nr = np.linalg.norm(a - b) / max(np.linalg.norm(a), np.linalg.norm(b))
        report[name + "_normwise"] = (nr, None)
        assert nr <= bar, f"{tag}: {name} normwise {nr:.3e} > {bar:.1e}"
    print(f"\n{tag}: worst tile " + ", ".join(f"{k_} {v[0]:.2e}" for k_, v in report.items()) +
          f"; diag(R) elementwise {diag:.2e}")
    return report


def explicit_q(apply, m, n, dev_tq=None):
    """Q[:, :n] formed by applying Q to [I; 0]."""
    Q = np.zeros((m, n), order="F")
    Q[np.arange(n), np.arange(n)] = 1.0
    if dev_tq is None:
        apply(Q)
        return Q
    Qd = dev_tq.to_device(Q)
    apply(Qd)
    return dev_tq.to_numpy(Qd)


@pytest.fixture(scope="module")
def host_blas(oracle):
    pytest.importorskip("scipy")
    with oracle.host_blas():
        yield oracle


def test_square_8192_flat_tree(tq, host_blas):
    """The headline workload: 8192^2 N(0,1) FP64, persistent kernel, vs the oracle;
    then explicit Q on both sides."""
    oracle = host_blas
    m = n = 8192
    rng = np.random.default_rng(20241203)
    A0 = F(rng.standard_normal((m, n)))
    A = tq.to_device(A0)
    T, tau = tq.tile_geqrf(A, NB, IB, dag=True)
    Ao = A0.copy(order="F")
    del A0
    To, tauo = oracle.tile_geqrf(Ao, NB, IB)
    Ag = tq.to_numpy(A)
    check_factor("8192^2", m, n, Ag, tq.to_numpy(T), tq.to_numpy(tau), Ao, To, tauo)
    del Ag
    Qg = explicit_q(lambda Q: tq.tile_unmqr("N", A, T, Q, NB, IB), m, n, tq)
    Qo = explicit_q(lambda Q: oracle.tile_unmqr("N", Ao, To, Q, NB, IB), m, n)
    w, where = tilewise(Qg, Qo, NB, NB)
    print(f"8192^2: explicit Q worst tile {w:.2e} at {where}")
    assert w <= RTOL * n, f"Q tile {where}: {w:.3e}"


def test_tall_skinny_65536x512_flat_and_hierarchical(tq, host_blas):
    """The tall-skinny workload, flat tree (persistent kernel) and the
    hierarchical tree with groups of 4 tiles (its task graph), each vs the
    oracle's driver of the same shape of tree, explicit Q included."""
    oracle = host_blas
    m, n = 65536, 512
    rng = np.random.default_rng(65536 + 512)
    A0 = F(rng.standard_normal((m, n)))
    # flat tree
    A = tq.to_device(A0)
    T, tau = tq.tile_geqrf(A, NB, IB, dag=True)
    Ao = A0.copy(order="F")
    To, tauo = oracle.tile_geqrf(Ao, NB, IB)
    check_factor("65536x512 flat", m, n, tq.to_numpy(A), tq.to_numpy(T), tq.to_numpy(tau), Ao, To, tauo)
    Qg = explicit_q(lambda Q: tq.tile_unmqr("N", A, T, Q, NB, IB), m, n, tq)
    Qo = explicit_q(lambda Q: oracle.tile_unmqr("N", Ao, To, Q, NB, IB), m, n)
    w, where = tilewise(Qg, Qo, NB, NB)
    print(f"65536x512 flat: explicit Q worst tile {w:.2e} at {where}")
    assert w <= RTOL * m
    # hierarchical, groups of 4 (the benchmark's tall-skinny form)
    grp = 4
    A = tq.to_device(A0)
    T, tau, T2, tau2 = tq.tile_geqrf_tree(A, NB, IB, dag=True, grp=grp)
    Ao = A0.copy(order="F")
    To, tauo, T2o, tau2o = oracle.tile_geqrf_hqr(Ao, NB, IB, grp)
    check_factor("65536x512 hqr4", m, n, tq.to_numpy(A), tq.to_numpy(T), tq.to_numpy(tau), Ao, To, tauo,
                 extra=(("T2", tq.to_numpy(T2), T2o, IB, NB), ("tau2", tq.to_numpy(tau2), tau2o, NB, 1)))
    Qg = explicit_q(lambda Q: tq.tile_unmqr_tree("N", A, T, T2, Q, NB, IB, grp=grp), m, n, tq)
    Qo = explicit_q(lambda Q: oracle.tile_unmqr_hqr("N", Ao, To, T2o, Q, NB, IB, grp), m, n)
    w, where = tilewise(Qg, Qo, NB, NB)
    print(f"65536x512 hqr4: explicit Q worst tile {w:.2e} at {where}")
    assert w <= RTOL * m


def test_least_squares_32768x4096_fp64_solve(tq, host_blas):
    """The FP64 solve of the mixed-precision configuration (Float32-stored
    A = U diag(sigma) V^T, sigma 1..1e-6, b = A x + 1e-10 noise, 4 RHS): the
    persistent kernel with B folded in as an extra tile column, then R X =
    Q^T B, against the oracle's tile QR, Q^T B and LeftUpperTRSM!."""
    import os
    import sys

    import torch
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    oracle = host_blas
    m, n, k = 32768, 4096, 4
    A32, b = bench.ls_problem(m, n, k, torch)
    A0 = F(A32.double().cpu().numpy())
    B0 = F(b.cpu().numpy())
    del A32, b
    A = tq.to_device(A0)
    B = tq.to_device(B0)
    ts, taus = tq.tile_shapes(m, n, NB, IB)
    # the benchmark's FP64 solve (tqr_dtile_gels_dag), with its T and tau kept
    import ctypes
    from tileqr import _lib
    T, tau = tq.zeros(*ts), tq.zeros(*taus)
    size = ctypes.c_size_t(0)
    assert _lib.lib().tqr_tile_gels_worksize(m, n, k, NB, IB, ctypes.byref(size)) == 0
    w = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
    wp = w.data_ptr() + ((-w.data_ptr()) % 256)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    st = torch.cuda.current_stream()
    rc = _lib.lib().tqr_dtile_gels_dag(m, n, k, NB, IB, P(A), m, P(T), ts[0], P(tau), taus[0], P(B), m,
                                       ctypes.c_void_p(wp), size.value, ctypes.c_void_p(st.cuda_stream))
    assert rc == 0
    st.synchronize()
    assert tq.dag_status(wp)[0] == 0
    Ao = A0.copy(order="F")
    To, tauo = oracle.tile_geqrf(Ao, NB, IB)
    Bo = B0.copy(order="F")
    oracle.tile_unmqr("C", Ao, To, Bo, NB, IB)
    QtB_o = Bo.copy(order="F")
    Xo = F(Bo[:n])
    oracle.trsm_lun(Ao[:n, :n], Xo)
    Bg = tq.to_numpy(B)
    check_factor("32768x4096 gels", m, n, tq.to_numpy(A), tq.to_numpy(T), tq.to_numpy(tau), Ao, To, tauo,
                 kappa=1e6)
    # Q^T B below row n is untouched by the solve: the residual part, of the
    # noise's size (1e-10 N(0,1)), so each tile's difference is measured
    # against ||B|| (the scale its rounding errors come from); R X = Q^T B's
    # top part through X (kappa = 1e6 bounds X's agreement)
    nB = np.linalg.norm(B0)
    w_q, where = 0.0, None
    for i in range(n, m, NB):
        d = np.linalg.norm(Bg[i:i + NB] - QtB_o[i:i + NB]) / nB
        if d > w_q:
            w_q, where = d, i // NB
    assert w_q <= RTOL * m, f"Q^T B tile {where}: {w_q:.3e} of ||B||"
    xr = np.linalg.norm(Bg[:n] - Xo) / np.linalg.norm(Xo)
    print(f"32768x4096 gels: Q^T B worst tile {w_q:.2e} of ||B||, X relative {xr:.2e}")
    assert xr <= 1e6 * RTOL * n ** 0.5
