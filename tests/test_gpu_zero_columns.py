"""Zero columns through the FP64 tile-QR drivers: the no-reflector paths of
the panel column loop (geqr2!'s tau = 0 with R_ii = alpha, src/geqr2.jl:48-73;
tsqrt!'s skipped column that keeps its T column, src/tsqrt.jl:61-64; the same
for ttqrt!) inside the flat-tree stream driver, the flat-tree persistent
kernel and the tree / hierarchical drivers, against the oracle's drivers on
the same matrix at the FP64 bar (1e-12 n relative, max-normalised)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def zero_column_matrix(m, n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((m, n))
    A[:, 5] = 0.0          # every tile of column 5: no reflector anywhere
    A[256:, 0] = 0.0       # column 0 below the first tile row: the merges skip it
    return np.asfortranarray(A)


@pytest.mark.parametrize("dag", [False, True])
def test_flat_tree_zero_columns(tq, oracle, dag):
    m, n, nb, ib = 1024, 768, 256, 32
    A0 = zero_column_matrix(m, n, 21)
    A = tq.to_device(A0)
    T, tau = tq.tile_geqrf(A, nb, ib, dag=dag)
    Ao = A0.copy(order="F")
    To, tauo = oracle.tile_geqrf(Ao, nb, ib)
    for x, y in ((A, Ao), (T, To), (tau, tauo)):
        assert rel(tq.to_numpy(x), y) < 1e-12 * n
    taug = tq.to_numpy(tau)
    assert taug[5, 0] == 0.0 and np.all(taug[0, 1:] == 0.0)   # geqrt!'s and the merges' skipped reflectors


@pytest.mark.parametrize("grp,dag", [(1, False), (1, True), (2, True)])
def test_tree_zero_columns(tq, oracle, grp, dag):
    m, n, nb, ib = 1024, 512, 256, 32
    A0 = zero_column_matrix(m, n, 22 + grp)
    A = tq.to_device(A0)
    T, tau, T2, tau2 = tq.tile_geqrf_tree(A, nb, ib, dag=dag, grp=grp)
    Ao = A0.copy(order="F")
    ref = oracle.tile_geqrf_hqr(Ao, nb, ib, grp)
    for x, y in zip((A, T, tau, T2, tau2), (Ao,) + tuple(ref)):
        assert rel(tq.to_numpy(x), y) < 1e-12 * n
    assert np.all(tq.to_numpy(tau)[5, :] == 0.0)
