"""ctypes front end of the CPU oracle (nextla_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
benchmark's CPU-baseline leg, never by the product library.

The functions mirror NextLA.jl's low-level signatures (geqrt!, tsqrt!,
tsmqr!, unmqr!, larfb!, larft!, geqr2!, parfb!) on column-major numpy
arrays, dispatching on the element type as the Julia methods do: float64
arrays run the FP64 routines (nextla_oracle.c), complex128 arrays the
ComplexF64 ones (nextla_oracle_z.c).  Views are allowed: the leading dimension is taken from the array's
column stride, as Julia's `stride(A, 2)` would give it.  Argument errors
raise ValueError (the reference raises ArgumentError).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "nextla_oracle.c")
_SRC_Z = os.path.join(_HERE, "nextla_oracle_z.c")     # complex elements
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

# -ffp-contract=off keeps x86 and Arm builds rounding identically (no fused
# multiply-add contraction), so the oracle gives the same bits on both hosts.
# -fopenmp parallelises only the tile driver's independent column loops.
CFLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp"]


def build(force=False):
    """Compile liboracle.so next to this file (gcc, a second or two)."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(_SRC), os.path.getmtime(_SRC_Z))):
        subprocess.check_call(["gcc", *CFLAGS, "-o", _LIB_PATH, _SRC, _SRC_Z, "-lm"])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


_I = ctypes.c_int
_C = ctypes.c_char
_P = ctypes.c_void_p


def _declare(L):
    sig = {
        "ora_dgeqr2": [_I, _I, _P, _I, _P, _P],
        "ora_dlarft": [_C, _C, _I, _I, _P, _I, _P, _P, _I],
        "ora_dlarfb": [_C, _C, _C, _C, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I],
        "ora_dgeqrt": [_I, _I, _I, _P, _I, _P, _I, _P, _P],
        "ora_dunmqr": [_C, _C, _I, _I, _I, _I, _P, _I, _I, _I, _P, _I, _P, _I, _P, _I],
        "ora_dparfb": [_C, _C, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _I],
        "ora_dtsmqr": [_C, _C, _I, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
        "ora_dtsqrt": [_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _P],
        "ora_dtile_geqrf": [_I, _I, _I, _I, _P, _I, _P, _I, _P, _I],
        "ora_dtile_unmqr": [_C, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I],
        "ora_dtrsm_lun": [_I, _I, _P, _I, _P, _I],
        "ora_dparfb_l": [_C, _C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _I],
        "ora_dttqrt": [_I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _P],
        "ora_dttmqr": [_C, _C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P],
        "ora_dtile_geqrf_tree": [_I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _P],
        "ora_dtile_unmqr_tree": [_C, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _P, _I],
        "ora_dtile_geqrf_hqr": [_I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _P],
        "ora_dpamm": [_C, _C, _C, _C, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I],
        "ora_dparfb_full": [_C, _C, _C, _C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _I, _P, _I, _P, _I],
        "ora_dtile_unmqr_hqr": [_C, _I, _I, _I, _I, _I, _I, _P, _I, _P, _I, _P, _P, _I],
        "ora_set_host_blas": [_P, _P],
        "ora_host_blas_on": [],
    }
    for name in ("geqr2", "larft", "larfb", "geqrt", "unmqr", "parfb", "parfb_l", "tsmqr", "tsqrt", "ttqrt",
                 "ttmqr", "tile_geqrf", "tile_unmqr", "trsm_lun", "pamm", "parfb_full", "tile_geqrf_hqr",
                 "tile_unmqr_hqr"):
        sig["ora_z" + name] = sig["ora_d" + name]
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _I


# ---------------------------------------------------------------------------
# Host BLAS for the oracle's products (see the note above ora_set_host_blas in
# nextla_oracle.c): NextLA's larfb! runs them through LinearAlgebra.mul!, i.e.
# the host BLAS on CPU arrays.  The Fortran-ABI dgemm/dtrmm are taken from
# scipy.linalg.cython_blas (scipy's bundled OpenBLAS, every host thread).
# ---------------------------------------------------------------------------

def _blas_pointers():
    import scipy.linalg.cython_blas as cb
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    out = []
    for name in ("dgemm", "dtrmm"):
        cap = cb.__pyx_capi__[name]
        out.append(get_ptr(cap, get_name(cap)))
    return out


def set_host_blas(on):
    """Route the oracle's GEMM/TRMM steps through the host BLAS (on=True) or
    back to its plain loops (on=False, the default).  Returns the old state."""
    L = lib()
    old = bool(L.ora_host_blas_on())
    if on:
        g, t = _blas_pointers()
        rc = L.ora_set_host_blas(ctypes.c_void_p(g), ctypes.c_void_p(t))
    else:
        rc = L.ora_set_host_blas(None, None)
    if rc != 0:
        raise RuntimeError("ora_set_host_blas failed")
    return old


class host_blas:
    """Context manager: the oracle's products run in the host BLAS inside."""

    def __enter__(self):
        self._old = set_host_blas(True)
        return self

    def __exit__(self, *exc):
        set_host_blas(self._old)
        return False


def blas_threads():
    """Threads the host BLAS uses (None when it cannot be queried)."""
    try:
        import scipy.linalg.cython_blas  # noqa: F401  (loads the BLAS)
        for name in ("scipy_openblas_get_num_threads64_", "scipy_openblas_get_num_threads",
                     "openblas_get_num_threads64_", "openblas_get_num_threads"):
            for lib_ in _loaded_blas_libs():
                f = getattr(lib_, name, None)
                if f is not None:
                    f.restype = ctypes.c_int
                    return int(f())
    except Exception:
        return None
    return None


def _loaded_blas_libs():
    out = []
    try:
        with open("/proc/self/maps") as fh:
            paths = {ln.split()[-1] for ln in fh if "openblas" in ln.lower() and ln.rstrip().endswith(".so")
                     or ("openblas" in ln.lower() and ".so" in ln)}
    except OSError:
        return out
    for pth in sorted(paths):
        if os.path.exists(pth):
            try:
                out.append(ctypes.CDLL(pth))
            except OSError:
                pass
    return out


def _mat(A):
    """(pointer, ld) of a column-major float64 or complex128 matrix or view."""
    if A is None:
        return None, 1
    if A.dtype not in (np.float64, np.complex128):
        raise TypeError("oracle works on float64 and complex128 arrays")
    es = A.dtype.itemsize
    if A.ndim == 1:
        if A.size > 1 and A.strides[0] != es:
            raise ValueError("vector must be contiguous")
        return A.ctypes.data, max(1, A.shape[0])
    if A.shape[0] > 1 and A.strides[0] != es:
        raise ValueError("matrix must be column-major (unit row stride)")
    ld = A.strides[1] // es if A.shape[1] > 1 else A.shape[0]
    return A.ctypes.data, max(1, ld)


def _fn(name, *arrays):
    """The oracle routine for the arrays' element type: ora_d<name> for
    float64, ora_z<name> for complex128 (all arrays must agree)."""
    kinds = {a.dtype for a in arrays if a is not None}
    if len(kinds) != 1:
        raise TypeError(f"{name}: arrays must share one element type, got {kinds}")
    return getattr(lib(), ("ora_z" if kinds.pop() == np.complex128 else "ora_d") + name)


def _ch(c):
    return c.encode() if isinstance(c, str) else c


def _check(info, name):
    if info < 0:
        raise ValueError(f"{name}: illegal value of argument {-info}")
    return info


def fmat(shape, rng=None, kind="uniform01"):
    """Column-major float64 matrix helper used by tests."""
    if rng is None:
        return np.zeros(shape, dtype=np.float64, order="F")
    if kind == "uniform01":
        return np.asfortranarray(rng.random(shape))
    if kind == "uniform11":
        return np.asfortranarray(rng.uniform(-1.0, 1.0, shape))
    return np.asfortranarray(rng.standard_normal(shape))


# ---- NextLA mirrors ---------------------------------------------------------

def geqr2(m, n, A, tau, work):
    pa, lda = _mat(A)
    return _check(_fn("geqr2", A, tau, work)(m, n, pa, lda, _mat(tau)[0], _mat(work)[0]), "geqr2")


def larft(direct, storev, n, k, V, tau, T):
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    return _check(_fn("larft", V, tau, T)(_ch(direct), _ch(storev), n, k, pv, ldv,
                                   _mat(tau)[0], pt, ldt), "larft")


def larfb(side, trans, direct, storev, m, n, k, V, ldv, T, C, work):
    pv, _ = _mat(V)
    pt, ldt = _mat(T)
    pc, ldc = _mat(C)
    pw, ldw = _mat(work)
    return _check(_fn("larfb", V, T, C, work)(_ch(side), _ch(trans), _ch(direct), _ch(storev), m, n, k,
                                   pv, ldv, pt, ldt, pc, ldc, pw, ldw), "larfb")


def geqrt(m, n, ib, A, T, tau, work):
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    return _check(_fn("geqrt", A, T, tau, work)(m, n, ib, pa, lda, pt, ldt, _mat(tau)[0],
                                   _mat(work)[0]), "geqrt")


def unmqr(side, trans, m, n, k, ib, A, lda, T, C, work):
    pa, _ = _mat(A)
    pt, ldt = _mat(T)
    pc, ldc = _mat(C)
    pw, ldw = _mat(work)
    return _check(_fn("unmqr", A, T, C, work)(_ch(side), _ch(trans), m, n, k, ib, pa, lda,
                                   A.shape[0], A.shape[1], pt, ldt, pc, ldc, pw, ldw), "unmqr")


def parfb(side, trans, m1, n1, m2, n2, k, A1, A2, V, T, work):
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    pw, ldw = _mat(work)
    return _check(_fn("parfb", A1, A2, V, T, work)(_ch(side), _ch(trans), m1, n1, m2, n2, k, p1, ld1, p2, ld2,
                                   pv, ldv, pt, ldt, pw, ldw), "parfb")


def tsmqr(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work):
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    kstored = min(V.shape[1], T.shape[1])
    return _check(_fn("tsmqr", A1, A2, V, T, work)(_ch(side), _ch(trans), m1, n1, m2, n2, k, ib, kstored,
                                   p1, ld1, p2, ld2, pv, ldv, pt, ldt, _mat(work)[0]), "tsmqr")


def tsqrt(m, n, ib, A1, A2, T, tau, work):
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pt, ldt = _mat(T)
    return _check(_fn("tsqrt", A1, A2, T, tau, work)(m, n, ib, A1.shape[0], p1, ld1, p2, ld2, pt, ldt,
                                   _mat(tau)[0], _mat(work)[0]), "tsqrt")


def tile_geqrf(A, nb, ib):
    """Flat-tree tile QR of A in place; returns (T, tau) in the tile layouts."""
    m, n = A.shape
    MT = (m + nb - 1) // nb
    T = np.zeros((MT * ib, n), order="F", dtype=A.dtype)
    tau = np.zeros((n, MT), order="F", dtype=A.dtype)
    pa, lda = _mat(A)
    _check(_fn("tile_geqrf", A, T, tau)(m, n, nb, ib, pa, lda, T.ctypes.data, MT * ib,
                                 tau.ctypes.data, n), "tile_geqrf")
    return T, tau


def tile_unmqr(trans, A, T, B, nb, ib):
    m, n = A.shape
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    pb, ldb = _mat(B)
    return _check(_fn("tile_unmqr", A, T, B)(_ch(trans), m, n, B.shape[1], nb, ib, pa, lda, pt, ldt,
                                        pb, ldb), "tile_unmqr")


def trsm_lun(R, B):
    pr, ldr = _mat(R)
    pb, ldb = _mat(B)
    return _check(_fn("trsm_lun", R, B)(R.shape[1], B.shape[1], pr, ldr, pb, ldb), "trsm")


def parfb_l(side, trans, m1, n1, m2, n2, k, l, A1, A2, V, T, work):
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    pw, ldw = _mat(work)
    return _check(_fn("parfb_l", A1, A2, V, T, work)(_ch(side), _ch(trans), m1, n1, m2, n2, k, l, p1, ld1, p2, ld2,
                                     pv, ldv, pt, ldt, pw, ldw), "parfb")


def ttqrt(m, n, ib, A1, A2, T, tau, work):
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pt, ldt = _mat(T)
    return _check(_fn("ttqrt", A1, A2, T, tau, work)(m, n, ib, p1, ld1, p2, ld2, pt, ldt, _mat(tau)[0],
                                   _mat(work)[0]), "ttqrt")


def ttmqr(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work):
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    return _check(_fn("ttmqr", A1, A2, V, T, work)(_ch(side), _ch(trans), m1, n1, m2, n2, k, ib, p1, ld1, p2, ld2,
                                   pv, ldv, pt, ldt, _mat(work)[0]), "ttmqr")


def tile_geqrf_tree(A, nb, ib):
    """Tile QR with a binary reduction tree per panel, in place; returns
    (T, tau, T2, tau2): geqrt's factors of every tile and the ttqrt ones."""
    m, n = A.shape
    MT = (m + nb - 1) // nb
    T = np.zeros((MT * ib, n), order="F")
    T2 = np.zeros((MT * ib, n), order="F")
    tau = np.zeros((n, MT), order="F")
    tau2 = np.zeros((n, MT), order="F")
    pa, lda = _mat(A)
    _check(lib().ora_dtile_geqrf_tree(m, n, nb, ib, pa, lda, T.ctypes.data, MT * ib, tau.ctypes.data, n,
                                      T2.ctypes.data, tau2.ctypes.data), "tile_geqrf_tree")
    return T, tau, T2, tau2


def pamm(op, side, storev, direct, m, n, k, l, A1, A2, V, W):
    """pamm!(op, side, storev, direct, m, n, k, l, A1, A2, V, W) -- src/pamm.jl:49."""
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pw, ldw = _mat(W)
    return _check(_fn("pamm", A1, A2, V, W)(_ch(op), _ch(side), _ch(storev), _ch(direct), m, n, k, l, p1, ld1,
                                            p2, ld2, pv, ldv, pw, ldw), "pamm")


def parfb_full(side, trans, direct, storev, m1, n1, m2, n2, k, l, A1, A2, V, T, W):
    """parfb! in every direct / storev form (src/parfb.jl:44-191); W is work
    (k x n2 for side 'L', m2 x k for 'R')."""
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    pw, ldw = _mat(W)
    return _check(_fn("parfb_full", A1, A2, V, T, W)(_ch(side), _ch(trans), _ch(direct), _ch(storev), m1, n1, m2,
                                                      n2, k, l, p1, ld1, p2, ld2, pv, ldv, pt, ldt, pw, ldw),
                  "parfb")


def tile_geqrf_hqr(A, nb, ib, grp):
    """Hierarchical tile QR in place: groups of grp tiles reduced flat into
    their first tile, the group leaders by the binary tree.  Returns
    (T, tau, T2, tau2) as tile_geqrf_tree does."""
    m, n = A.shape
    MT = (m + nb - 1) // nb
    T = np.zeros((MT * ib, n), order="F", dtype=A.dtype)
    T2 = np.zeros((MT * ib, n), order="F", dtype=A.dtype)
    tau = np.zeros((n, MT), order="F", dtype=A.dtype)
    tau2 = np.zeros((n, MT), order="F", dtype=A.dtype)
    pa, lda = _mat(A)
    _check(_fn("tile_geqrf_hqr", A, T, tau, T2, tau2)(m, n, nb, ib, grp, pa, lda, T.ctypes.data, MT * ib,
                                                      tau.ctypes.data, n, T2.ctypes.data, tau2.ctypes.data),
           "tile_geqrf_hqr")
    return T, tau, T2, tau2


def tile_unmqr_hqr(trans, A, T, T2, B, nb, ib, grp):
    m, n = A.shape
    pa, lda = _mat(A)
    pb, ldb = _mat(B)
    return _check(_fn("tile_unmqr_hqr", A, T, T2, B)(_ch(trans), m, n, B.shape[1], nb, ib, grp, pa, lda,
                                                     T.ctypes.data, T.shape[0], T2.ctypes.data, pb, ldb),
                  "tile_unmqr_hqr")


def tile_unmqr_tree(trans, A, T, T2, B, nb, ib):
    m, n = A.shape
    pa, lda = _mat(A)
    pb, ldb = _mat(B)
    return _check(lib().ora_dtile_unmqr_tree(_ch(trans), m, n, B.shape[1], nb, ib, pa, lda, T.ctypes.data,
                                             T.shape[0], T2.ctypes.data, pb, ldb), "tile_unmqr_tree")


def tile_lstsq(A, B, nb, ib):
    """min ||A X - B|| by tile QR: returns X (n-by-nrhs); A and B are copied."""
    dt = np.complex128 if np.iscomplexobj(A) or np.iscomplexobj(B) else np.float64
    A = np.array(A, order="F", dtype=dt)
    B = np.array(B, order="F", dtype=dt)
    n = A.shape[1]
    T, _ = tile_geqrf(A, nb, ib)
    tile_unmqr("C", A, T, B, nb, ib)
    X = np.array(B[:n], order="F")
    trsm_lun(A[:n, :n], X)
    return X


# ---------------------------------------------------------------------------
# Differentiable QR: FP64 CPU reference of the forward (explicit thin Q) and of
# the adjoint.  The forward is the same flat-tree tile QR as above (one tile
# column when n <= nb), so Q and R carry the same diagonal signs as the GPU's.
# ---------------------------------------------------------------------------

def qr_explicit(A, nb=256, ib=32):
    """(Q, R, F): thin Q (m-by-n), R (n-by-n upper) and the packed factor
    (float64, or complex128 for complex input)."""
    dt = np.complex128 if np.iscomplexobj(A) else np.float64
    F = np.array(A, order="F", dtype=dt)
    m, n = F.shape
    T, _ = tile_geqrf(F, nb, ib)
    Q = np.asfortranarray(np.eye(m, n, dtype=dt))
    tile_unmqr("N", F, T, Q, nb, ib)
    R = np.triu(F[:n, :n])
    return Q, R, F


def qr_adjoint(Q, R, Qbar, Rbar):
    """Thin-QR pullback (Walter & Lehmann 2018, Algorithms for the QR
    adjoint; Liao, Liu, Wang & Xiang 2019): M = R Rbar^T - Qbar^T Q,
    Abar = (Qbar + Q copyltu(M)) R^-T, copyltu(M) = tril(M) + tril(M, -1)^T.
    Only the upper triangle of Rbar enters (R has no other entries)."""
    from scipy.linalg import solve_triangular
    if np.iscomplexobj(Q) or np.iscomplexobj(Qbar) or np.iscomplexobj(Rbar):
        # complex, R's diagonal real: Abar = (Qbar + Q X) R^-H with
        # X = tril(M,-1) + tril(M,-1)^H + Re diag(M), M = R Rbar^H - Qbar^H Q
        # (the gradient of a real loss as dL/dRe + i dL/dIm); needs m > n so
        # that every column has a reflector (src/geqr2.jl:32-35 leaves a
        # one-row last column with tau = 0 and a complex R_nn)
        if Q.shape[0] <= Q.shape[1]:
            raise ValueError("complex QR adjoint needs m > n")
        M = R @ np.triu(Rbar).conj().T - Qbar.conj().T @ Q
        C = np.tril(M, -1) + np.tril(M, -1).conj().T + np.diag(M.diagonal().real)
        Y = Qbar + Q @ C
        return solve_triangular(R, Y.conj().T, lower=False).conj().T      # Y R^-H = (R^-1 Y^H)^H
    M = R @ np.triu(Rbar).T - Qbar.T @ Q
    C = np.tril(M) + np.tril(M, -1).T
    Y = Qbar + Q @ C
    return solve_triangular(R, Y.T, lower=False).T


def ls_loss_cotangents(Q, R, b, y, dQ, dR):
    """Value and (Qbar, Rbar) of f = 1/2 ||R^-1 Q^T b - y||^2 + <dQ, Q> + <dR, R>
    for one problem (b: m, y: n)."""
    from scipy.linalg import solve_triangular
    c = Q.T @ b
    x = solve_triangular(R, c, lower=False)
    r = x - y
    f = 0.5 * float(r @ r) + float(np.sum(dQ * Q)) + float(np.sum(dR * np.triu(R)))
    cbar = solve_triangular(R, r, lower=False, trans="T")
    Qbar = dQ + np.outer(b, cbar)
    Rbar = np.triu(dR) - np.triu(np.outer(cbar, x))
    return f, Qbar, Rbar
