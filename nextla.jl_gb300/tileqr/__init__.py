"""tileqr -- Python front end of libtileqr.so, mirroring NextLA.jl's tile-QR API.

Function names and argument lists follow NextLA's in-place kernels
(`geqrt!`, `tsqrt!`, `tsmqr!`, `unmqr!`, `larfb!`, `larft!`, `geqr2!`,
`parfb!`) and their allocating helper methods, dispatched on the number of
arguments the way Julia dispatches on the method signature.  Arrays are
column-major CUDA tensors -- float64, float32, complex128 (ComplexF64) or
complex64 (ComplexF32), the element types the reference tests; the complex
types cover the tile kernels and the flat tile QR -- built with `empty`,
`zeros` or `to_device`, and pass slices of them as NextLA passes `@view`s; the
leading dimension is read from the column stride.

Errors: an illegal argument raises ArgumentError (a ValueError), mirroring the
reference's ArgumentError; a CUDA failure raises RuntimeError.  Calls are
blocking by default, like the reference (every NextLA kernel synchronises);
`set_blocking(False)` leaves them asynchronous on torch's current stream.
"""
import torch

from . import _lib

__all__ = [
    "ArgumentError", "set_blocking", "empty", "zeros", "to_device", "to_numpy",
    "geqr2", "larft", "larfb", "geqrt", "unmqr", "tsqrt", "tsmqr", "parfb", "pamm", "ttqrt", "ttmqr",
    "tile_geqrf", "tile_unmqr", "trsm_lun", "tile_gels", "tile_shapes",
    "autotune_tiling", "tile_geqrf_tuned",
]

_BLOCKING = True


class ArgumentError(ValueError):
    """Raised where NextLA.jl raises ArgumentError."""


def set_blocking(flag):
    global _BLOCKING
    _BLOCKING = bool(flag)


# ---- column-major tensors ---------------------------------------------------

def empty(m, n, dtype=torch.float64, device="cuda"):
    """m-by-n column-major tensor (stride (1, m))."""
    return torch.empty((n, m), dtype=dtype, device=device).t()


def zeros(m, n, dtype=torch.float64, device="cuda"):
    return torch.zeros((n, m), dtype=dtype, device=device).t()


def to_device(x, dtype=None, device="cuda"):
    """Copy a numpy array or tensor into a column-major CUDA tensor."""
    t = torch.as_tensor(x)
    if dtype is not None:
        t = t.to(dtype)
    if t.dim() == 1:
        return t.to(device).contiguous()
    out = empty(t.shape[0], t.shape[1], dtype=t.dtype, device=device)
    out.copy_(t)
    return out


def to_numpy(t):
    import numpy as np
    return np.asfortranarray(t.detach().cpu().numpy())


# ---- plumbing ----------------------------------------------------------------

def _prefix(*ts):
    dt = None
    for t in ts:
        if t is None:
            continue
        if dt is None:
            dt = t.dtype
        elif t.dtype != dt:
            raise TypeError("all arrays must share one element type")
    if dt == torch.float64:
        return "d"
    if dt == torch.float32:
        return "s"
    if dt == torch.complex128:
        return "z"
    if dt == torch.complex64:
        return "c"
    raise TypeError(f"unsupported element type {dt}")


def _mat(t):
    """(device pointer, leading dimension) of a column-major matrix or view."""
    if t is None:
        return None, 1
    if not t.is_cuda:
        raise TypeError("tileqr works on CUDA tensors")
    if t.dim() == 1:
        if t.numel() > 1 and t.stride(0) != 1:
            raise ArgumentError("vectors must be contiguous")
        return t.data_ptr(), max(1, t.shape[0])
    if t.dim() != 2:
        raise ArgumentError("expected a matrix")
    m, n = t.shape
    if m > 1 and t.stride(0) != 1:
        raise ArgumentError("matrices must be column-major (unit row stride)")
    ld = t.stride(1) if n > 1 else m
    return t.data_ptr(), max(1, ld)


def _ptr(t):
    return _mat(t)[0]


def _ch(c):
    if isinstance(c, bytes):
        return c
    return str(c).encode()


def _call(prefix, name, *args):
    st = torch.cuda.current_stream()
    rc = _lib.fn(prefix, name)(*args, st.cuda_stream)
    if rc < 0:
        raise ArgumentError(f"{name}!: illegal value of argument {-rc}")
    if rc > 0:
        raise RuntimeError(f"{name}!: CUDA error {rc}")
    if _BLOCKING:
        st.synchronize()


def _arity(name, args, *counts):
    if len(args) not in counts:
        raise TypeError(f"{name}: no method with {len(args)} arguments")


# ---- NextLA kernels ---------------------------------------------------------

def geqr2(*args):
    """geqr2!(m, n, A, tau, work) | geqr2!(A, tau) -- src/geqr2.jl:107-140."""
    _arity("geqr2", args, 5, 2)
    if len(args) == 2:
        A, tau = args
        m, n = A.shape
        return geqr2(m, n, A, tau, None)
    m, n, A, tau, work = args
    pa, lda = _mat(A)
    _call(_prefix(A, tau), "geqr2", m, n, pa, lda, _ptr(tau), None)


def larft(*args):
    """larft!(direct, storev, n, k, V, tau, T) | larft!(direct, storev, V, tau, T)
    -- src/larft.jl:205-272."""
    _arity("larft", args, 7, 5)
    if len(args) == 5:
        direct, storev, V, tau, T = args
        if _ch(storev) == b"C":
            n, k = V.shape
            if tau.shape[0] != k:
                raise ArgumentError("For columnwise storage, length(tau) must equal size(V,2)")
        else:
            k, n = V.shape
            if tau.shape[0] != k:
                raise ArgumentError("For rowwise storage, length(tau) must equal size(V,1)")
        return larft(direct, storev, n, k, V, tau, T)
    direct, storev, n, k, V, tau, T = args
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    _call(_prefix(V, tau, T), "larft", _ch(direct), _ch(storev), n, k, pv, ldv, _ptr(tau), pt, ldt)


def larfb(*args):
    """larfb!(side, trans, direct, storev, m, n, k, V, ldv, T, C, work)
    | larfb!(side, trans, direct, storev, V, T, C) -- src/larfb.jl:37-210."""
    _arity("larfb", args, 12, 7)
    if len(args) == 7:
        side, trans, direct, storev, V, T, C = args
        m, n = C.shape
        k = T.shape[0]
        return larfb(side, trans, direct, storev, m, n, k, V, V.shape[0], T, C, None)
    side, trans, direct, storev, m, n, k, V, ldv, T, C, work = args
    pv, _ = _mat(V)
    pt, ldt = _mat(T)
    pc, ldc = _mat(C)
    _call(_prefix(V, T, C), "larfb", _ch(side), _ch(trans), _ch(direct), _ch(storev), m, n, k,
          pv, ldv, pt, ldt, pc, ldc, None, 1)


def geqrt(*args):
    """geqrt!(m, n, ib, A, T, tau, work) | geqrt!(A, T) -- src/geqrt.jl:22-91.
    The helper returns (A, T, tau)."""
    _arity("geqrt", args, 7, 2)
    if len(args) == 2:
        A, T = args
        m, n = A.shape
        ib = T.shape[0]
        tau = torch.zeros(min(m, n), dtype=A.dtype, device=A.device)
        geqrt(m, n, ib, A, T, tau, None)
        return A, T, tau
    m, n, ib, A, T, tau, work = args
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    _call(_prefix(A, T, tau), "geqrt", m, n, ib, pa, lda, pt, ldt, _ptr(tau), None)


def unmqr(*args):
    """unmqr!(side, trans, m, n, k, ib, A, lda, T, C, work)
    | unmqr!(side, trans, A, T, C) -- src/unmqr.jl:52-237."""
    _arity("unmqr", args, 11, 5)
    if len(args) == 5:
        side, trans, A, T, C = args
        m, n = C.shape
        ib, k = T.shape
        nq = m if _ch(side) == b"L" else n
        k = min(k, nq)
        if ib <= 0:
            raise ArgumentError(f"Block size ib must be positive, got {ib}")
        if A.shape[0] != nq:
            raise ArgumentError("A_qr rows must match the order of Q")
        if A.shape[1] < k:
            raise ArgumentError(f"A_qr columns ({A.shape[1]}) must be >= k ({k})")
        lda = max(1, _mat(A)[1])
        return unmqr(side, trans, m, n, k, ib, A, lda, T, C, None)
    side, trans, m, n, k, ib, A, lda, T, C, work = args
    if k >= 0:
        k = min(k, A.shape[1])                 # src/unmqr.jl:83 (size(A, 2))
    pa, _ = _mat(A)
    pt, ldt = _mat(T)
    pc, ldc = _mat(C)
    _call(_prefix(A, T, C), "unmqr", _ch(side), _ch(trans), m, n, k, ib, pa, lda, pt, ldt,
          pc, ldc, None, 1)


def tsqrt(*args):
    """tsqrt!(m, n, ib, A1, A2, T, tau, work) | tsqrt!(A1, A2, T) -- src/tsqrt.jl:128-211.
    The helper returns (A1, A2, T, tau)."""
    _arity("tsqrt", args, 8, 3)
    if len(args) == 3:
        A1, A2, T = args
        m1, n = A1.shape
        m = A2.shape[0]
        ib = T.shape[0]
        if ib <= 0:
            raise ArgumentError(f"Block size ib must be positive, got {ib}")
        tau = torch.zeros(min(m1, n), dtype=A1.dtype, device=A1.device)
        tsqrt(m, n, ib, A1, A2, T, tau, None)
        return A1, A2, T, tau
    m, n, ib, A1, A2, T, tau, work = args
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pt, ldt = _mat(T)
    _call(_prefix(A1, A2, T, tau), "tsqrt", m, n, ib, A1.shape[0], p1, ld1, p2, ld2, pt, ldt,
          _ptr(tau), None)


def tsmqr(*args):
    """tsmqr!(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work)
    | tsmqr!(side, trans, A1, A2, V, T) -- src/tsmqr.jl:47-228."""
    _arity("tsmqr", args, 13, 6)
    if len(args) == 6:
        side, trans, A1, A2, V, T = args
        m1, n1 = A1.shape
        m2, n2 = A2.shape
        ib, k = T.shape
        if _ch(side) == b"L" and n2 != n1:
            raise ArgumentError("For side='L', A1 and A2 must have same number of columns")
        if _ch(side) == b"R" and m2 != m1:
            raise ArgumentError("For side='R', A1 and A2 must have same number of rows")
        if ib <= 0:
            raise ArgumentError(f"Block size ib must be positive, got {ib}")
        return tsmqr(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, None)
    side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work = args
    if k >= 0 and V is not None and T is not None:
        k = min(k, V.shape[1], T.shape[1])     # src/tsmqr.jl:94-96 (stored columns)
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    _call(_prefix(A1, A2, V, T), "tsmqr", _ch(side), _ch(trans), m1, n1, m2, n2, k, ib,
          p1, ld1, p2, ld2, pv, ldv, pt, ldt, None, 0)


def parfb(*args):
    """parfb!(side, trans, direct, storev, m1, n1, m2, n2, k, l, A1, A2, V, T, work)
    | parfb!(side, trans, direct, storev, A1, A2, V, T) -- src/parfb.jl:44-239."""
    _arity("parfb", args, 15, 8)
    if len(args) == 8:
        side, trans, direct, storev, A1, A2, V, T = args
        m1, n1 = A1.shape
        m2, n2 = A2.shape
        k = T.shape[0]
        l = V.shape[1]                         # the reference helper's choice (src/parfb.jl:226)
        return parfb(side, trans, direct, storev, m1, n1, m2, n2, k, l, A1, A2, V, T, None)
    side, trans, direct, storev, m1, n1, m2, n2, k, l, A1, A2, V, T, work = args
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    pw, ldw = None, 1
    if _ch(direct) != b"F" or _ch(storev) != b"C":
        # backward or rowwise forms run through pamm! and need the work block
        # (k x n2 for side 'L', m2 x k for 'R'), as the reference's parfb! does
        if work is None or work.dim() != 2:
            work = zeros(*((k, n2) if _ch(side) == b"L" else (m2, k)), dtype=A1.dtype, device=A1.device)
        pw, ldw = _mat(work)
    _call(_prefix(A1, A2, V, T), "parfb", _ch(side), _ch(trans), _ch(direct), _ch(storev),
          m1, n1, m2, n2, k, l, p1, ld1, p2, ld2, pv, ldv, pt, ldt, pw, ldw)


def pamm(op, side, storev, direct, m, n, k, l, A1, A2, V, W):
    """pamm!(op, side, storev, direct, m, n, k, l, A1, A2, V, W) -- src/pamm.jl:49-473
    (op 'W': W = A1 + op(V) A2 or A1 + A2 op(V); op 'A': A2 -= op(V) W or W op(V),
    every storev / direct form, V's trapezoid of order l)."""
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pw, ldw = _mat(W)
    _call(_prefix(A1, A2, V, W), "pamm", _ch(op), _ch(side), _ch(storev), _ch(direct), m, n, k, l,
          p1, ld1, p2, ld2, pv, ldv, pw, ldw)


def ttqrt(*args):
    """ttqrt!(m, n, ib, A1, A2, T, tau, work) | ttqrt!(A, B, T) -- src/ttqrt.jl:81-144.
    QR of [A1; A2] with both upper triangular.  The helper returns (A1, A2, T, tau)."""
    _arity("ttqrt", args, 8, 3)
    if len(args) == 3:
        A1, A2, T = args
        m, n = A1.shape
        if A2.shape[1] != n:
            raise ArgumentError(f"A and B must have the same number of columns: got {n} and {A2.shape[1]}")
        ib = T.shape[0]
        tau = torch.zeros(min(m, n), dtype=A1.dtype, device=A1.device)
        ttqrt(m, n, ib, A1, A2, T, tau, None)
        return A1, A2, T, tau
    m, n, ib, A1, A2, T, tau, work = args
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pt, ldt = _mat(T)
    _call(_prefix(A1, A2, T, tau), "ttqrt", m, n, ib, p1, ld1, p2, ld2, pt, ldt, _ptr(tau), None)


def ttmqr(*args):
    """ttmqr!(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work)
    | ttmqr!(side, trans, A1, A2, V, T) -- src/ttmqr.jl:1-134."""
    _arity("ttmqr", args, 13, 6)
    if len(args) == 6:
        side, trans, A1, A2, V, T = args
        m1, n1 = A1.shape
        m2, n2 = A2.shape
        ib = T.shape[0]
        kmax = m1 if _ch(side) == b"L" else n1
        k = min(T.shape[1], kmax, V.shape[1])      # src/ttmqr.jl:120-123
        return ttmqr(side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, None)
    side, trans, m1, n1, m2, n2, k, ib, A1, A2, V, T, work = args
    p1, ld1 = _mat(A1)
    p2, ld2 = _mat(A2)
    pv, ldv = _mat(V)
    pt, ldt = _mat(T)
    _call(_prefix(A1, A2, V, T), "ttmqr", _ch(side), _ch(trans), m1, n1, m2, n2, k, ib,
          p1, ld1, p2, ld2, pv, ldv, pt, ldt, None, 0)


# ---- tile QR, Q application, solve ------------------------------------------

def tile_shapes(m, n, nb, ib):
    """Shapes of the T and tau arrays tile_geqrf fills."""
    MT = (m + nb - 1) // nb
    return (MT * ib, n), (n, MT)


_WORK = {}


def dag_worksize(m, n, nb, ib):
    """Scratch bytes of the persistent-kernel tile QR, or None if the shape
    is outside it (m, n multiples of nb <= 256, nb a multiple of ib)."""
    import ctypes
    b = ctypes.c_size_t(0)
    rc = _lib.lib().tqr_tile_dag_worksize(m, n, nb, ib, ctypes.byref(b))
    return int(b.value) if rc == 0 else None


def dag_workspace(m, n, nb, ib, device):
    """Cached device scratch for the DAG tile QR (one per shape and device)."""
    size = dag_worksize(m, n, nb, ib)
    if size is None:
        return None
    key = (str(device), size)
    w = _WORK.get(key)
    if w is None:
        w = torch.empty(size + 256, dtype=torch.uint8, device=device)
        _WORK[key] = w
    off = (-w.data_ptr()) % 256
    return w, off, size


def dag_check(m, n, nb, ib):
    """Host replay of the task schedule for a shape: (status, number of tasks)."""
    import ctypes
    nt = ctypes.c_longlong(0)
    rc = _lib.lib().tqr_tile_dag_check(m, n, nb, ib, ctypes.byref(nt))
    return rc, int(nt.value)


def dag_status(work_ptr):
    import ctypes
    s, t = ctypes.c_int(0), ctypes.c_int(0)
    rc = _lib.lib().tqr_tile_dag_status(ctypes.c_void_p(work_ptr), ctypes.byref(s), ctypes.byref(t),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise RuntimeError(f"tile_dag_status: CUDA error {rc}")
    return s.value, t.value


_LAST_DAG_WORK = None

DAG_TASKS = ("GB", "GA", "UN", "TB", "TA", "TM")


def dag_stats():
    """Busy time per task type, total wait time and span (ms, summed over CTAs)
    of the last persistent-kernel tile QR; synchronises the current stream."""
    import ctypes
    if _LAST_DAG_WORK is None:
        return None
    out = (ctypes.c_ulonglong * 9)()
    rc = _lib.lib().tqr_tile_dag_stats(ctypes.c_void_p(_LAST_DAG_WORK), out,
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    if rc != 0:
        raise RuntimeError(f"tile_dag_stats: CUDA error {rc}")
    res = {f"busy_ms_{t}": out[q] / 1e6 for q, t in enumerate(DAG_TASKS)}
    res["wait_ms"] = out[6] / 1e6
    res["span_ms"] = (out[8] - out[7]) / 1e6 if out[8] > out[7] else None
    return res


def tile_geqrf(A, nb=256, ib=32, T=None, tau=None, dag=True):
    """Flat-tree tile QR of A in place; returns (T, tau).

    dag=True runs the single persistent-kernel schedule when the shape allows
    it (scratch from a cached workspace), otherwise the stream driver; both
    give the same bits."""
    import ctypes
    m, n = A.shape
    ts, taus = tile_shapes(m, n, nb, ib)
    if T is None:
        T = zeros(*ts, dtype=A.dtype, device=A.device)
    if tau is None:
        tau = zeros(*taus, dtype=A.dtype, device=A.device)
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    pu, ldu = _mat(tau)
    ws = dag_workspace(m, n, nb, ib, A.device) if dag else None
    if ws is None:
        _call(_prefix(A, T, tau), "tile_geqrf", m, n, nb, ib, pa, lda, pt, ldt, pu, ldu)
        return T, tau
    global _LAST_DAG_WORK
    w, off, size = ws
    wp = w.data_ptr() + off
    _LAST_DAG_WORK = wp
    p = _prefix(A, T, tau)
    st = torch.cuda.current_stream()
    rc = getattr(_lib.lib(), f"tqr_{p}tile_geqrf_dag")(m, n, nb, ib, pa, lda, pt, ldt, pu, ldu,
                                                      ctypes.c_void_p(wp), size, st.cuda_stream)
    if rc == -3:
        # outside the persistent path for this element type (ComplexF64's
        # tasks need twice the shared memory): the stream driver
        _call(p, "tile_geqrf", m, n, nb, ib, pa, lda, pt, ldt, pu, ldu)
        return T, tau
    if rc < 0:
        raise ArgumentError(f"tile_geqrf: illegal value of argument {-rc}")
    if rc > 0:
        raise RuntimeError(f"tile_geqrf: CUDA error {rc}")
    if _BLOCKING:
        status, task = dag_status(wp)
        if status != 0:
            raise RuntimeError(f"tile_geqrf: schedule wait timed out at task {task} (status {status})")
    return T, tau


def tile_geqrf_f64p(A, nb=256, ib=32, T=None, tau=None):
    """The FP32 tile QR of the mixed solve on its own: A float32, trailing
    updates in FP32, panel tasks (larfg, larft, tsqrt blocks and diagonal R
    triangles) in FP64, V/T/tau rounded to FP32 (tqr_stile_geqrf_dag_f64p).
    Needs the persistent-kernel shape (m, n multiples of nb).  Returns (T, tau)."""
    import ctypes
    if A.dtype != torch.float32:
        raise TypeError("tile_geqrf_f64p factors a float32 matrix")
    m, n = A.shape
    ts, taus = tile_shapes(m, n, nb, ib)
    if T is None:
        T = zeros(*ts, dtype=A.dtype, device=A.device)
    if tau is None:
        tau = zeros(*taus, dtype=A.dtype, device=A.device)
    ws = dag_workspace(m, n, nb, ib, A.device)
    if ws is None:
        raise ArgumentError("tile_geqrf_f64p: shape outside the persistent path")
    global _LAST_DAG_WORK
    w, off, size = ws
    wp = w.data_ptr() + off
    _LAST_DAG_WORK = wp
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    pu, ldu = _mat(tau)
    st = torch.cuda.current_stream()
    rc = _lib.lib().tqr_stile_geqrf_dag_f64p(m, n, nb, ib, pa, lda, pt, ldt, pu, ldu, ctypes.c_void_p(wp), size,
                                            st.cuda_stream)
    if rc < 0:
        raise ArgumentError(f"tile_geqrf_f64p: illegal value of argument {-rc}")
    if rc > 0:
        raise RuntimeError(f"tile_geqrf_f64p: CUDA error {rc}")
    if _BLOCKING:
        status, task = dag_status(wp)
        if status != 0:
            raise RuntimeError(f"tile_geqrf_f64p: schedule wait timed out at task {task} (status {status})")
    return T, tau


def dsgels_hqr_group(grp):
    """Factorisation schedule of lstsq_mixed: grp > 0 = the hierarchical tree
    with groups of grp tiles when A has at least 2 grp tile rows (default
    16), 0 = the flat tree always; returns the previous setting."""
    return int(_lib.lib().tqr_dsgels_hqr_group(int(grp)))


def dsgels_fp64_panels(on):
    """Whether lstsq_mixed factors with FP64 panels (default True); returns
    the previous setting."""
    return bool(_lib.lib().tqr_dsgels_fp64_panels(1 if on else 0))


def autotune_tiling(m, n, dtype=torch.float64, force=False):
    """(nb, ib) for the tile QR of an m x n matrix of `dtype` (float64 or
    float32), chosen by timing every candidate tiling on a seeded matrix of
    that shape (libtileqr's tqr_tile_autotune).  Cached per (dtype, m, n):
    the first call for a shape allocates and synchronises, later calls return
    the cached pair; force=True times again."""
    import ctypes
    if dtype not in (torch.float64, torch.float32):
        raise ArgumentError("autotune_tiling: dtype must be float64 or float32")
    nb, ib = ctypes.c_int(0), ctypes.c_int(0)
    st = torch.cuda.current_stream()
    rc = _lib.lib().tqr_tile_autotune(8 if dtype == torch.float64 else 4, m, n, 1 if force else 0,
                                      ctypes.byref(nb), ctypes.byref(ib), st.cuda_stream)
    if rc < 0 and rc > -1000:
        raise ArgumentError(f"autotune_tiling: illegal value of argument {-rc}")
    if rc != 0:
        raise RuntimeError(f"autotune_tiling: error {rc}")
    return nb.value, ib.value


def tile_geqrf_tuned(A, T=None, tau=None):
    """Tile QR of A in place with the autotuned (nb, ib) for its shape and
    element type; returns (T, tau, nb, ib) -- T and tau in the layout of that
    tiling, which later calls (tile_unmqr, tile_gels) must use."""
    m, n = A.shape
    nb, ib = autotune_tiling(m, n, A.dtype)
    T, tau = tile_geqrf(A, nb, ib, T, tau)
    return T, tau, nb, ib


def tree_dag_workspace(m, n, nb, ib, nrhs, device, grp=1):
    """(buffer, aligned pointer, bytes) for the tree task-graph kernel, or None
    when the shape is outside it."""
    import ctypes
    size = ctypes.c_size_t(0)
    if _lib.lib().tqr_tile_hqr_dag_worksize(m, n, nb, ib, grp, nrhs, ctypes.byref(size)) != 0:
        return None
    key = ("tree", str(device), size.value)
    w = _WORK.get(key)
    if w is None:
        w = torch.empty(size.value + 256, dtype=torch.uint8, device=device)
        _WORK[key] = w
    return w, w.data_ptr() + ((-w.data_ptr()) % 256), size.value


def tree_dag_check(m, n, nb, ib, nrhs=0, grp=1):
    """Host check of the tree task graph; returns the task count."""
    import ctypes
    nt = ctypes.c_longlong(0)
    rc = _lib.lib().tqr_tile_hqr_dag_check(m, n, nb, ib, grp, nrhs, ctypes.byref(nt))
    if rc != 0:
        raise RuntimeError(f"tree task graph check failed ({rc})")
    return nt.value


def tile_geqrf_tree(A, nb=256, ib=32, B=None, dag=True, grp=1, f64p=False):
    """Tile QR of A in place with a binary reduction tree per panel (geqrt!
    on every tile, ttqrt!/ttmqr! merges).  Returns (T, tau, T2, tau2); with B,
    B is overwritten by Q^T B in the same pass.  dag=True runs it as one
    persistent launch when the shape allows (same results as the stream
    driver for FP64).  grp > 1: the hierarchical form -- groups of grp tiles
    reduced flat into their first tile (tsqrt!/tsmqr!), the group leaders by
    the binary tree.  f64p=True (float32 A, task graph only): the mixed
    solve's form, panel steps in FP64 (tqr_stile_geqrf_hqr_dag_f64p)."""
    import ctypes
    m, n = A.shape
    ts, taus = tile_shapes(m, n, nb, ib)
    T = zeros(*ts, dtype=A.dtype, device=A.device)
    T2 = zeros(*ts, dtype=A.dtype, device=A.device)
    tau = zeros(*taus, dtype=A.dtype, device=A.device)
    tau2 = zeros(*taus, dtype=A.dtype, device=A.device)
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    pu, ldu = _mat(tau)
    nrhs, pb, ldb = 0, None, 1
    if B is not None:
        nrhs = B.shape[1]
        pb, ldb = _mat(B)
    ws = tree_dag_workspace(m, n, nb, ib, nrhs, A.device, grp) if dag else None
    if ws is None and f64p:
        raise ArgumentError("tile_geqrf_tree: f64p needs the persistent task graph's shape")
    if ws is None:
        _call(_prefix(A, T, tau, B), "tile_geqrf_hqr", m, n, nb, ib, grp, pa, lda, pt, _ptr(T2), ldt, pu,
              _ptr(tau2), ldu, nrhs, pb, ldb)
        return T, tau, T2, tau2
    _, wp, size = ws
    p = _prefix(A, T, tau, B)
    st = torch.cuda.current_stream()
    if f64p and p != "s":
        raise TypeError("tile_geqrf_tree: f64p needs a float32 matrix")
    fn = "tqr_stile_geqrf_hqr_dag_f64p" if f64p else f"tqr_{p}tile_geqrf_hqr_dag"
    rc = getattr(_lib.lib(), fn)(m, n, nb, ib, grp, pa, lda, pt, _ptr(T2), ldt, pu, _ptr(tau2), ldu, nrhs, pb, ldb,
                                 ctypes.c_void_p(wp), size, st.cuda_stream)
    if rc < 0:
        raise ArgumentError(f"tile_geqrf_tree: illegal value of argument {-rc}")
    if rc > 0:
        raise RuntimeError(f"tile_geqrf_tree: CUDA error {rc}")
    if _BLOCKING:
        err, item = ctypes.c_int(0), ctypes.c_int(0)
        _lib.lib().tqr_tile_tree_dag_status(ctypes.c_void_p(wp), ctypes.byref(err), ctypes.byref(item),
                                            st.cuda_stream)
        if err.value != 0:
            raise RuntimeError(f"tile_geqrf_tree: task graph stopped at task {item.value} (status {err.value})")
    return T, tau, T2, tau2


def tile_unmqr_tree(trans, A, T, T2, B, nb=256, ib=32, grp=1):
    """B := Q^T B ('C') or Q B ('N') with Q from tile_geqrf_tree (same grp)."""
    m, n = A.shape
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    pb, ldb = _mat(B)
    _call(_prefix(A, T, T2, B), "tile_unmqr_hqr", _ch(trans), m, n, B.shape[1], nb, ib, grp, pa, lda, pt,
          _ptr(T2), ldt, pb, ldb)


def tile_unmqr(trans, A, T, B, nb=256, ib=32):
    """B := Q^T B (trans 'C'/'T') or Q B (trans 'N') with Q from tile_geqrf."""
    m, n = A.shape
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    pb, ldb = _mat(B)
    _call(_prefix(A, T, B), "tile_unmqr", _ch(trans), m, n, B.shape[1], nb, ib, pa, lda, pt, ldt,
          pb, ldb)


def trsm_lun(R, B):
    """Solve R X = B in place (upper triangle of the square R)."""
    pr, ldr = _mat(R)
    pb, ldb = _mat(B)
    _call(_prefix(R, B), "trsm_lun", R.shape[1], B.shape[1], pr, ldr, pb, ldb)


def tile_gels(A, B, nb=256, ib=32):
    """Least squares min ||A X - B|| (m >= n) in place: A := tile QR, B[:n] := X.
    Returns (X view, T, tau)."""
    m, n = A.shape
    ts, taus = tile_shapes(m, n, nb, ib)
    T = zeros(*ts, dtype=A.dtype, device=A.device)
    tau = zeros(*taus, dtype=A.dtype, device=A.device)
    pa, lda = _mat(A)
    pt, ldt = _mat(T)
    pu, ldu = _mat(tau)
    pb, ldb = _mat(B)
    _call(_prefix(A, T, tau, B), "tile_gels", m, n, B.shape[1], nb, ib, pa, lda, pt, ldt, pu, ldu,
          pb, ldb)
    return B[:n], T, tau


# ---- mixed-precision least squares -----------------------------------------

def lstsq_mixed(A32, B, nb=256, ib=32, maxit=50, tol=1e-13):
    """min ||A X - B|| for a float32 A and float64 B: FP32 tile QR, then CGLS
    with FP64 iterates preconditioned by R, its products with A summed in
    double-float (tqr_dsgels).  Returns (X, iterations, relative
    preconditioned residual reached).  A and B are left unchanged."""
    import ctypes
    if A32.dtype != torch.float32 or B.dtype != torch.float64:
        raise TypeError("lstsq_mixed wants a float32 A and a float64 B")
    m, n = A32.shape
    k = B.shape[1]
    pa, lda = _mat(A32)
    pb, ldb = _mat(B)
    X = zeros(n, k, dtype=torch.float64, device=A32.device)
    px, ldx = _mat(X)
    L = _lib.lib()
    size = ctypes.c_size_t(0)
    L.tqr_dsgels_worksize(m, n, k, nb, ib, ctypes.byref(size))
    key = ("sgels", str(A32.device), size.value)
    w = _WORK.get(key)
    if w is None:
        w = torch.empty(size.value + 256, dtype=torch.uint8, device=A32.device)
        _WORK[key] = w
    wp = w.data_ptr() + ((-w.data_ptr()) % 256)
    it = ctypes.c_int(0)
    rr = ctypes.c_double(0)
    st = torch.cuda.current_stream()
    rc = L.tqr_dsgels(m, n, k, nb, ib, pa, lda, pb, ldb, px, ldx, maxit, tol, ctypes.c_void_p(wp),
                      size.value, ctypes.byref(it), ctypes.byref(rr), st.cuda_stream)
    if rc < 0:
        raise ArgumentError(f"dsgels: illegal value of argument {-rc}")
    if rc > 0:
        raise RuntimeError(f"dsgels: CUDA error {rc}")
    if _BLOCKING:
        st.synchronize()
    return X, it.value, rr.value


def dsgels_phases():
    """Device ms of the last mixed solve: (FP32 QR, X0, CGLS), iterations."""
    import ctypes
    ms = (ctypes.c_double * 3)()
    it = ctypes.c_int(0)
    _lib.lib().tqr_dsgels_phases(ms, ctypes.byref(it))
    return {"qr32_ms": ms[0], "x0_ms": ms[1], "cgls_ms": ms[2], "iterations": it.value}


def lstsq_fp64(A, B, nb=256, ib=32):
    """The plain FP64 least-squares solve on the tile QR: factors A in place
    (persistent kernel when the shape allows), B := Q^T B, then R X = B[0:n].
    Returns the view of B holding X."""
    import ctypes
    m, n = A.shape
    k = B.shape[1]
    size = ctypes.c_size_t(0)
    L = _lib.lib()
    if 0 < k <= nb and L.tqr_tile_gels_worksize(m, n, k, nb, ib, ctypes.byref(size)) == 0:
        # one persistent launch factors A with B as an extra tile column, then R X = Q^T B
        ts, taus = tile_shapes(m, n, nb, ib)
        T = zeros(*ts, dtype=A.dtype, device=A.device)
        tau = zeros(*taus, dtype=A.dtype, device=A.device)
        key = ("gels", str(A.device), size.value)
        w = _WORK.get(key)
        if w is None:
            w = torch.empty(size.value + 256, dtype=torch.uint8, device=A.device)
            _WORK[key] = w
        wp = w.data_ptr() + ((-w.data_ptr()) % 256)
        pa, lda = _mat(A)
        pt, ldt = _mat(T)
        pu, ldu = _mat(tau)
        pb, ldb = _mat(B)
        p = _prefix(A, B)
        st = torch.cuda.current_stream()
        rc = getattr(L, f"tqr_{p}tile_gels_dag")(m, n, k, nb, ib, pa, lda, pt, ldt, pu, ldu, pb, ldb,
                                                 ctypes.c_void_p(wp), size.value, st.cuda_stream)
        if rc < 0:
            raise ArgumentError(f"tile_gels: illegal value of argument {-rc}")
        if rc > 0:
            raise RuntimeError(f"tile_gels: CUDA error {rc}")
        if _BLOCKING:
            st.synchronize()
        return B[:n]
    T, _ = tile_geqrf(A, nb, ib)
    tile_unmqr("C", A, T, B, nb, ib)
    X = B[:n]
    trsm_lun(A[:n, :n], X)
    return X
