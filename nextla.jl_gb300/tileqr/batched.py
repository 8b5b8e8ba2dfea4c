"""Batched uneven QR + least squares on one persistent launch (tqr_?batched_*).

NextLA factors one matrix at a time; this is the batched form of its
single-tile path, geqrt! + unmqr!('L','T') + LeftUpperTRSM! per problem
(src/geqrt.jl:22-68, src/unmqr.jl:52-149, src/trsm.jl:36-63).

All problems of a batch live in two flat device buffers: problem q's A is the
column-major m_q-by-n_q block at A[a_off : a_off + m_q n_q] and its B the
m_q-by-k_q block at B[b_off : b_off + m_q k_q]; the offsets come from the
plan (every block 32-element aligned).  After a solve the A block holds
geqrt!'s R (upper triangle) and V (below it), and rows 0:n_q of the B block
hold X_q.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import ArgumentError

PROBLEM_DTYPE = np.dtype([("m", "<i4"), ("n", "<i4"), ("k", "<i4"), ("ib", "<i4"), ("nw", "<i4"),
                          ("pad", "<i4"), ("a_off", "<i8"), ("b_off", "<i8")])
MAX_M = 512
MAX_K = 8

_TUNED = set()


def _check(rc, what):
    if rc < 0:
        raise ArgumentError(f"{what}: illegal value of argument {-rc}")
    if rc > 0:
        raise RuntimeError(f"{what}: CUDA error {rc}")


def _nbytes(dtype):
    if dtype in (torch.float64, torch.complex64):
        return 8
    if dtype == torch.float32:
        return 4
    if dtype == torch.complex128:
        return 16
    raise TypeError(f"unsupported element type {dtype}")


_PREFIX = {torch.float64: "d", torch.float32: "s", torch.complex128: "z", torch.complex64: "c"}


def autotune(dtype=torch.float64, force=False):
    """Time every (ib, strip width) candidate per column-count class and keep
    the fastest (allocates; run before planning, outside graph capture).
    Real types only; complex batches plan with the table of their real
    precision."""
    if dtype.is_complex:
        raise TypeError("the batched autotuner times real batches only")
    nb = _nbytes(dtype)
    st = torch.cuda.current_stream()
    _check(_lib.lib().tqr_batched_autotune(nb, 1 if force else 0, st.cuda_stream), "batched_autotune")
    _TUNED.add(nb)


def tuning(dtype, n):
    """(ib, strip width) the table holds for problems with n columns."""
    ib = ctypes.c_int(0)
    nw = ctypes.c_int(0)
    _check(_lib.lib().tqr_batched_tuning(_nbytes(dtype), int(n), ctypes.byref(ib), ctypes.byref(nw)),
           "batched_tuning")
    return ib.value, nw.value


def plan(ms, ns, ks, dtype=torch.float64):
    """Descriptors (PROBLEM_DTYPE array), order (int32, most flops first) and
    the packed lengths of A and B for problems of the given sizes."""
    ms = np.ascontiguousarray(ms, dtype=np.int32)
    ns = np.ascontiguousarray(ns, dtype=np.int32)
    ks = np.ascontiguousarray(ks, dtype=np.int32)
    if not (ms.shape == ns.shape == ks.shape) or ms.ndim != 1:
        raise ArgumentError("m, n, k must be vectors of one length")
    L = _lib.lib()
    if L.tqr_batched_problem_bytes() != PROBLEM_DTYPE.itemsize:
        raise RuntimeError("descriptor layout of the library differs from the bindings")
    nprob = len(ms)
    desc = np.zeros(nprob, dtype=PROBLEM_DTYPE)
    order = np.zeros(nprob, dtype=np.int32)
    ae = ctypes.c_longlong(0)
    be = ctypes.c_longlong(0)
    rc = L.tqr_batched_plan(_nbytes(dtype), nprob, ms.ctypes.data, ns.ctypes.data, ks.ctypes.data,
                            desc.ctypes.data, order.ctypes.data, ctypes.byref(ae), ctypes.byref(be))
    if rc <= -1000:
        q = -rc - 1000
        raise ArgumentError(f"batched problem {q} out of range: m={ms[q]}, n={ns[q]}, k={ks[q]} "
                            f"(need 1 <= n <= m <= {MAX_M}, 0 <= k <= {MAX_K})")
    _check(rc, "batched_plan")
    return desc, order, ae.value, be.value


class BatchedGels:
    """One batch of independent problems min ||A_q X_q - B_q||: the plan, the
    packed device buffers, the workspace and (optionally) a CUDA graph of the
    launch.  Fill `A` and `B` (flat tensors), then `run()` or `replay()`."""

    def __init__(self, ms, ns, ks, dtype=torch.float64, device="cuda", tune=True):
        self.dtype = dtype
        self.device = torch.device(device)
        nb = _nbytes(dtype)
        if tune and not dtype.is_complex and nb not in _TUNED:
            autotune(dtype)
        self.desc, self.order, a_elems, b_elems = plan(ms, ns, ks, dtype)
        self.nprob = len(self.desc)
        self.d_desc = torch.from_numpy(self.desc.view(np.uint8).copy()).to(self.device)
        self.d_order = torch.from_numpy(self.order.copy()).to(self.device)
        self.A = torch.zeros(a_elems, dtype=dtype, device=self.device)
        self.B = torch.zeros(b_elems, dtype=dtype, device=self.device)
        size = ctypes.c_size_t(0)
        _check(_lib.lib().tqr_batched_worksize(nb, ctypes.byref(size)), "batched_worksize")
        self.lwork = size.value
        self._work = torch.empty(self.lwork + 256, dtype=torch.uint8, device=self.device)
        self.work_ptr = self._work.data_ptr() + ((-self._work.data_ptr()) % 256)
        self._graph = None

    # -- problem views ------------------------------------------------------
    def a_view(self, q, buf=None):
        d = self.desc[q]
        buf = self.A if buf is None else buf
        m, n, off = int(d["m"]), int(d["n"]), int(d["a_off"])
        return buf[off:off + m * n].view(n, m).t()

    def b_view(self, q, buf=None):
        d = self.desc[q]
        buf = self.B if buf is None else buf
        m, k, off = int(d["m"]), int(d["k"]), int(d["b_off"])
        return buf[off:off + m * k].view(k, m).t()

    def x_view(self, q, buf=None):
        return self.b_view(q, buf)[: int(self.desc[q]["n"])]

    def load(self, As, Bs):
        """Copy per-problem matrices (numpy or tensors) into the packed buffers."""
        for q in range(self.nprob):
            self.a_view(q).copy_(torch.as_tensor(As[q], dtype=self.dtype))
            if int(self.desc[q]["k"]) > 0:
                self.b_view(q).copy_(torch.as_tensor(Bs[q], dtype=self.dtype))

    # -- solve ----------------------------------------------------------------
    def _fn(self):
        return getattr(_lib.lib(), f"tqr_{_PREFIX[self.dtype]}batched_gels")

    def run(self, stream=None, sync=True):
        st = stream or torch.cuda.current_stream()
        rc = self._fn()(self.nprob, ctypes.c_void_p(self.d_desc.data_ptr()),
                        ctypes.c_void_p(self.d_order.data_ptr()), ctypes.c_void_p(self.A.data_ptr()),
                        ctypes.c_void_p(self.B.data_ptr()), ctypes.c_void_p(self.work_ptr), self.lwork,
                        ctypes.c_void_p(st.cuda_stream))
        _check(rc, "batched_gels")
        if sync:
            st.synchronize()

    def capture(self):
        """Instantiate a CUDA graph of the launch (counter reset + solve); real
        batches."""
        if self.dtype.is_complex:
            raise TypeError("graph capture of a batch is available for real element types")
        if self._graph is None:
            ex = ctypes.c_void_p(0)
            rc = _lib.lib().tqr_batched_graph(_nbytes(self.dtype), self.nprob,
                                              ctypes.c_void_p(self.d_desc.data_ptr()),
                                              ctypes.c_void_p(self.d_order.data_ptr()),
                                              ctypes.c_void_p(self.A.data_ptr()),
                                              ctypes.c_void_p(self.B.data_ptr()),
                                              ctypes.c_void_p(self.work_ptr), self.lwork, ctypes.byref(ex))
            _check(rc, "batched_graph")
            self._graph = ex
        return self._graph

    def replay(self, stream=None, sync=True):
        st = stream or torch.cuda.current_stream()
        ex = self.capture()
        _check(_lib.lib().tqr_batched_graph_launch(ex, ctypes.c_void_p(st.cuda_stream)), "batched_graph_launch")
        if sync:
            st.synchronize()

    def status(self):
        """(rejected descriptors, first rejected index or -1) of the last launch."""
        bad = ctypes.c_int(0)
        first = ctypes.c_int(0)
        st = torch.cuda.current_stream()
        _check(_lib.lib().tqr_batched_status(ctypes.c_void_p(self.work_ptr), ctypes.byref(bad),
                                             ctypes.byref(first), ctypes.c_void_p(st.cuda_stream)),
               "batched_status")
        return bad.value, first.value

    def residuals(self, A0, B0):
        """Per-problem ||A^T (B - A X)|| / (||A|| (||A|| ||X|| + ||B||)) (float64
        tensor) from the original packed A0, B0 and the current solution."""
        if self.dtype.is_complex:
            raise TypeError("the residual kernel is available for real element types")
        res = torch.empty(self.nprob, dtype=torch.float64, device=self.device)
        fn = getattr(_lib.lib(), f"tqr_{_PREFIX[self.dtype]}batched_residual")
        st = torch.cuda.current_stream()
        _check(fn(self.nprob, ctypes.c_void_p(self.d_desc.data_ptr()), ctypes.c_void_p(A0.data_ptr()),
                  ctypes.c_void_p(B0.data_ptr()), ctypes.c_void_p(self.B.data_ptr()),
                  ctypes.c_void_p(res.data_ptr()), ctypes.c_void_p(st.cuda_stream)), "batched_residual")
        st.synchronize()
        return res

    def flops(self):
        """Algorithmic flops of the batch: QR 2mn^2 - 2n^3/3, Q^T B
        k(4mn - 2n^2), triangular solve k n^2 per problem."""
        m = self.desc["m"].astype(np.float64)
        n = self.desc["n"].astype(np.float64)
        k = self.desc["k"].astype(np.float64)
        return float(np.sum(2 * m * n * n - 2 * n ** 3 / 3 + k * (4 * m * n - n * n)))

    def close(self):
        if self._graph is not None:
            _lib.lib().tqr_batched_graph_destroy(self._graph)
            self._graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def random_sizes(nprob, seed=0, max_m=MAX_M, min_m=32, min_n=16, max_k=MAX_K):
    """m ~ U[min_m, max_m], n ~ U[min_n, m], k ~ U[1, max_k] (integers, seeded)."""
    rng = np.random.default_rng(seed)
    ms = rng.integers(min_m, max_m + 1, size=nprob)
    ns = np.array([rng.integers(min(min_n, m), m + 1) for m in ms])
    ks = rng.integers(1, max_k + 1, size=nprob)
    return ms.astype(np.int32), ns.astype(np.int32), ks.astype(np.int32)


def problem_cost(ms, ns, ks):
    """Flops of each problem: 2 m n^2 - 2 n^3 / 3 (QR) + 4 m n k (Q^T B) + n^2 k (solve)."""
    m = np.asarray(ms, dtype=np.float64)
    n = np.asarray(ns, dtype=np.float64)
    k = np.asarray(ks, dtype=np.float64)
    return 2 * m * n * n - 2 * n ** 3 / 3 + 4 * m * n * k + n * n * k


def shard(ms, ns, ks, world, rank):
    """Indices of the problems rank `rank` of `world` solves: the batch split by
    cost, largest problem first onto the least-loaded rank (ties to the lower
    rank), so every rank computes the same partition without communication.
    The ranks' results are gathered on the host afterwards; the solves need no
    collective."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    cost = problem_cost(ms, ns, ks)
    order = np.lexsort((np.arange(cost.size), -cost))       # cost descending, index ascending
    load = np.zeros(world)
    owner = np.empty(cost.size, dtype=np.int64)
    for q in order:
        r = int(np.argmin(load))
        owner[q] = r
        load[r] += cost[q]
    return np.nonzero(owner == rank)[0]
