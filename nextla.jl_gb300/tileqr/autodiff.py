"""Differentiable batched QR: forward and adjoint kernels behind an autograd rule.

`qr(A)` factors a batch of m-by-n matrices (m >= n, n <= 256) with the tile
QR of NextLA's kernels (geqrt! on the top 256-row tile, tsqrt! against every
further tile; src/geqrt.jl:22-68, src/tsqrt.jl:46-126) and returns the thin
Q and R.  `QRFunction` is the torch.autograd.Function that plays the part of
a ChainRulesCore `rrule` for Julia callers: its forward saves only the packed
factor and tau, and its backward runs the hand-written adjoint kernel, which
recomputes every T factor from V and tau (larft!, src/larft.jl:53-86) and
returns Abar = (Qbar + Q copyltu(R Rbar^T - Qbar^T Q)) R^-T.

Complex tensors (complex128, complex64) take the same path with conjugate
transposes and the real part of M's diagonal (R's diagonal is real):
Abar = (Qbar + Q X) R^-H, X = tril(M,-1) + tril(M,-1)^H + Re diag(M),
M = R Rbar^H - Qbar^H Q -- gradients in torch's convention for a real loss
(dL/dRe + i dL/dIm).
"""
import ctypes

import torch

from . import _lib
from . import ArgumentError

TILE = 256
_WORK = {}


def _check(rc, what):
    if rc < 0:
        raise ArgumentError(f"{what}: illegal value of argument {-rc}")
    if rc > 0:
        raise RuntimeError(f"{what}: CUDA error {rc}")


def _prefix(dtype):
    if dtype == torch.float64:
        return "d", 8
    if dtype == torch.float32:
        return "s", 4
    if dtype == torch.complex128:
        return "z", 16
    if dtype == torch.complex64:
        return "c", 8
    raise TypeError(f"unsupported element type {dtype}")


def cm_empty(batch, m, n, dtype, device):
    """(batch, m, n) tensor with every matrix column-major and packed."""
    return torch.empty((batch, n, m), dtype=dtype, device=device).transpose(1, 2)


def cm_copy(x, dtype=None):
    b, m, n = x.shape
    out = cm_empty(b, m, n, dtype or x.dtype, x.device)
    out.copy_(x)
    return out


def workspace(dtype, m, n, ib, device):
    _, nb = _prefix(dtype)
    size = ctypes.c_size_t(0)
    _check(_lib.lib().tqr_qr_batched_worksize(nb, m, n, ib, ctypes.byref(size)), "qr_batched_worksize")
    key = (str(device), nb, m, n, ib, str(dtype))
    w = _WORK.get(key)
    if w is None:
        w = torch.empty(size.value + 256, dtype=torch.uint8, device=device)
        _WORK[key] = w
    return w.data_ptr() + ((-w.data_ptr()) % 256), size.value


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def qr_forward(A, ib=32):
    """(Q, R, F, tau): explicit thin Q, R and the saved packed factor."""
    if A.dim() == 2:
        A = A.unsqueeze(0)
    b, m, n = A.shape
    p, _ = _prefix(A.dtype)
    F = cm_copy(A)
    mt = (m + TILE - 1) // TILE
    tau = torch.zeros((b, mt * n), dtype=A.dtype, device=A.device)
    Q = cm_empty(b, m, n, A.dtype, A.device)
    R = cm_empty(b, n, n, A.dtype, A.device)
    wp, lw = workspace(A.dtype, m, n, ib, A.device)
    st = torch.cuda.current_stream()
    _check(getattr(_lib.lib(), f"tqr_{p}qr_batched_fwd")(b, m, n, ib, _ptr(F), _ptr(tau), _ptr(Q), _ptr(R),
                                                         ctypes.c_void_p(wp), lw, ctypes.c_void_p(st.cuda_stream)),
           "qr_batched_fwd")
    return Q, R, F, tau


def qr_backward(F, tau, Qbar, Rbar, ib=32):
    """Abar (batch, m, n) from the saved factor and the cotangents."""
    b, m, n = F.shape
    p, _ = _prefix(F.dtype)
    Qb = cm_copy(Qbar, F.dtype) if Qbar is not None else cm_empty(b, m, n, F.dtype, F.device).zero_()
    Rb = cm_copy(Rbar, F.dtype) if Rbar is not None else cm_empty(b, n, n, F.dtype, F.device).zero_()
    Abar = cm_empty(b, m, n, F.dtype, F.device)
    wp, lw = workspace(F.dtype, m, n, ib, F.device)
    st = torch.cuda.current_stream()
    _check(getattr(_lib.lib(), f"tqr_{p}qr_batched_bwd")(b, m, n, ib, _ptr(F), _ptr(tau), _ptr(Qb), _ptr(Rb),
                                                         _ptr(Abar), ctypes.c_void_p(wp), lw,
                                                         ctypes.c_void_p(st.cuda_stream)),
           "qr_batched_bwd")
    return Abar


class QRFunction(torch.autograd.Function):
    """(Q, R) = qr(A) for a (batch, m, n) A; backward by the adjoint kernel."""

    @staticmethod
    def forward(ctx, A, ib):
        squeeze = A.dim() == 2
        Q, R, F, tau = qr_forward(A, ib)
        ctx.save_for_backward(F, tau)
        ctx.ib = ib
        ctx.squeeze = squeeze
        if squeeze:
            return Q[0], R[0]
        return Q, R

    @staticmethod
    def backward(ctx, Qbar, Rbar):
        F, tau = ctx.saved_tensors
        if ctx.squeeze:
            Qbar = Qbar.unsqueeze(0) if Qbar is not None else None
            Rbar = Rbar.unsqueeze(0) if Rbar is not None else None
        Abar = qr_backward(F, tau, Qbar, Rbar, ctx.ib)
        return (Abar[0] if ctx.squeeze else Abar), None


def qr(A, ib=32):
    """Thin QR of a matrix or a (batch, m, n) stack, differentiable."""
    return QRFunction.apply(A, ib)
