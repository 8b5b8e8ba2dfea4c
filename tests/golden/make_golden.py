"""Generate the LAPACK golden vectors that pin the oracle and the CUDA library.

The reference (NextLA.jl) checks its tile kernels against LAPACK through
libblastrampoline (test/lapack_helpers.jl: dtpqrt for tsqrt!, dtpmqrt for
tsmqr!, ormqr/geqrt for geqrt!).  Julia is not available here, so the same
LAPACK routines are called through scipy (scipy 1.18.1, OpenBLAS 0.3.34) on
seeded inputs at the reference's own test shapes, plus one nb=256, ib=32 tile,
the configuration the tile QR runs at.

Run from the repository root:  python tests/golden/make_golden.py
Writes tests/golden/lapack_golden.npz.
"""
import os

import numpy as np
from scipy.linalg import lapack

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lapack_golden.npz")


def F(a):
    return np.asfortranarray(a, dtype=np.float64)


def Q24(a):
    """Round inputs to 24 significant bits so the stored inputs compress well;
    the LAPACK outputs computed from them stay full FP64."""
    return F(np.ldexp(np.round(np.ldexp(a, 24)), -24))


def Z(a):
    return np.asfortranarray(a, dtype=np.complex128)


def QZ(re, im):
    """Complex input with both parts rounded to 24 significant bits."""
    return Z(Q24(re) + 1j * Q24(im))


def crand(rng, shape):
    """rand(ComplexF64, shape): real and imaginary parts uniform in [0, 1)."""
    return QZ(rng.random(shape), rng.random(shape))


def crandn(rng, shape):
    return QZ(rng.standard_normal(shape), rng.standard_normal(shape))


def complex_vectors(rng, g):
    """ComplexF64 vectors (every reference kernel test runs ComplexF64 too,
    test/lapack_helpers.jl:11) against zgeqrt / ztpqrt / ztpmqrt / zgemqrt /
    zlarfg, at the reference's test shapes plus one 128 x 128, ib = 32 tile.
    Keys start with "z_"."""
    # geqrt (test/geqrt.jl:6-11) vs zgeqrt
    for (m, n, ib) in [(20, 15, 4), (32, 32, 8), (64, 32, 16), (32, 64, 8), (128, 128, 32)]:
        A = crand(rng, (m, n))
        a, t, info = lapack.zgeqrt(ib, A.copy(order="F"))
        assert info == 0
        key = f"z_geqrt_{m}_{n}_{ib}"
        g[key + "_A"], g[key + "_outA"], g[key + "_outT"] = A, Z(a), Z(t[:, : min(m, n)])
    # tsqrt (test/tsqrt.jl:8-13, A1 = triu(rand) + 2I) vs ztpqrt(l = 0)
    for (m, n, ib) in [(32, 24, 8), (48, 32, 16), (20, 20, 10), (128, 128, 32)]:
        A1 = Z(np.triu(crand(rng, (n, n))) + 2.0 * np.eye(n))
        A2 = crand(rng, (m, n))
        a1, a2, t, info = lapack.ztpqrt(0, ib, A1.copy(order="F"), A2.copy(order="F"))
        assert info == 0
        key = f"z_tsqrt_{m}_{n}_{ib}"
        g[key + "_A1"], g[key + "_A2"] = A1, A2
        g[key + "_outA1"], g[key + "_outA2"], g[key + "_outT"] = Z(a1), Z(a2), Z(t)
    # tsmqr (test/tsmqr.jl:6-40) and ttmqr (test/ttmqr.jl:6-37, V = triu) vs
    # ztpmqrt(l = 0), all side x trans forms
    for kind in ("tsmqr", "ttmqr"):
        for side in "LR":
            for trans in "NC":
                if kind == "tsmqr":
                    if side == "L":
                        m1, n1, m2, k, ib = 32, 24, 20, 16, 8
                        n2 = n1
                    else:
                        m1, n1, n2, k, ib = 24, 32, 20, 16, 8
                        m2 = m1
                    V = crand(rng, (m2, k) if side == "L" else (n2, k))
                else:
                    m1 = n1 = m2 = n2 = 24
                    k, ib = 16, 8
                    V = Z(np.triu(crandn(rng, (24, k))))
                A1 = crand(rng, (m1, n1))
                A2 = crand(rng, (m2, n2))
                T = Z(np.triu(crand(rng, (ib, k))))
                out1 = A1.copy(order="F")
                sub = out1[:k] if side == "L" else out1[:, :k]
                a1, a2, info = lapack.ztpmqrt(0, V, T, Z(sub), A2.copy(order="F"), side=side, trans=trans)
                assert info == 0
                if side == "L":
                    out1[:k] = a1
                else:
                    out1[:, :k] = a1
                key = f"z_{kind}_{side}{trans}"
                g[key + "_A1"], g[key + "_A2"], g[key + "_V"], g[key + "_T"] = A1, A2, V, T
                g[key + "_outA1"], g[key + "_outA2"] = Z(out1), Z(a2)
                g[key + "_dims"] = np.array([m1, n1, m2, n2, k, ib])
    # unmqr (test/unmqr.jl:1-79) vs zgemqrt
    m, n, k, ib = 64, 48, 32, 8
    Aq = crand(rng, (m, k))
    aq, tq, info = lapack.zgeqrt(ib, Aq.copy(order="F"))
    assert info == 0
    g["z_unmqr_Aqr"], g["z_unmqr_T"] = Z(aq), Z(tq)
    for side in "LR":
        for trans in "NC":
            C = crand(rng, (m, n) if side == "L" else (n, m))
            c, info = lapack.zgemqrt(aq, tq, C.copy(order="F"), side=side, trans=trans)
            assert info == 0
            g[f"z_unmqr_{side}{trans}_C"], g[f"z_unmqr_{side}{trans}_out"] = C, Z(c)
    # larfg (test/larfg.jl) vs zlarfg
    for n in (2, 7, 33, 256):
        x = crandn(rng, (n,))
        alpha, xo, tau = lapack.zlarfg(n, x[0], x[1:].copy())
        g[f"z_larfg_{n}_x"] = x
        g[f"z_larfg_{n}_out"] = np.concatenate([[alpha], xo, [tau]])
    # ttqrt (test/ttqrt.jl:6-11) vs ztpqrt(l = n), with its Q applied both
    # ways (ttmqr 'L') vs ztpmqrt(l = n)
    for (n, ib) in [(16, 4), (24, 8), (48, 16)]:
        A1 = Z(np.triu(crandn(rng, (n, n))) + 2.0 * np.eye(n))
        A2 = Z(np.triu(crandn(rng, (n, n))) + 2.0 * np.eye(n))
        a1, a2, t, info = lapack.ztpqrt(n, ib, A1.copy(order="F"), A2.copy(order="F"))
        assert info == 0
        key = f"z_ttqrt_{n}_{ib}"
        g[key + "_A1"], g[key + "_A2"] = A1, A2
        g[key + "_outA1"], g[key + "_outA2"], g[key + "_outT"] = Z(a1), Z(a2), Z(t)
        for trans in "NC":
            C1, C2 = crandn(rng, (n, 40)), crandn(rng, (n, 40))
            c1, c2, info = lapack.ztpmqrt(n, Z(a2), Z(t), C1.copy(order="F"), C2.copy(order="F"),
                                          side="L", trans=trans)
            assert info == 0
            g[f"{key}_L{trans}_C1"], g[f"{key}_L{trans}_C2"] = C1, C2
            g[f"{key}_L{trans}_out1"], g[f"{key}_L{trans}_out2"] = Z(c1), Z(c2)


def main():
    rng = np.random.default_rng(20240611)
    g = {}
    # geqrt (test/geqrt.jl:6-11 shapes) vs dgeqrt (same T layout, nb = ib).
    for (m, n, ib) in [(20, 15, 4), (32, 32, 8), (64, 32, 16), (32, 64, 8), (256, 256, 32)]:
        A = Q24(rng.random((m, n)))
        a, t, info = lapack.dgeqrt(ib, A.copy(order="F"))
        assert info == 0
        key = f"geqrt_{m}_{n}_{ib}"
        g[key + "_A"] = A
        g[key + "_outA"] = F(a)
        g[key + "_outT"] = F(t[:, : min(m, n)])
    # tsqrt (test/tsqrt.jl:8-13 shapes, A1 = triu(rand) + 2I) vs dtpqrt(l=0, nb=ib).
    for (m, n, ib) in [(32, 24, 8), (48, 32, 16), (64, 48, 16), (20, 20, 10), (256, 256, 32)]:
        A1 = Q24(np.triu(rng.random((n, n))) + 2.0 * np.eye(n))
        A2 = Q24(rng.random((m, n)))
        a1, a2, t, info = lapack.dtpqrt(0, ib, A1.copy(order="F"), A2.copy(order="F"))
        assert info == 0
        key = f"tsqrt_{m}_{n}_{ib}"
        g[key + "_A1"], g[key + "_A2"] = A1, A2
        g[key + "_outA1"], g[key + "_outA2"], g[key + "_outT"] = F(a1), F(a2), F(t)
    # tsmqr (test/tsmqr.jl:6-40: side x trans, random V, triu(T)) vs dtpmqrt(l=0).
    for side in "LR":
        for trans in "NC":
            if side == "L":
                m1, n1, m2, k, ib = 32, 24, 20, 16, 8
                n2 = n1
            else:
                m1, n1, n2, k, ib = 24, 32, 20, 16, 8
                m2 = m1
            A1 = F(rng.random((m1, n1)))
            A2 = F(rng.random((m2, n2)))
            V = F(rng.random((m2, k) if side == "L" else (n2, k)))
            T = F(np.triu(rng.random((ib, k))))
            out1 = A1.copy(order="F")
            sub = out1[:k] if side == "L" else out1[:, :k]
            a1, a2, info = lapack.dtpmqrt(0, V, T, F(sub), A2.copy(order="F"), side=side,
                                          trans="T" if trans == "C" else "N")
            assert info == 0
            if side == "L":
                out1[:k] = a1
            else:
                out1[:, :k] = a1
            key = f"tsmqr_{side}{trans}"
            g[key + "_A1"], g[key + "_A2"], g[key + "_V"], g[key + "_T"] = A1, A2, V, T
            g[key + "_outA1"], g[key + "_outA2"] = F(out1), F(a2)
            g[key + "_dims"] = np.array([m1, n1, m2, n2, k, ib])
    # tsmqr at the tile size the driver uses (nb = 256, ib = 32, 128 columns),
    # left, transposed.
    A1 = Q24(rng.standard_normal((256, 128)))
    A2 = Q24(rng.standard_normal((256, 128)))
    V = Q24(rng.standard_normal((256, 256)) / 16.0)
    T = Q24(np.triu(rng.standard_normal((32, 256))) / 16.0)
    a1, a2, info = lapack.dtpmqrt(0, V, T, A1.copy(order="F"), A2.copy(order="F"),
                                  side="L", trans="T")
    assert info == 0
    g["tsmqr_big_A1"], g["tsmqr_big_A2"], g["tsmqr_big_V"], g["tsmqr_big_T"] = A1, A2, V, T
    g["tsmqr_big_outA1"], g["tsmqr_big_outA2"] = F(a1), F(a2)
    # unmqr (test/unmqr.jl:1-79, m, n, k, ib = 64, 48, 32, 8) vs dgemqrt.
    m, n, k, ib = 64, 48, 32, 8
    Aq = F(rng.random((m, k)))
    aq, tq, info = lapack.dgeqrt(ib, Aq.copy(order="F"))
    assert info == 0
    g["unmqr_Aqr"], g["unmqr_T"] = F(aq), F(tq)
    for side in "LR":
        for trans in "NC":
            C = F(rng.random((m, n) if side == "L" else (n, m)))
            c, info = lapack.dgemqrt(aq, tq, C.copy(order="F"), side=side,
                                     trans="T" if trans == "C" else "N")
            assert info == 0
            g[f"unmqr_{side}{trans}_C"], g[f"unmqr_{side}{trans}_out"] = C, F(c)
    # larfg (test/larfg.jl:56-79) vs dlarfg.
    for n in (2, 7, 33, 256):
        x = rng.standard_normal(n)
        alpha, xo, tau = lapack.dlarfg(n, x[0], x[1:].copy())
        g[f"larfg_{n}_x"] = x
        g[f"larfg_{n}_out"] = np.concatenate([[alpha], xo, [tau]])
    # ttqrt (test/ttqrt.jl:6-11 shapes, A1, A2 = triu(randn) + 2I) vs dtpqrt(l = n, nb = ib);
    # appended after the vectors above so their random streams are unchanged.
    for (n, ib) in [(16, 4), (24, 8), (32, 8), (48, 16), (256, 32)]:
        A1 = Q24(np.triu(rng.standard_normal((n, n))) + 2.0 * np.eye(n))
        A2 = Q24(np.triu(rng.standard_normal((n, n))) + 2.0 * np.eye(n))
        a1, a2, t, info = lapack.dtpqrt(n, ib, A1.copy(order="F"), A2.copy(order="F"))
        assert info == 0
        key = f"ttqrt_{n}_{ib}"
        g[key + "_A1"], g[key + "_A2"] = A1, A2
        g[key + "_outA1"], g[key + "_outA2"], g[key + "_outT"] = F(a1), F(a2), F(t)
        # the Q of that factorisation applied to a random pair (ttmqr 'L', both
        # trans) vs dtpmqrt(l = n)
        for trans in "NC":
            C1 = Q24(rng.standard_normal((n, 40)))
            C2 = Q24(rng.standard_normal((n, 40)))
            c1, c2, info = lapack.dtpmqrt(n, F(a2), F(t), C1.copy(order="F"), C2.copy(order="F"),
                                          side="L", trans="T" if trans == "C" else "N")
            assert info == 0
            g[f"{key}_L{trans}_C1"], g[f"{key}_L{trans}_C2"] = C1, C2
            g[f"{key}_L{trans}_out1"], g[f"{key}_L{trans}_out2"] = F(c1), F(c2)
    # ttmqr (test/ttmqr.jl:6-37: n = 24, k = 16, ib = 8, V = triu(randn(n, k)),
    # T = triu(rand(ib, k))) vs dtpmqrt(l = 0), all four side x trans forms.
    for side in "LR":
        for trans in "NC":
            n, k, ib = 24, 16, 8
            A1 = F(rng.standard_normal((n, n)))
            A2 = F(rng.standard_normal((n, n)))
            V = F(np.triu(rng.standard_normal((n, k))))
            T = F(np.triu(rng.random((ib, k))))
            out1 = A1.copy(order="F")
            sub = out1[:k] if side == "L" else out1[:, :k]
            a1, a2, info = lapack.dtpmqrt(0, V, T, F(sub), A2.copy(order="F"), side=side,
                                          trans="T" if trans == "C" else "N")
            assert info == 0
            if side == "L":
                out1[:k] = a1
            else:
                out1[:, :k] = a1
            key = f"ttmqr_{side}{trans}"
            g[key + "_A1"], g[key + "_A2"], g[key + "_V"], g[key + "_T"] = A1, A2, V, T
            g[key + "_outA1"], g[key + "_outA2"] = F(out1), F(a2)
    complex_vectors(rng, g)
    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
