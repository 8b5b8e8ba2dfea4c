/*
 * nextla_oracle_z.c -- CPU restatement of NextLA.jl's tile-QR kernels for
 * complex elements (ComplexF64; ComplexF32 results are checked against it).
 *
 * TEST INFRASTRUCTURE ONLY, like nextla_oracle.c (same library, same rules):
 * only the tests, the smoke check and the benchmark's CPU-baseline leg load
 * it; nothing in the product links it or falls back to it.
 *
 * The routines follow the reference's complex branches:
 *   - Householder (src/geqr2.jl:38-68, src/tsqrt.jl:52-73, src/ttqrt.jl:12-31):
 *     xnorm^2 = sum |x|^2; no reflector only when xnorm == 0 AND imag(alpha)
 *     == 0; beta = -copysign(sqrt(re^2 + im^2 + xnorm^2), re(alpha)) (real);
 *     tau = ((beta - re)/beta, -im/beta); x *= conj(alpha - beta)/|alpha - beta|^2.
 *   - the rank-1 updates apply H^H = I - conj(tau) v v^H (geqr2.jl:78-99,
 *     tsqrt.jl:77-100);
 *   - larft's V^H v products conjugate the left factor (larft.jl:71-84,
 *     larft.jl:146-158); larfb / parfb / pamm use V^H, T^H and C^H where the
 *     real code transposes (larfb.jl:61-141, parfb.jl:95-99, pamm.jl:97-127).
 * geqr2 keeps the reference's "len <= 1 => tau = 0" rule (geqr2.jl:32-35):
 * with m <= n the last diagonal entry of R can stay complex, where LAPACK's
 * zgeqrt2 makes it real with one more (1-element) reflector.
 *
 * 'T' is accepted wherever the reference accepts it and acts as 'C'
 * (src/tsmqr.jl:20).  Argument errors return -i as in nextla_oracle.c.
 */
#include <complex.h>
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

typedef double complex zc;

#define IDX(i, j, ld) ((size_t)(j) * (size_t)(ld) + (size_t)(i))

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* Householder scalars of (alpha, x) in the reference's complex convention.
   Returns 0 when no reflector is generated (tau = 0). */
static int zhouse(zc alpha, double xnorm_sq, double *beta, zc *tau, zc *scale)
{
    double ar = creal(alpha), ai = cimag(alpha);
    double xnorm = sqrt(xnorm_sq);
    if (xnorm == 0.0 && ai == 0.0) return 0;
    double b = -copysign(sqrt(ar * ar + ai * ai + xnorm_sq), ar);
    *beta = b;
    *tau = CMPLX((b - ar) / b, -ai / b);
    double dr = ar - b, di = ai;
    double abs2 = dr * dr + di * di;
    *scale = CMPLX(dr / abs2, -di / abs2);
    return 1;
}

static zc zmul(zc a, zc b)      /* plain (a.re b.re - a.im b.im, ...) product */
{
    double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
    return CMPLX(ar * br - ai * bi, ar * bi + ai * br);
}

/* ------------------------------------------------------------------------ */
/* geqr2 (src/geqr2.jl:23-105)                                               */
/* ------------------------------------------------------------------------ */
int ora_zgeqr2(int m, int n, zc *A, int lda, zc *tau, zc *work)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (m == 0 || n == 0) return 0;
    int k = imin(m, n);
    for (int i = 0; i < k; ++i) {
        int len = m - i;
        if (len <= 1) { tau[i] = 0.0; continue; }           /* geqr2.jl:32-35 */
        zc alpha = A[IDX(i, i, lda)];
        double xnorm_sq = 0.0;
        for (int p = 1; p < len; ++p) {
            zc vp = A[IDX(i + p, i, lda)];
            xnorm_sq += creal(vp) * creal(vp) + cimag(vp) * cimag(vp);
        }
        double beta;
        zc tv, scale;
        if (!zhouse(alpha, xnorm_sq, &beta, &tv, &scale)) { tau[i] = 0.0; continue; }
        for (int p = 1; p < len; ++p) A[IDX(i + p, i, lda)] = zmul(A[IDX(i + p, i, lda)], scale);
        A[IDX(i, i, lda)] = beta;
        tau[i] = tv;
        if (i < n - 1) {                                    /* geqr2.jl:76-102 */
            A[IDX(i, i, lda)] = 1.0;
            int nr = len, nc = n - i - 1;
            for (int j = 1; j <= nc; ++j) {                 /* w = C^H v */
                zc wj = 0.0;
                for (int p = 0; p < nr; ++p)
                    wj += zmul(conj(A[IDX(i + p, i + j, lda)]), A[IDX(i + p, i, lda)]);
                work[j - 1] = wj;
            }
            zc tc = conj(tv);
            for (int j = 1; j <= nc; ++j) {                 /* C -= conj(tau) v w^H */
                zc wc = conj(work[j - 1]);
                for (int p = 0; p < nr; ++p)
                    A[IDX(i + p, i + j, lda)] -= zmul(zmul(tc, A[IDX(i + p, i, lda)]), wc);
            }
            A[IDX(i, i, lda)] = beta;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* larft (src/larft.jl:48-203), all four direct / storev forms               */
/* ------------------------------------------------------------------------ */
int ora_zlarft(char direct, char storev, int n, int k, const zc *V, int ldv,
               const zc *tau, zc *T, int ldt)
{
    if (n == 0) return 0;
    if (direct != 'F' && direct != 'B') return -1;
    if (storev != 'C' && storev != 'R') return -2;
    zc *work = (zc *)malloc(sizeof(zc) * (size_t)imax(k, 1));
    if (!work) return -100;
#define Vc(r, c) V[IDX(r, c, ldv)]
#define Tm(r, c) T[IDX(r, c, ldt)]
    if (direct == 'F') {
        int prevlastv = n - 1;
        for (int i = 0; i < k; ++i) {
            prevlastv = imax(prevlastv, i);
            zc ti = tau[i];
            if (ti == 0.0) {
                for (int j = 0; j <= i; ++j) Tm(j, i) = 0.0;
                continue;
            }
            int lastv, j;
            if (storev == 'C') {                            /* larft.jl:63-86 */
                lastv = n - 1;
                while (lastv >= i + 1 && Vc(lastv, i) == 0.0) lastv--;
                j = imin(lastv, prevlastv);
                for (int p = 0; p < i; ++p) Tm(p, i) = zmul(-ti, conj(Vc(i, p)));
                if (i + 1 <= j) {
                    for (int p = 0; p < i; ++p) {
                        zc acc = 0.0;
                        for (int r = i + 1; r <= j; ++r) acc += zmul(conj(Vc(r, p)), Vc(r, i));
                        Tm(p, i) += zmul(-ti, acc);
                    }
                }
            } else {                                        /* larft.jl:87-111 */
                lastv = n - 1;
                while (lastv >= i + 1 && Vc(i, lastv) == 0.0) lastv--;
                j = imin(lastv, prevlastv);
                for (int p = 0; p < i; ++p) Tm(p, i) = zmul(-ti, Vc(p, i));
                if (i > 0 && i + 1 <= j) {
                    for (int p = 0; p < i; ++p) {
                        zc acc = 0.0;
                        for (int r = i + 1; r <= j; ++r) acc += zmul(Vc(p, r), conj(Vc(i, r)));
                        Tm(p, i) += zmul(-ti, acc);
                    }
                }
            }
            prevlastv = (i > 0) ? imax(prevlastv, lastv) : lastv;
            for (int p = 0; p < i; ++p) work[p] = Tm(p, i);
            for (int p = 0; p < i; ++p) {
                zc acc = 0.0;
                for (int q = p; q < i; ++q) acc += zmul(Tm(p, q), work[q]);
                Tm(p, i) = acc;
            }
            Tm(i, i) = ti;
        }
    } else {                                                /* larft.jl:127-202 */
        int prevlastv = 0;
        for (int i = k - 1; i >= 0; --i) {
            zc ti = tau[i];
            if (ti == 0.0) {
                for (int j = i; j < k; ++j) Tm(j, i) = 0.0;
                continue;
            }
            if (i < k - 1) {
                int lastv, j;
                lastv = 0;
                while (lastv <= i - 1 && Vc(lastv, i) == 0.0) lastv++;
                j = imax(lastv, prevlastv);
                if (storev == 'C') {
                    for (int p = i + 1; p < k; ++p) Tm(p, i) = zmul(-ti, conj(Vc(n - k + i, p)));
                    if (j <= n - k + i) {
                        for (int p = i + 1; p < k; ++p) {
                            zc acc = 0.0;
                            for (int r = j; r <= n - k + i; ++r) acc += zmul(conj(Vc(r, p)), Vc(r, k - 1));
                            Tm(p, i) += zmul(-ti, acc);
                        }
                    }
                } else {
                    for (int p = i + 1; p < k; ++p) Tm(p, i) = zmul(-ti, Vc(p, n - k + i));
                    if (i + 1 <= k - 1 && j <= n - k + i - 1) {
                        for (int p = i + 1; p < k; ++p) {
                            zc acc = 0.0;
                            for (int r = j; r <= n - k + i - 1; ++r) acc += zmul(Vc(p, r), conj(Vc(i, r)));
                            Tm(p, i) += zmul(-ti, acc);
                        }
                    }
                }
                prevlastv = (i > 0) ? imin(prevlastv, lastv) : lastv;
                for (int p = i + 1; p < k; ++p) work[p] = Tm(p, i);
                for (int p = i + 1; p < k; ++p) {
                    zc acc = 0.0;
                    for (int q = i + 1; q <= p; ++q) acc += zmul(Tm(p, q), work[q]);
                    Tm(p, i) = acc;
                }
            }
            Tm(i, i) = ti;
        }
    }
#undef Vc
#undef Tm
    free(work);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* larfb, forward columnwise (src/larfb.jl:37-142).  W: n-by-k (L), m-by-k (R) */
/* ------------------------------------------------------------------------ */
int ora_zlarfb(char side, char trans, char direct, char storev, int m, int n, int k,
               const zc *V, int ldv, const zc *T, int ldt, zc *C, int ldc, zc *W, int ldw)
{
    if (m <= 0 || n <= 0 || k <= 0) return 0;
    if (storev != 'C' || direct != 'F') return -3;
    if (side != 'L' && side != 'R') return -1;
    if (trans != 'N' && trans != 'C' && trans != 'T') return -2;
#define Vm(r, c) V[IDX(r, c, ldv)]
#define Tm(r, c) T[IDX(r, c, ldt)]
#define Cm(r, c) C[IDX(r, c, ldc)]
#define Wm(r, c) W[IDX(r, c, ldw)]
    int L = (side == 'L');
    int rows = L ? n : m;
    int len = L ? m : n;
    zc *tmp = (zc *)malloc(sizeof(zc) * (size_t)k);
    if (!tmp) return -100;
    /* W := C1^H (L) or C1 (R) */
    for (int p = 0; p < k; ++p)
        for (int r = 0; r < rows; ++r) Wm(r, p) = L ? conj(Cm(p, r)) : Cm(r, p);
    /* W := W V1 */
    for (int r = 0; r < rows; ++r) {
        for (int p = 0; p < k; ++p) {
            zc acc = Wm(r, p);
            for (int q = p + 1; q < k; ++q) acc += zmul(Wm(r, q), Vm(q, p));
            tmp[p] = acc;
        }
        for (int p = 0; p < k; ++p) Wm(r, p) = tmp[p];
    }
    /* W += C2^H V2 (L) or C2 V2 (R) */
    if (len > k) {
        for (int p = 0; p < k; ++p)
            for (int r = 0; r < rows; ++r) {
                zc acc = 0.0;
                for (int q = k; q < len; ++q) acc += zmul(L ? conj(Cm(q, r)) : Cm(r, q), Vm(q, p));
                Wm(r, p) += acc;
            }
    }
    /* W := W T^H or W T (larfb.jl:79-85, 120-126) */
    int useTH = L ? (trans == 'N') : (trans != 'N');
    for (int r = 0; r < rows; ++r) {
        for (int p = 0; p < k; ++p) {
            zc acc = 0.0;
            if (useTH) { for (int q = p; q < k; ++q) acc += zmul(Wm(r, q), conj(Tm(p, q))); }
            else       { for (int q = 0; q <= p; ++q) acc += zmul(Wm(r, q), Tm(q, p)); }
            tmp[p] = acc;
        }
        for (int p = 0; p < k; ++p) Wm(r, p) = tmp[p];
    }
    /* C2 -= V2 W^H (L) or W V2^H (R) */
    if (len > k) {
        for (int q = k; q < len; ++q)
            for (int r = 0; r < rows; ++r) {
                zc acc = 0.0;
                if (L) { for (int p = 0; p < k; ++p) acc += zmul(Vm(q, p), conj(Wm(r, p))); Cm(q, r) -= acc; }
                else   { for (int p = 0; p < k; ++p) acc += zmul(Wm(r, p), conj(Vm(q, p))); Cm(r, q) -= acc; }
            }
    }
    /* W := W V1^H */
    for (int r = 0; r < rows; ++r) {
        for (int p = 0; p < k; ++p) {
            zc acc = Wm(r, p);
            for (int q = 0; q < p; ++q) acc += zmul(Wm(r, q), conj(Vm(p, q)));
            tmp[p] = acc;
        }
        for (int p = 0; p < k; ++p) Wm(r, p) = tmp[p];
    }
    /* C1 -= W^H (L) or W (R) */
    for (int p = 0; p < k; ++p)
        for (int r = 0; r < rows; ++r) {
            if (L) Cm(p, r) -= conj(Wm(r, p)); else Cm(r, p) -= Wm(r, p);
        }
#undef Vm
#undef Tm
#undef Cm
#undef Wm
    free(tmp);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* geqrt (src/geqrt.jl:22-68)                                                */
/* ------------------------------------------------------------------------ */
int ora_zgeqrt(int m, int n, int ib, zc *A, int lda, zc *T, int ldt, zc *tau, zc *work)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (ib < 0 || (ib == 0 && m > 0 && n > 0)) return -3;
    if (m == 0 || n == 0 || ib == 0) return 0;
    int k = imin(m, n);
    for (int i = 0; i < k; i += ib) {
        int sb = imin(ib, k - i);
        zc *av = A + IDX(i, i, lda);
        zc *tv = T + IDX(0, i, ldt);
        ora_zgeqr2(m - i, sb, av, lda, tau + i, work);
        ora_zlarft('F', 'C', m - i, sb, av, lda, tau + i, tv, ldt);
        if (n >= i + sb + 1) {
            int nw = n - i - sb;
            ora_zlarfb('L', 'C', 'F', 'C', m - i, nw, sb, av, lda, tv, ldt,
                       A + IDX(i, i + sb, lda), lda, work, nw);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* unmqr (src/unmqr.jl:52-149)                                               */
/* ------------------------------------------------------------------------ */
int ora_zunmqr(char side, char trans, int m, int n, int k, int ib, const zc *A, int lda,
               int arows, int kcols, const zc *T, int ldt, zc *C, int ldc, zc *work, int ldwork)
{
    if (side != 'L' && side != 'R') return -1;
    int nq = (side == 'L') ? m : n;
    if (trans != 'N' && trans != 'C' && trans != 'T') return -2;
    if (m < 0) return -3;
    if (n < 0) return -4;
    if (k < 0) return -5;
    k = imin(imin(k, nq), kcols);
    if (ib < 0) return -6;
    if (lda < imax(1, nq) && nq > 0) return -8;
    if (m == 0 || n == 0 || k == 0) return 0;
    int fwd = (side == 'L' && trans != 'N') || (side == 'R' && trans == 'N');
    int i1 = fwd ? 0 : ((k - 1) / ib) * ib, i3 = fwd ? ib : -ib;
    int nblk = (k - 1) / ib + 1;
    for (int b = 0, i = i1; b < nblk; ++b, i += i3) {
        int kb = imin(ib, k - i);
        int mi = m, ni = n, ic = 0, jc = 0;
        if (side == 'L') { mi = m - i; ic = i; } else { ni = n - i; jc = i; }
        ora_zlarfb(side, trans, 'F', 'C', mi, ni, kb, A + IDX(i, i, lda), lda,
                   T + IDX(0, i, ldt), ldt, C + IDX(ic, jc, ldc), ldc, work, ldwork);
        (void)arows;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* parfb / pamm, columnwise forward, with a trapezoidal part of order l     */
/* (src/parfb.jl:121-137, src/pamm.jl:97-175, 301-368)                      */
/* ------------------------------------------------------------------------ */
static zc zvtrap(const zc *V, int ldv, int r, int p, int mv, int l)
{
    if (p < l && r >= mv - l && r - (mv - l) > p) return 0.0;
    return V[IDX(r, p, ldv)];
}

static void zparfb_lv(char side, char trans, int m2, int n2, int k, int l,
                      zc *A1, int lda1, zc *A2, int lda2,
                      const zc *V, int ldv, const zc *T, int ldt, zc *W, int ldw)
{
#define A1m(r, c) A1[IDX(r, c, lda1)]
#define A2m(r, c) A2[IDX(r, c, lda2)]
#define Vm(r, c) zvtrap(V, ldv, r, c, side == 'L' ? m2 : n2, l)
#define Tm(r, c) T[IDX(r, c, ldt)]
#define Wm(r, c) W[IDX(r, c, ldw)]
    int tr = (trans != 'N');
    zc *tmp = (zc *)malloc(sizeof(zc) * (size_t)k);
    if (side == 'L') {
        /* W = V^H A2 + A1 */
        for (int c = 0; c < n2; ++c)
            for (int p = 0; p < k; ++p) {
                zc acc = 0.0;
                for (int r = 0; r < m2; ++r) acc += zmul(conj(Vm(r, p)), A2m(r, c));
                Wm(p, c) = acc;
            }
        for (int p = 0; p < k; ++p)
            for (int c = 0; c < n2; ++c) Wm(p, c) += A1m(p, c);
        /* W = op(T) W */
        for (int c = 0; c < n2; ++c) {
            for (int p = 0; p < k; ++p) {
                zc acc = 0.0;
                if (!tr) { for (int q = p; q < k; ++q) acc += zmul(Tm(p, q), Wm(q, c)); }
                else     { for (int q = 0; q <= p; ++q) acc += zmul(conj(Tm(q, p)), Wm(q, c)); }
                tmp[p] = acc;
            }
            for (int p = 0; p < k; ++p) Wm(p, c) = tmp[p];
        }
        for (int p = 0; p < k; ++p)
            for (int c = 0; c < n2; ++c) A1m(p, c) -= Wm(p, c);
        /* A2 -= V W */
        for (int c = 0; c < n2; ++c)
            for (int r = 0; r < m2; ++r) {
                zc acc = 0.0;
                for (int p = 0; p < k; ++p) acc += zmul(Vm(r, p), Wm(p, c));
                A2m(r, c) -= acc;
            }
    } else {
        /* W = A2 V + A1 */
        for (int p = 0; p < k; ++p)
            for (int r = 0; r < m2; ++r) {
                zc acc = 0.0;
                for (int c = 0; c < n2; ++c) acc += zmul(A2m(r, c), Vm(c, p));
                Wm(r, p) = acc;
            }
        for (int p = 0; p < k; ++p)
            for (int r = 0; r < m2; ++r) Wm(r, p) += A1m(r, p);
        /* W = W op(T) */
        for (int r = 0; r < m2; ++r) {
            for (int p = 0; p < k; ++p) {
                zc acc = 0.0;
                if (!tr) { for (int q = 0; q <= p; ++q) acc += zmul(Wm(r, q), Tm(q, p)); }
                else     { for (int q = p; q < k; ++q) acc += zmul(Wm(r, q), conj(Tm(p, q))); }
                tmp[p] = acc;
            }
            for (int p = 0; p < k; ++p) Wm(r, p) = tmp[p];
        }
        for (int p = 0; p < k; ++p)
            for (int r = 0; r < m2; ++r) A1m(r, p) -= Wm(r, p);
        /* A2 -= W V^H */
        for (int c = 0; c < n2; ++c)
            for (int r = 0; r < m2; ++r) {
                zc acc = 0.0;
                for (int p = 0; p < k; ++p) acc += zmul(Wm(r, p), conj(Vm(c, p)));
                A2m(r, c) -= acc;
            }
    }
    free(tmp);
#undef A1m
#undef A2m
#undef Vm
#undef Tm
#undef Wm
}

int ora_zparfb(char side, char trans, int m1, int n1, int m2, int n2, int k,
               zc *A1, int lda1, zc *A2, int lda2, const zc *V, int ldv,
               const zc *T, int ldt, zc *W, int ldw)
{
    if (side != 'L' && side != 'R') return -1;              /* parfb.jl:47-85 */
    if (trans != 'N' && trans != 'C' && trans != 'T') return -2;
    if (m1 < 0) return -3;
    if (n1 < 0) return -4;
    if (m2 < 0 || (side == 'R' && m1 != m2)) return -5;
    if (n2 < 0 || (side == 'L' && n1 != n2)) return -6;
    if (k < 0) return -7;
    if (m1 == 0 || n1 == 0 || n2 == 0 || k == 0 || m2 == 0) return 0;
    zparfb_lv(side, trans, m2, n2, k, 0, A1, lda1, A2, lda2, V, ldv, T, ldt, W, ldw);
    return 0;
}

int ora_zparfb_l(char side, char trans, int m1, int n1, int m2, int n2, int k, int l,
                 zc *A1, int lda1, zc *A2, int lda2, const zc *V, int ldv,
                 const zc *T, int ldt, zc *W, int ldw)
{
    if (side != 'L' && side != 'R') return -1;
    if (trans != 'N' && trans != 'C' && trans != 'T') return -2;
    if (m1 < 0) return -3;
    if (n1 < 0) return -4;
    if (m2 < 0 || (side == 'R' && m1 != m2)) return -5;
    if (n2 < 0 || (side == 'L' && n1 != n2)) return -6;
    if (k < 0) return -7;
    if (l < 0 || l > k) return -8;
    if (m1 == 0 || n1 == 0 || n2 == 0 || k == 0 || m2 == 0) return 0;
    zparfb_lv(side, trans, m2, n2, k, l, A1, lda1, A2, lda2, V, ldv, T, ldt, W, ldw);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* tsmqr (src/tsmqr.jl:47-146)                                               */
/* ------------------------------------------------------------------------ */
int ora_ztsmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib,
               int kstored, zc *A1, int lda1, zc *A2, int lda2,
               const zc *V, int ldv, const zc *T, int ldt, zc *work)
{
    if (side != 'L' && side != 'R') return -1;
    if (trans != 'N' && trans != 'C' && trans != 'T') return -2;
    if (m1 < 0) return -3;
    if (n1 < 0) return -4;
    if (m2 < 0 || (m2 != m1 && side == 'R')) return -5;
    if (n2 < 0 || (n2 != n1 && side == 'L')) return -6;
    if (k < 0) return -7;
    if (ib < 0) return -8;
    k = imin(imin(k, side == 'L' ? m1 : n1), kstored);
    if (m1 == 0 || n1 == 0 || m2 == 0 || n2 == 0 || k == 0 || ib == 0) return 0;
    int fwd = (side == 'L' && trans != 'N') || (side == 'R' && trans == 'N');
    int i1 = fwd ? 0 : ((k - 1) / ib) * ib, i3 = fwd ? ib : -ib;
    int nblk = (k - 1) / ib + 1;
    for (int b = 0, i = i1; b < nblk; ++b, i += i3) {
        int kb = imin(ib, k - i);
        if (side == 'L')
            zparfb_lv('L', trans, m2, n2, kb, 0, A1 + IDX(i, 0, lda1), lda1, A2, lda2,
                      V + IDX(0, i, ldv), ldv, T + IDX(0, i, ldt), ldt, work, kb);
        else
            zparfb_lv('R', trans, m2, n2, kb, 0, A1 + IDX(0, i, lda1), lda1, A2, lda2,
                      V + IDX(0, i, ldv), ldv, T + IDX(0, i, ldt), ldt, work, m1);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* tsqrt (src/tsqrt.jl:46-156) and ttqrt (src/ttqrt.jl:1-119): one loop     */
/* with the triangle's row bound tri (0: tsqrt, 1: ttqrt, column r's        */
/* reflector then uses A2 rows [0, min(r + 1, m)), and the T products only  */
/* the rows both reflectors occupy).                                         */
/* ------------------------------------------------------------------------ */
static int zts_tt_qrt(int tri, int m, int n, int ib, int m1, zc *A1, int lda1, zc *A2, int lda2,
                      zc *T, int ldt, zc *tau, zc *work)
{
    int k = tri ? imin(m, n) : imin(m1, n);
    if (m == 0 || n == 0 || ib == 0 || k == 0) return 0;
#define A1m(r, c) A1[IDX(r, c, lda1)]
#define A2m(r, c) A2[IDX(r, c, lda2)]
#define Tm(r, c) T[IDX(r, c, ldt)]
    for (int ii = 0; ii < k; ii += ib) {
        int sb = imin(k - ii, ib);
        for (int i = 0; i < sb; ++i) {
            int r = ii + i;
            int mi = tri ? imin(r + 1, m) : m;
            zc alpha = A1m(r, r);
            double xnorm_sq = 0.0;
            for (int p = 0; p < mi; ++p) {
                zc vp = A2m(p, r);
                xnorm_sq += creal(vp) * creal(vp) + cimag(vp) * cimag(vp);
            }
            double beta;
            zc tv, scale;
            if (!zhouse(alpha, xnorm_sq, &beta, &tv, &scale)) { tau[r] = 0.0; continue; }
            for (int p = 0; p < mi; ++p) A2m(p, r) = zmul(A2m(p, r), scale);
            A1m(r, r) = beta;
            tau[r] = tv;
            if ((sb - i - 1) > 0 && (r + 1) < n) {          /* tsqrt.jl:77-100 */
                int ncc = sb - i - 1;
                zc tc = conj(tv);
                for (int j = 1; j <= ncc; ++j) {
                    zc wj = conj(A1m(r, r + j));
                    for (int p = 0; p < mi; ++p) wj += zmul(conj(A2m(p, r + j)), A2m(p, r));
                    work[j - 1] = conj(wj);
                }
                for (int j = 1; j <= ncc; ++j) A1m(r, r + j) -= zmul(tc, work[j - 1]);
                for (int j = 1; j <= ncc; ++j) {
                    zc wj = work[j - 1];
                    for (int p = 0; p < mi; ++p) A2m(p, r + j) -= zmul(zmul(tc, A2m(p, r)), wj);
                }
            }
            if (i > 0) {                                    /* tsqrt.jl:103-122 */
                for (int p = 0; p < i; ++p) {
                    int mq = tri ? imin(ii + p + 1, m) : m;
                    zc acc = 0.0;
                    for (int q = 0; q < mq; ++q) acc += zmul(conj(A2m(q, ii + p)), A2m(q, r));
                    Tm(p, r) = zmul(-tv, acc);
                }
                for (int p = 0; p < i; ++p) work[p] = Tm(p, r);
                for (int p = 0; p < i; ++p) {
                    zc acc = 0.0;
                    for (int q = p; q < i; ++q) acc += zmul(Tm(p, ii + q), work[q]);
                    Tm(p, r) = acc;
                }
            }
            Tm(i, r) = tv;
        }
        if (n > ii + sb) {
            int ni = n - (ii + sb);
            if (!tri) {
                ora_ztsmqr('L', 'C', sb, ni, m, ni, sb, ib, sb, A1 + IDX(ii, ii + sb, lda1), lda1,
                           A2 + IDX(0, ii + sb, lda2), lda2, A2 + IDX(0, ii, lda2), lda2,
                           T + IDX(0, ii, ldt), ldt, work);
            } else {
                int mi2 = imin(ii + sb, m);
                int l = imin(sb, imax(0, mi2 - ii));
                zparfb_lv('L', 'C', mi2, ni, sb, l, A1 + IDX(ii, ii + sb, lda1), lda1,
                          A2 + IDX(0, ii + sb, lda2), lda2, A2 + IDX(0, ii, lda2), lda2,
                          T + IDX(0, ii, ldt), ldt, work, sb);
            }
        }
    }
#undef A1m
#undef A2m
#undef Tm
    return 0;
}

int ora_ztsqrt(int m, int n, int ib, int m1, zc *A1, int lda1, zc *A2, int lda2,
               zc *T, int ldt, zc *tau, zc *work)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (ib < 0) return -3;
    return zts_tt_qrt(0, m, n, ib, m1, A1, lda1, A2, lda2, T, ldt, tau, work);
}

int ora_zttqrt(int m, int n, int ib, zc *A1, int lda1, zc *A2, int lda2,
               zc *T, int ldt, zc *tau, zc *work)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (ib < 0) return -3;
    return zts_tt_qrt(1, m, n, ib, 0, A1, lda1, A2, lda2, T, ldt, tau, work);
}

/* ------------------------------------------------------------------------ */
/* ttmqr (src/ttmqr.jl:1-95), the block row bound of nextla_oracle.c        */
/* ------------------------------------------------------------------------ */
int ora_zttmqr(char side, char trans, int m1, int n1, int m2, int n2, int k, int ib,
               zc *A1, int lda1, zc *A2, int lda2, const zc *V, int ldv,
               const zc *T, int ldt, zc *work)
{
    if (side != 'L' && side != 'R') return -1;
    if (trans != 'N' && trans != 'C' && trans != 'T') return -2;
    if (m1 < 0) return -3;
    if (n1 < 0) return -4;
    if (m2 < 0 || (m2 != m1 && side == 'R')) return -5;
    if (n2 < 0 || (n2 != n1 && side == 'L')) return -6;
    if (k < 0) return -7;
    k = imin(k, side == 'L' ? m1 : n1);
    if (ib < 0) return -8;
    if (m1 == 0 || n1 == 0 || m2 == 0 || n2 == 0 || k == 0 || ib == 0) return 0;
    int fwd = (side == 'L' && trans != 'N') || (side == 'R' && trans == 'N');
    int i1 = fwd ? 0 : ((k - 1) / ib) * ib, i3 = fwd ? ib : -ib;
    int nblk = (k - 1) / ib + 1;
    for (int b = 0, i = i1; b < nblk; ++b, i += i3) {
        int kb = imin(ib, k - i);
        if (side == 'L') {
            int mi2 = imin(i + kb, m2);
            int l = imin(kb, imax(0, mi2 - i));
            zparfb_lv('L', trans, mi2, n2, kb, l, A1 + IDX(i, 0, lda1), lda1, A2, lda2,
                      V + IDX(0, i, ldv), ldv, T + IDX(0, i, ldt), ldt, work, kb);
        } else {
            int ni2 = imin(i + kb, n2);
            int l = imin(kb, imax(0, ni2 - i));
            zparfb_lv('R', trans, m2, ni2, kb, l, A1 + IDX(0, i, lda1), lda1, A2, lda2,
                      V + IDX(0, i, ldv), ldv, T + IDX(0, i, ldt), ldt, work, m1);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Flat-tree tile QR and its Q application: the driver of nextla_oracle.c  */
/* (geqrt, unmqr, tsqrt, tsmqr in PLASMA order) on complex tiles; same T    */
/* and tau layouts.                                                          */
/* ------------------------------------------------------------------------ */
int ora_ztile_geqrf(int m, int n, int nb, int ib, zc *A, int lda, zc *T, int ldt,
                    zc *tau, int ldtau)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (nb <= 0) return -3;
    if (ib <= 0 || ib > nb) return -4;
    if (m == 0 || n == 0) return 0;
    int MT = (m + nb - 1) / nb, NT = (n + nb - 1) / nb;
    if (lda < m) return -6;
    if (ldt < MT * ib) return -8;
    if (ldtau < n) return -10;
    zc *work = (zc *)malloc(sizeof(zc) * (size_t)nb * (size_t)nb);
    zc *tv = (zc *)malloc(sizeof(zc) * (size_t)nb);
    if (!work || !tv) { free(work); free(tv); return -100; }
    int KT = imin(MT, NT);
    for (int k = 0; k < KT; ++k) {
        int mk = imin(nb, m - k * nb), nk = imin(nb, n - k * nb);
        zc *Akk = A + IDX(k * nb, k * nb, lda);
        zc *Tkk = T + IDX(k * ib, k * nb, ldt);
        ora_zgeqrt(mk, nk, ib, Akk, lda, Tkk, ldt, tv, work);
        for (int c = 0; c < imin(mk, nk); ++c) tau[IDX(k * nb + c, k, ldtau)] = tv[c];
#pragma omp parallel for schedule(dynamic)
        for (int j = k + 1; j < NT; ++j) {
            int nj = imin(nb, n - j * nb);
            zc *w = (zc *)malloc(sizeof(zc) * (size_t)nb * (size_t)nb);
            ora_zunmqr('L', 'C', mk, nj, imin(mk, nk), ib, Akk, lda, mk, nk, Tkk, ldt,
                       A + IDX(k * nb, j * nb, lda), lda, w, nj);
            free(w);
        }
        for (int i = k + 1; i < MT; ++i) {
            int mi = imin(nb, m - i * nb);
            zc *Aik = A + IDX(i * nb, k * nb, lda);
            zc *Tik = T + IDX(i * ib, k * nb, ldt);
            ora_ztsqrt(mi, nk, ib, mk, Akk, lda, Aik, lda, Tik, ldt, tv, work);
            for (int c = 0; c < imin(mk, nk); ++c) tau[IDX(k * nb + c, i, ldtau)] = tv[c];
#pragma omp parallel for schedule(dynamic)
            for (int j = k + 1; j < NT; ++j) {
                int nj = imin(nb, n - j * nb);
                zc *w = (zc *)malloc(sizeof(zc) * (size_t)nb * (size_t)nb);
                ora_ztsmqr('L', 'C', mk, nj, mi, nj, imin(mk, nk), ib, imin(mk, nk),
                           A + IDX(k * nb, j * nb, lda), lda, A + IDX(i * nb, j * nb, lda), lda,
                           Aik, lda, Tik, ldt, w);
                free(w);
            }
        }
    }
    free(work);
    free(tv);
    return 0;
}

int ora_ztile_unmqr(char trans, int m, int n, int nrhs, int nb, int ib, const zc *A,
                    int lda, const zc *T, int ldt, zc *B, int ldb)
{
    if (trans != 'N' && trans != 'C' && trans != 'T') return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (nrhs < 0) return -4;
    if (nb <= 0) return -5;
    if (ib <= 0 || ib > nb) return -6;
    if (m == 0 || n == 0 || nrhs == 0) return 0;
    int MT = (m + nb - 1) / nb, NT = (n + nb - 1) / nb, KT = imin(MT, NT);
    zc *work = (zc *)malloc(sizeof(zc) * (size_t)nrhs * (size_t)nb);
    if (!work) return -100;
    if (trans != 'N') {
        for (int k = 0; k < KT; ++k) {
            int mk = imin(nb, m - k * nb), nk = imin(nb, n - k * nb), kk = imin(mk, nk);
            ora_zunmqr('L', 'C', mk, nrhs, kk, ib, A + IDX(k * nb, k * nb, lda), lda, mk, nk,
                       T + IDX(k * ib, k * nb, ldt), ldt, B + IDX(k * nb, 0, ldb), ldb, work, nrhs);
            for (int i = k + 1; i < MT; ++i) {
                int mi = imin(nb, m - i * nb);
                ora_ztsmqr('L', 'C', mk, nrhs, mi, nrhs, kk, ib, kk, B + IDX(k * nb, 0, ldb), ldb,
                           B + IDX(i * nb, 0, ldb), ldb, A + IDX(i * nb, k * nb, lda), lda,
                           T + IDX(i * ib, k * nb, ldt), ldt, work);
            }
        }
    } else {
        for (int k = KT - 1; k >= 0; --k) {
            int mk = imin(nb, m - k * nb), nk = imin(nb, n - k * nb), kk = imin(mk, nk);
            for (int i = MT - 1; i > k; --i) {
                int mi = imin(nb, m - i * nb);
                ora_ztsmqr('L', 'N', mk, nrhs, mi, nrhs, kk, ib, kk, B + IDX(k * nb, 0, ldb), ldb,
                           B + IDX(i * nb, 0, ldb), ldb, A + IDX(i * nb, k * nb, lda), lda,
                           T + IDX(i * ib, k * nb, ldt), ldt, work);
            }
            ora_zunmqr('L', 'N', mk, nrhs, kk, ib, A + IDX(k * nb, k * nb, lda), lda, mk, nk,
                       T + IDX(k * ib, k * nb, ldt), ldt, B + IDX(k * nb, 0, ldb), ldb, work, nrhs);
        }
    }
    free(work);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Hierarchical / binary-tree tile QR and its Q application on complex      */
/* tiles: the driver of nextla_oracle.c (ora_dtile_geqrf_hqr: geqrt on every */
/* group leader and unmqr of its row, tsqrt/tsmqr of each other tile of the  */
/* group into its leader, the ragged last tile into the last leader, then    */
/* ttqrt/ttmqr between leaders at distances grp, 2 grp, ...), with the       */
/* complex kernels above; same T, tau, T2, tau2 layouts.  grp = 1 is the     */
/* binary tree of the TT kernels (src/ttqrt.jl:81-118, src/ttmqr.jl:1-95).   */
/* ------------------------------------------------------------------------ */
static int ztree_ragged(int m, int nb, int MT, int k, int nk)
{
    int p = MT - 1;
    return p > k && imin(nb, m - p * nb) < nk;
}

int ora_ztile_geqrf_hqr(int m, int n, int nb, int ib, int grp, zc *A, int lda, zc *T, int ldt,
                        zc *tau, int ldtau, zc *T2, zc *tau2)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (nb <= 0) return -3;
    if (ib <= 0 || ib > nb) return -4;
    if (grp <= 0) return -5;
    if (m == 0 || n == 0) return 0;
    int MT = (m + nb - 1) / nb, NT = (n + nb - 1) / nb, KT = imin(MT, NT);
    if (lda < m) return -7;
    if (ldt < MT * ib) return -9;
    if (ldtau < n) return -11;
    zc *w = (zc *)malloc(sizeof(zc) * (size_t)nb * (size_t)nb);
    zc *tv = (zc *)malloc(sizeof(zc) * (size_t)nb);
    if (!w || !tv) { free(w); free(tv); return -100; }
    for (int k = 0; k < KT; ++k) {
        int nk = imin(nb, n - k * nb);
        int rag = ztree_ragged(m, nb, MT, k, nk);
        int MTt = rag ? MT - 1 : MT;
        int last = k + ((MTt - 1 - k) / grp) * grp;
        for (int i = k; i < MTt; i += grp) {
            int mi = imin(nb, m - i * nb), kk = imin(mi, nk);
            zc *Aik = A + IDX(i * nb, k * nb, lda);
            zc *Tik = T + IDX(i * ib, k * nb, ldt);
            ora_zgeqrt(mi, nk, ib, Aik, lda, Tik, ldt, tv, w);
            for (int c = 0; c < kk; ++c) tau[IDX(k * nb + c, i, ldtau)] = tv[c];
            for (int j = k + 1; j < NT; ++j) {
                int nj = imin(nb, n - j * nb);
                ora_zunmqr('L', 'C', mi, nj, kk, ib, Aik, lda, mi, nk, Tik, ldt,
                           A + IDX(i * nb, j * nb, lda), lda, w, nj);
            }
        }
        for (int d = 1; d <= grp; ++d) {
            for (int i = k; i < MTt; i += grp) {
                int p = (d < grp) ? i + d : (rag && i == last ? MT - 1 : -1);
                if (p < 0 || (d < grp && p >= MTt)) continue;
                int mp = imin(nb, m - p * nb), mi = imin(nb, m - i * nb);
                zc *Apk = A + IDX(p * nb, k * nb, lda);
                zc *T2p = T2 + IDX(p * ib, k * nb, ldt);
                ora_ztsqrt(mp, nk, ib, mi, A + IDX(i * nb, k * nb, lda), lda, Apk, lda, T2p, ldt, tv, w);
                for (int c = 0; c < imin(mi, nk); ++c) tau2[IDX(k * nb + c, p, ldtau)] = tv[c];
                for (int j = k + 1; j < NT; ++j) {
                    int nj = imin(nb, n - j * nb);
                    ora_ztsmqr('L', 'C', mi, nj, mp, nj, imin(mi, nk), ib, imin(mi, nk),
                               A + IDX(i * nb, j * nb, lda), lda, A + IDX(p * nb, j * nb, lda), lda, Apk, lda,
                               T2p, ldt, w);
                }
            }
        }
        for (int s = grp; k + s < MTt; s *= 2) {
            for (int i = k; i < MTt - s; i += 2 * s) {
                int p = i + s;
                int mp = imin(nb, m - p * nb), kt = imin(mp, nk);
                zc *Apk = A + IDX(p * nb, k * nb, lda);
                zc *T2p = T2 + IDX(p * ib, k * nb, ldt);
                ora_zttqrt(mp, nk, ib, A + IDX(i * nb, k * nb, lda), lda, Apk, lda, T2p, ldt, tv, w);
                for (int c = 0; c < kt; ++c) tau2[IDX(k * nb + c, p, ldtau)] = tv[c];
                for (int j = k + 1; j < NT; ++j) {
                    int nj = imin(nb, n - j * nb);
                    ora_zttmqr('L', 'C', nb, nj, mp, nj, kt, ib, A + IDX(i * nb, j * nb, lda), lda,
                               A + IDX(p * nb, j * nb, lda), lda, Apk, lda, T2p, ldt, w);
                }
            }
        }
    }
    free(w);
    free(tv);
    return 0;
}

int ora_ztile_unmqr_hqr(char trans, int m, int n, int nrhs, int nb, int ib, int grp, const zc *A,
                        int lda, const zc *T, int ldt, const zc *T2, zc *B, int ldb)
{
    if (trans != 'N' && trans != 'C' && trans != 'T') return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (nrhs < 0) return -4;
    if (nb <= 0) return -5;
    if (ib <= 0 || ib > nb) return -6;
    if (grp <= 0) return -7;
    if (m == 0 || n == 0 || nrhs == 0) return 0;
    int MT = (m + nb - 1) / nb, NT = (n + nb - 1) / nb, KT = imin(MT, NT);
    zc *work = (zc *)malloc(sizeof(zc) * (size_t)nrhs * (size_t)nb);
    if (!work) return -100;
    const int tr = (trans != 'N');
    for (int kx = 0; kx < KT; ++kx) {
        int k = tr ? kx : KT - 1 - kx;
        int nk = imin(nb, n - k * nb);
        int rag = ztree_ragged(m, nb, MT, k, nk);
        int MTt = rag ? MT - 1 : MT;
        int last = k + ((MTt - 1 - k) / grp) * grp;
        int smax = grp;
        while (k + smax < MTt) smax *= 2;
#define ZGRP_MERGE(i, p, op)                                                                       \
        do {                                                                                       \
            int mi_ = imin(nb, m - (i) * nb), mp_ = imin(nb, m - (p) * nb);                        \
            ora_ztsmqr('L', op, mi_, nrhs, mp_, nrhs, imin(mi_, nk), ib, imin(mi_, nk),            \
                       B + IDX((i) * nb, 0, ldb), ldb, B + IDX((p) * nb, 0, ldb), ldb,             \
                       A + IDX((p) * nb, k * nb, lda), lda, T2 + IDX((p) * ib, k * nb, ldt), ldt,   \
                       work);                                                                      \
        } while (0)
#define ZTREE_MERGE(i, p, op)                                                                      \
        do {                                                                                       \
            int mp_ = imin(nb, m - (p) * nb);                                                      \
            ora_zttmqr('L', op, nb, nrhs, mp_, nrhs, imin(mp_, nk), ib, B + IDX((i) * nb, 0, ldb),  \
                       ldb, B + IDX((p) * nb, 0, ldb), ldb, A + IDX((p) * nb, k * nb, lda), lda,    \
                       T2 + IDX((p) * ib, k * nb, ldt), ldt, work);                                \
        } while (0)
        if (tr) {
            for (int i = k; i < MTt; i += grp) {
                int mi = imin(nb, m - i * nb);
                ora_zunmqr('L', 'C', mi, nrhs, imin(mi, nk), ib, A + IDX(i * nb, k * nb, lda), lda, mi,
                           nk, T + IDX(i * ib, k * nb, ldt), ldt, B + IDX(i * nb, 0, ldb), ldb, work, nrhs);
            }
            for (int d = 1; d < grp; ++d)
                for (int i = k; i + d < MTt; i += grp) ZGRP_MERGE(i, i + d, 'C');
            if (rag) ZGRP_MERGE(last, MT - 1, 'C');
            for (int s = grp; k + s < MTt; s *= 2)
                for (int i = k; i < MTt - s; i += 2 * s) ZTREE_MERGE(i, i + s, 'C');
        } else {
            for (int s = smax / 2; s >= grp; s /= 2)
                for (int i = k; i < MTt - s; i += 2 * s) ZTREE_MERGE(i, i + s, 'N');
            if (rag) ZGRP_MERGE(last, MT - 1, 'N');
            for (int d = grp - 1; d >= 1; --d)
                for (int i = k; i + d < MTt; i += grp) ZGRP_MERGE(i, i + d, 'N');
            for (int i = k; i < MTt; i += grp) {
                int mi = imin(nb, m - i * nb);
                ora_zunmqr('L', 'N', mi, nrhs, imin(mi, nk), ib, A + IDX(i * nb, k * nb, lda), lda, mi,
                           nk, T + IDX(i * ib, k * nb, ldt), ldt, B + IDX(i * nb, 0, ldb), ldb, work, nrhs);
            }
        }
#undef ZGRP_MERGE
#undef ZTREE_MERGE
    }
    free(work);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Upper-triangular solve R X = B with LeftUpperTRSM!'s arithmetic           */
/* (src/trsm.jl:38-63): B scaled by the diagonal first, then                 */
/* b[r] -= (A[r,i] / A[r,r]) b[i].  Complex division in Smith's scaled form  */
/* (R. L. Smith, "Algorithm 116: Complex division", CACM 5(8), 1962).        */
/* ------------------------------------------------------------------------ */
static zc zdiv(zc a, zc b)
{
    double ar = creal(a), ai = cimag(a), br = creal(b), bi = cimag(b);
    if (fabs(br) >= fabs(bi)) {
        double r = bi / br, d = br + bi * r;
        return CMPLX((ar + ai * r) / d, (ai - ar * r) / d);
    }
    double r = br / bi, d = bi + br * r;
    return CMPLX((ar * r + ai) / d, (ai * r - ar) / d);
}

int ora_ztrsm_lun(int n, int nrhs, const zc *A, int lda, zc *B, int ldb)
{
    if (n < 0) return -1;
    if (nrhs < 0) return -2;
    for (int c = 0; c < nrhs; ++c) {
        zc *b = B + IDX(0, c, ldb);
        for (int r = 0; r < n; ++r) b[r] = zdiv(b[r], A[IDX(r, r, lda)]);
        for (int i = n - 1; i >= 0; --i)
            for (int r = 0; r < i; ++r) b[r] -= zmul(zdiv(A[IDX(r, i, lda)], A[IDX(r, r, lda)]), b[i]);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* pamm for complex elements: the forms of ora_dpamm (nextla_oracle.c) with */
/* the reference's conjugations -- op 'W' conjugates Ve for (L, C) and      */
/* (R, R) (pamm.jl:120,139-153,...: 'C' / adjoint), op 'A' for (L, R) and   */
/* (R, C) (pamm.jl:330-343, 351-365, ...).                                  */
/* ------------------------------------------------------------------------ */
static int zpamm_valid(int fwd, int r, int p, int mv, int k, int l)
{
    if (fwd) return !(p < l && r >= mv - l && r - (mv - l) > p);
    return !(p >= k - l && r < l && r < p - (k - l));
}

int ora_zpamm(char op, char side, char storev, char direct, int m, int n, int k, int l,
              const zc *A1, int lda1, zc *A2, int lda2, const zc *V, int ldv, zc *W, int ldw)
{
    if (op != 'W' && op != 'A') return -1;
    if (side != 'L' && side != 'R') return -2;
    if (storev != 'C' && storev != 'R') return -3;
    if (direct != 'F' && direct != 'B') return -4;
    if (m < 0) return -5;
    if (n < 0) return -6;
    if (k < 0) return -7;
    if (l < 0) return -8;
    if (m == 0 || n == 0 || k == 0) return 0;
    int L = (side == 'L'), C = (storev == 'C'), fwd = (direct == 'F');
    int mv = L ? m : n;
    if (l > k || l > mv) return -8;
    int cjw = (L && C) || (!L && !C), cja = (L && !C) || (!L && C);
#define VE(r, p) (C ? V[IDX(r, p, ldv)] : V[IDX(p, r, ldv)])
    if (op == 'W') {
        if (L) {
            for (int c = 0; c < n; ++c)
                for (int p = 0; p < k; ++p) {
                    zc acc = 0.0;
                    for (int r = 0; r < m; ++r)
                        if (zpamm_valid(fwd, r, p, mv, k, l))
                            acc += zmul(cjw ? conj(VE(r, p)) : VE(r, p), A2[IDX(r, c, lda2)]);
                    W[IDX(p, c, ldw)] = A1[IDX(p, c, lda1)] + acc;
                }
        } else {
            for (int p = 0; p < k; ++p)
                for (int i = 0; i < m; ++i) {
                    zc acc = 0.0;
                    for (int c = 0; c < n; ++c)
                        if (zpamm_valid(fwd, c, p, mv, k, l))
                            acc += zmul(A2[IDX(i, c, lda2)], cjw ? conj(VE(c, p)) : VE(c, p));
                    W[IDX(i, p, ldw)] = A1[IDX(i, p, lda1)] + acc;
                }
        }
        return 0;
    }
    if (L) {
        for (int c = 0; c < n; ++c)
            for (int r = 0; r < m; ++r) {
                zc acc = 0.0;
                for (int p = 0; p < k; ++p)
                    if (zpamm_valid(fwd, r, p, mv, k, l))
                        acc += zmul(cja ? conj(VE(r, p)) : VE(r, p), W[IDX(p, c, ldw)]);
                A2[IDX(r, c, lda2)] -= acc;
            }
    } else {
        for (int c = 0; c < n; ++c)
            for (int i = 0; i < m; ++i) {
                zc acc = 0.0;
                for (int p = 0; p < k; ++p)
                    if (zpamm_valid(fwd, c, p, mv, k, l))
                        acc += zmul(W[IDX(i, p, ldw)], cja ? conj(VE(c, p)) : VE(c, p));
                A2[IDX(i, c, lda2)] -= acc;
            }
    }
    int b0 = fwd ? 0 : k - l;
    int cnt = L ? n : m;
    zc *tmp = (zc *)malloc(sizeof(zc) * (size_t)(l > 0 ? l : 1));
    for (int x = 0; x < cnt; ++x) {
        for (int t = 0; t < l; ++t) {
            int rt = fwd ? mv - l + t : t;
            zc acc = 0.0;
            for (int p = b0; p < b0 + l; ++p)
                if (zpamm_valid(fwd, rt, p, mv, k, l)) {
                    zc v = cja ? conj(VE(rt, p)) : VE(rt, p);
                    acc += L ? zmul(v, W[IDX(p, x, ldw)]) : zmul(W[IDX(x, p, ldw)], v);
                }
            tmp[t] = acc;
        }
        for (int t = 0; t < l; ++t) {
            if (L) W[IDX(b0 + t, x, ldw)] = tmp[t]; else W[IDX(x, b0 + t, ldw)] = tmp[t];
        }
    }
    free(tmp);
#undef VE
    return 0;
}

/* parfb in every direct / storev form for complex elements: the sequence of */
/* ora_dparfb_full (nextla_oracle.c) with the adjoint conjugating T.         */
int ora_zparfb_full(char side, char trans, char direct, char storev, int m1, int n1, int m2, int n2,
                    int k, int l, zc *A1, int lda1, zc *A2, int lda2, const zc *V, int ldv,
                    const zc *T, int ldt, zc *W, int ldw)
{
    if (side != 'L' && side != 'R') return -1;
    if (trans != 'N' && trans != 'C' && trans != 'T') return -2;
    if (direct != 'F' && direct != 'B') return -3;
    if (storev != 'C' && storev != 'R') return -4;
    if (m1 < 0) return -5;
    if (n1 < 0) return -6;
    if (m2 < 0 || (side == 'R' && m1 != m2)) return -7;
    if (n2 < 0 || (side == 'L' && n1 != n2)) return -8;
    if (k < 0) return -9;
    if (l < 0 || l > k) return -10;
    if (m1 == 0 || n1 == 0 || n2 == 0 || k == 0 || m2 == 0) return 0;
    int L = (side == 'L'), up = (direct == 'F'), adj = (trans != 'N');
    int rc = ora_zpamm('W', side, storev, direct, m2, n2, k, l, A1, lda1, A2, lda2, V, ldv, W, ldw);
    if (rc) return rc;
#define TRI(i, j) ((up ? (i) <= (j) : (i) >= (j)) ? T[IDX(i, j, ldt)] : (zc)0.0)
#define M(i, j) (adj ? conj(TRI(j, i)) : TRI(i, j))
    int cnt = L ? n2 : m2;
    zc *tmp = (zc *)malloc(sizeof(zc) * (size_t)k);
    for (int x = 0; x < cnt; ++x) {
        for (int i = 0; i < k; ++i) {
            zc acc = 0.0;
            for (int j = 0; j < k; ++j)
                acc += L ? zmul(M(i, j), W[IDX(j, x, ldw)]) : zmul(W[IDX(x, j, ldw)], M(j, i));
            tmp[i] = acc;
        }
        for (int i = 0; i < k; ++i) {
            if (L) W[IDX(i, x, ldw)] = tmp[i]; else W[IDX(x, i, ldw)] = tmp[i];
        }
    }
    free(tmp);
#undef TRI
#undef M
    for (int x = 0; x < cnt; ++x)
        for (int i = 0; i < k; ++i) {
            if (L) A1[IDX(i, x, lda1)] -= W[IDX(i, x, ldw)]; else A1[IDX(x, i, lda1)] -= W[IDX(x, i, ldw)];
        }
    return ora_zpamm('A', side, storev, direct, m2, n2, k, l, A1, lda1, A2, lda2, V, ldv, W, ldw);
}
