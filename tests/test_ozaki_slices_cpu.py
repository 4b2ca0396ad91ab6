"""CPU check of the arithmetic behind the tensor-core products of the mixed batched
refinement (genericschur.jl_gb300/csrc/refine_tc.cu).

The kernel forms FP64-accurate products C = op(X) Y of n x n matrices (n <= 128) from BF16
slice products: rows of op(X) and columns of Y are scaled by powers of two (max |x| < 2^e),
cut into eight 7-bit slices (56 bits), every slice product is summed over k in an FP32
accumulator per level s + t, and the eight level sums are combined as integers in two
64-bit Horner sums of four levels each, which stay below 2^46, and

    C_ij = 2^(e_i + f_j - 14) (hs 2^-21 + ls 2^-49).

This test restates those steps with exact integer arithmetic on the CPU and checks the
claims the kernel relies on: every level sum is below 2^24 (so the tensor core's FP32
accumulation of a level is exact in any order), the Horner sums are below 2^46 (exact FP64
conversions), and the result agrees with the exact product to within the rounding error of
an FP64 dot product of the same length.  No GPU is used.
"""
from fractions import Fraction
import math

import numpy as np
import pytest

BITS, SLICES, LEVELS = 7, 8, 8


def _scale_exps(rows):
    """e with max |x| < 2^e per row (frexp), None for a zero row."""
    out = []
    for r in rows:
        m = float(np.max(np.abs(r))) if r.size else 0.0
        out.append(None if m == 0.0 else math.frexp(m)[1])
    return out


def _slices(v, e):
    """The eight signed 7-bit slices of v relative to 2^e: floor(|v| 2^(56-e)) in groups."""
    if e is None or v == 0.0:
        return [0] * SLICES
    f = Fraction(abs(v)) * Fraction(2) ** (56 - e)
    F = int(f)  # truncation toward zero
    assert 0 <= F < 2 ** 56
    sign = -1 if v < 0 else 1
    return [sign * ((F >> (56 - BITS * (s + 1))) & 127) for s in range(SLICES)]


def _emulate(X, Y):
    """C = X Y by the kernel's scheme; returns C, the largest |level| and the largest |hs|, |ls|."""
    n = X.shape[0]
    ex = _scale_exps([X[i, :] for i in range(n)])
    fy = _scale_exps([Y[:, j] for j in range(n)])
    xs = np.array([[_slices(X[i, k], ex[i]) for k in range(n)] for i in range(n)], dtype=np.int64)  # i, k, s
    ys = np.array([[_slices(Y[k, j], fy[j]) for k in range(n)] for j in range(n)], dtype=np.int64)  # j, k, t
    lev = np.zeros((LEVELS, n, n), dtype=np.int64)
    for s in range(SLICES):
        for t in range(SLICES):
            if s + t < LEVELS:
                lev[s + t] += xs[:, :, s] @ ys[:, :, t].T  # sum over k, exact in int64
    hs = np.zeros((n, n), dtype=np.int64)
    ls = np.zeros((n, n), dtype=np.int64)
    for L in range(4):
        hs = hs * 128 + lev[L]
    for L in range(4, 8):
        ls = ls * 128 + lev[L]
    C = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            if ex[i] is None or fy[j] is None:
                continue
            s = float(hs[i, j]) * 2.0 ** -21 + float(ls[i, j]) * 2.0 ** -49
            C[i, j] = math.ldexp(s, ex[i] + fy[j] - 2 * BITS)
    return C, int(np.max(np.abs(lev))), int(max(np.max(np.abs(hs)), np.max(np.abs(ls)))), ex, fy


def _exact(X, Y):
    n = X.shape[0]
    Xf = [[Fraction(float(X[i, k])) for k in range(n)] for i in range(n)]
    Yf = [[Fraction(float(Y[k, j])) for j in range(n)] for k in range(n)]
    return [[sum(Xf[i][k] * Yf[k][j] for k in range(n)) for j in range(n)] for i in range(n)]


@pytest.mark.parametrize("n,kind", [(5, "gauss"), (24, "scaled"), (40, "orthogonal")])
def test_slice_products_exact_levels_and_accuracy(n, kind):
    rng = np.random.default_rng(100 + n)
    if kind == "gauss":
        X, Y = rng.standard_normal((n, n)), rng.standard_normal((n, n))
    elif kind == "scaled":  # rows and columns over many binades, one zero row
        X = rng.standard_normal((n, n)) * np.exp2(rng.integers(-40, 40, size=(n, 1)))
        Y = rng.standard_normal((n, n)) * np.exp2(rng.integers(-40, 40, size=(1, n)))
        X[3, :] = 0.0
    else:  # Z^T Z of a nearly orthogonal Z, the product whose small part is the signal
        Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        X = (Q + 1e-7 * rng.standard_normal((n, n))).T
        Y = X.T.copy()
    C, levmax, hlmax, ex, fy = _emulate(X, Y)
    assert levmax < 2 ** 24, levmax
    assert hlmax < 2 ** 46, hlmax
    E = _exact(X, Y)
    C64 = X @ Y
    worst = worst64 = 0.0
    for i in range(n):
        for j in range(n):
            if ex[i] is None or fy[j] is None:
                assert C[i, j] == 0.0
                continue
            scale = math.ldexp(1.0, ex[i] + fy[j])
            err = abs(Fraction(C[i, j]) - E[i][j])
            # truncation 2^-56 per operand and the dropped levels: far below n eps of the scale
            assert err <= Fraction(n) * Fraction(2) ** -52 * Fraction(scale), (i, j, float(err) / scale)
            worst = max(worst, float(err) / scale)
            worst64 = max(worst64, float(abs(Fraction(float(C64[i, j])) - E[i][j])) / scale)
    # as accurate as an FP64 product of the same operands (measured: 0.3 to 1.1 times its error)
    assert worst <= max(2.0 * worst64, 4 * 2.0 ** -52), (worst, worst64)


def test_level_bound_at_the_largest_order():
    """The worst case the kernel's exactness rests on: n = 128 and every slice at 127."""
    n = 128
    worst_pair = 127 * 127 * n
    assert worst_pair < 2 ** 21
    for L in range(LEVELS):
        pairs = sum(1 for s in range(SLICES) for t in range(SLICES) if s + t == L)
        assert pairs * worst_pair < 2 ** 24
    # the two 64-bit Horner sums
    lev = [sum(1 for s in range(SLICES) for t in range(SLICES) if s + t == L) * worst_pair for L in range(LEVELS)]
    hs = ((lev[0] * 128 + lev[1]) * 128 + lev[2]) * 128 + lev[3]
    ls = ((lev[4] * 128 + lev[5]) * 128 + lev[6]) * 128 + lev[7]
    assert max(hs, ls) < 2 ** 46
