"""GPU tests of Schur reordering (gordschur!, ordschur.jl:24-74 complex, rordschur.jl:3-47
real), restating the reference's own checks (test/ordschur.jl:1-28, 60-125): the result
is a Schur form (triangular / quasi-triangular in standard form), A = Z T Z^H and Z^H Z
= I to 10 n eps, and the selected eigenvalues come first."""
import numpy as np
import pytest

from common import EPS, checkblocks, checkeigvals, randn_matrix

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [2, 8, 32, 100, 200])
def test_ordschur_complex(gs, n):
    rng = np.random.default_rng(5100 + n)
    A = randn_matrix(rng, n, cplx=True)
    S = gs.gschur(A)
    select = np.ones(n, dtype=bool)
    select[: n >> 1] = False  # the reference's choice: the second half moves to the front
    S2 = gs.gordschur(S, select)
    T2, Z2 = S2.T, S2.Z
    assert np.all(np.tril(T2, -1) == 0)
    nA = np.linalg.norm(A)
    assert np.linalg.norm(Z2 @ T2 @ Z2.conj().T - A) / (n * nA * EPS) < 10
    assert np.linalg.norm(np.eye(n) - Z2 @ Z2.conj().T) / (n * EPS) < 10
    wanted = S.values[select]
    for i in range(int(select.sum())):
        w = T2[i, i]
        assert np.min(np.abs(wanted - w)) / (EPS + abs(w)) < 10 * n


@pytest.mark.parametrize("n", [4, 10, 32, 100, 200])
def test_ordschur_real(gs, n):
    rng = np.random.default_rng(5200 + n)
    A = randn_matrix(rng, n)
    S = gs.gschur(A)
    # select every third eigenvalue (both members of a conjugate pair)
    w = S.values
    select = np.zeros(n, dtype=bool)
    k = 0
    while k < n:
        pair = k + 1 < n and S.T[k + 1, k] != 0
        if k % 3 == 0:
            select[k] = True
            if pair:
                select[k + 1] = True
        k += 2 if pair else 1
    S2 = gs.gordschur(S, select)
    T2, Z2, w2 = S2.T, S2.Z, S2.values
    assert np.all(np.tril(T2, -2) == 0)
    assert checkblocks(T2)
    nA = np.linalg.norm(A)
    assert np.linalg.norm(Z2 @ T2 @ Z2.T - A) / (n * nA * EPS) < 10
    assert np.linalg.norm(np.eye(n) - Z2 @ Z2.T) / (n * EPS) < 10
    assert checkeigvals(T2, w2, 10)
    wanted = w[select]
    wscale = np.max(np.abs(w2))
    for i in range(int(select.sum())):
        assert np.min(np.abs(wanted - w2[i])) / (EPS + wscale) < 10 * n


def test_ordschur_identity_selection(gs):
    """Selecting everything (or nothing) leaves the pair unchanged."""
    rng = np.random.default_rng(5300)
    A = randn_matrix(rng, 20)
    S = gs.gschur(A)
    for sel in (np.ones(20, dtype=bool), np.zeros(20, dtype=bool)):
        S2 = gs.gordschur(S, sel)
        np.testing.assert_array_equal(S2.T, S.T)
        np.testing.assert_array_equal(S2.Z, S.Z)
