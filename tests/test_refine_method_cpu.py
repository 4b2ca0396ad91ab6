"""CPU check of the Newton refinement that the mixed batched form runs on the GPU
(genericschur.jl_gb300/csrc/refine_batched.cu, refine_tc.cu, refine_bin_impl.cuh).

The method (Bujanovic, Kressner and Schroeder, "Iterative refinement of Schur
decompositions", Numer. Algorithms 2023), as the kernels apply it to an FP32 Schur pair
(T32, Z32) of A with the 1x1/2x2 block structure of T32:

    At = Z^T A Z,  N = (I - Z^T Z) / 2,  L = block-lower part of At,
    W block-lower with  T_pp W_pq - W_pq T_qq = -(L + N At + At N)_pq
                                                 - sum_{r>p} T_pr W_rq + sum_{r<q} W_pr T_rq,
    X = N + W - W^T,  Z <- Z + Z X,  the step is the last once max|X| <= 1e-9, and then
    T = At + X^T At + At X with its block-lower part set to zero.

This test restates those equations in FP64 on the CPU, starting from LAPACK's FP32 Schur
form (scipy), and checks what the kernels rely on: two Newton steps reach the final
tolerance for random matrices, and the result meets the parity bounds (backward error and
orthogonality below 10 n eps, block upper triangular T).  No GPU is used.
"""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")

EPS = np.finfo(np.float64).eps


def _block_starts(T):
    n = T.shape[0]
    bs, i = [], 0
    while i < n:
        bs.append(i)
        i += 2 if (i + 1 < n and T[i + 1, i] != 0.0) else 1
    bs.append(n)
    return bs


def _sylvester_waves(T, R, bs):
    """Block-lower W of the block-triangular Sylvester equation, by anti-diagonal waves."""
    n = T.shape[0]
    N = len(bs) - 1
    W = np.zeros((n, n))
    for D in range(N - 1, 0, -1):
        for q in range(N - D):
            p = q + D
            i0, i1, j0, j1 = bs[p], bs[p + 1], bs[q], bs[q + 1]
            r = R[i0:i1, j0:j1] - T[i0:i1, i1:] @ W[i1:, j0:j1] + W[i0:i1, :j0] @ T[:j0, j0:j1]
            ip, jq = i1 - i0, j1 - j0
            K = np.kron(np.eye(jq), T[i0:i1, i0:i1]) - np.kron(T[j0:j1, j0:j1].T, np.eye(ip))
            W[i0:i1, j0:j1] = np.linalg.solve(K, r.reshape(-1, order="F")).reshape((ip, jq), order="F")
    return W


def _refine(A, T32, Z32, max_steps=6):
    n = A.shape[0]
    bs = _block_starts(T32)
    bid = np.zeros(n, dtype=int)
    for p in range(len(bs) - 1):
        bid[bs[p]:bs[p + 1]] = p
    lower = bid[:, None] > bid[None, :]
    Z = Z32.astype(np.float64)
    for step in range(max_steps):
        At = Z.T @ (A @ Z)
        Nm = 0.5 * (np.eye(n) - Z.T @ Z)
        Tu = np.where(lower, 0.0, At)
        M = Nm @ At + At @ Nm
        R = np.where(lower, -(At + M), 0.0)
        W = _sylvester_waves(Tu, R, bs)
        X = np.where(lower, Nm + W, 0.0) + np.where(lower.T, Nm - W.T, 0.0) + np.where(~lower & ~lower.T, Nm, 0.0)
        xmax = float(np.max(np.abs(X)))
        assert xmax <= 1e-1, "diverged"
        if xmax <= 1e-9:
            T = At + X.T @ At + At @ X
            T[lower] = 0.0
            return T, Z + Z @ X, step + 1
        Z = Z + Z @ X
    raise AssertionError("not converged in %d steps" % max_steps)


@pytest.mark.parametrize("n,seed", [(8, 1), (31, 2), (64, 3), (100, 4)])
def test_two_newton_steps_reach_fp64_accuracy(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n))
    A /= 2.0 ** np.floor(np.log2(np.max(np.abs(A))))  # the kernels' unit scaling (exact)
    T32, Z32 = scipy_linalg.schur(A.astype(np.float32), output="real")
    T, Z, steps = _refine(A, T32.astype(np.float64), Z32)
    assert steps == 2, steps
    bwd = np.linalg.norm(A - Z @ T @ Z.T) / np.linalg.norm(A)
    orth = np.linalg.norm(Z.T @ Z - np.eye(n))
    assert bwd <= 10 * n * EPS, bwd / (n * EPS)
    assert orth <= 10 * n * EPS, orth / (n * EPS)
    # far below the bound: the refined pair is as accurate as an FP64 Schur form
    assert bwd <= n * EPS and orth <= n * EPS
