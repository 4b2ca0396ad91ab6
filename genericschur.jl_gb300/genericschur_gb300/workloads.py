"""Seeded synthetic workloads with the sizes and value laws of the benchmark configs.

The reference publishes no datasets; the configs name their inputs by law and
seed, and these generators reproduce those laws with numpy's PCG64 streams (the
reference's Julia randn stream cannot be reproduced outside Julia).
"""
import numpy as np

from . import pack_batch


def batch_sizes(count, seed, lo=8, hi=128):
    """Orders iid uniform on the integers [lo, hi]."""
    rng = np.random.default_rng(seed)
    return rng.integers(lo, hi + 1, size=count).astype(np.int32)


def batched_real(count=20000, seed=4, lo=8, hi=128):
    """Packed batch of real N(0,1) matrices with orders ~ U{lo..hi}.
    Returns (packed, ns, offs, woffs)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(lo, hi + 1, size=count).astype(np.int32)
    sq = ns.astype(np.int64) ** 2
    offs = np.zeros(count, dtype=np.int64)
    offs[1:] = np.cumsum(sq)[:-1]
    woffs = np.zeros(count, dtype=np.int64)
    woffs[1:] = np.cumsum(ns.astype(np.int64))[:-1]
    packed = rng.standard_normal(int(sq.sum()))  # column-major per matrix by construction
    return packed, ns, offs, woffs


def batched_cplx(count=5000, seed=5, lo=8, hi=128):
    """Packed batch of complex matrices, real and imaginary parts iid N(0, 1/2)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(lo, hi + 1, size=count).astype(np.int32)
    sq = ns.astype(np.int64) ** 2
    offs = np.zeros(count, dtype=np.int64)
    offs[1:] = np.cumsum(sq)[:-1]
    woffs = np.zeros(count, dtype=np.int64)
    woffs[1:] = np.cumsum(ns.astype(np.int64))[:-1]
    m = int(sq.sum())
    packed = (rng.standard_normal(m) + 1j * rng.standard_normal(m)) / np.sqrt(2.0)
    return packed, ns, offs, woffs


def real_flops(ns):
    """Algorithmic FLOPs of a real Schur decomposition with Z: 25 n^3 per matrix."""
    return 25.0 * float(np.sum(np.asarray(ns, dtype=np.float64) ** 3))


def cplx_flops(ns):
    """Complex Schur with Z: 25 n^3 complex operations = 100 n^3 real FLOPs."""
    return 100.0 * float(np.sum(np.asarray(ns, dtype=np.float64) ** 3))


__all__ = ["batch_sizes", "batched_real", "batched_cplx", "real_flops", "cplx_flops", "pack_batch", "conditioned_matrix",
           "large_real", "LARGE_SEEDS", "adjoint_batch", "logsumexp_loss"]


def conditioned_matrix(n=2048, seed=6, cond=1e3, lo=1e-3, hi=1e3):
    """A = V diag(l) V^-1 with l real, |l| log-uniform in [lo, hi] with random signs,
    and V Gaussian with its singular values replaced by a log-uniform spread from 1 to
    cond (V = U diag(s) W^T from the SVD of a Gaussian matrix)."""
    rng = np.random.default_rng(seed)
    lam = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n)) * rng.choice([-1.0, 1.0], size=n)
    G = rng.standard_normal((n, n))
    U, _, Wt = np.linalg.svd(G)
    s = np.exp(np.linspace(0.0, np.log(cond), n))
    V = (U * s) @ Wt
    Vinv = (Wt.T / s) @ U.T
    return np.asfortranarray((V * lam) @ Vinv)


LARGE_SEEDS = {4096: 1, 1024: 2, 2048: 3}


def large_real(n=4096, seed=None):
    """One real n x n matrix with iid N(0,1) entries (column-major); the default seeds
    are 1 for n=4096, 2 for n=1024 and 3 for n=2048."""
    if seed is None:
        seed = LARGE_SEEDS.get(n, n)
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((n, n)))


def adjoint_batch(count=4096, n=64, seed=7):
    """The differentiation workload: count complex n x n matrices, entries iid complex
    N(0, 1/2) / sqrt(n) (real and imaginary parts N(0, 1/2), then scaled).
    Returns (packed, ns, offs, woffs)."""
    rng = np.random.default_rng(seed)
    ns = np.full(count, n, dtype=np.int32)
    offs = (np.arange(count, dtype=np.int64) * n * n)
    woffs = (np.arange(count, dtype=np.int64) * n)
    m = count * n * n
    packed = (rng.standard_normal(m) + 1j * rng.standard_normal(m)) / np.sqrt(2.0) / np.sqrt(n)
    return packed, ns, offs, woffs


def logsumexp_loss(w_packed, woffs, n, tau=0.1):
    """L = sum_b logsumexp(Re(l_b) / tau) and its cotangent dL/dRe(l) (as complex)."""
    W = np.asarray(w_packed).reshape(-1, n)
    x = W.real / tau
    m = x.max(axis=1, keepdims=True)
    e = np.exp(x - m)
    s = e.sum(axis=1, keepdims=True)
    L = float(np.sum(m[:, 0] + np.log(s[:, 0])))
    gbar = (e / s / tau).astype(np.complex128).ravel()
    return L, gbar
