"""GPU tests of the eigenvalue adjoint (reverse-mode rule of A -> eigenvalues).

Loss as in the differentiation workload: L = sum_b logsumexp(Re(l_b) / 0.1).
The GPU gradient is checked (a) against central finite differences (h = 1e-6) of L
on random complex directions, with eigenvalues from the CPU oracle, to 1e-6
relative, and (b) against the gradient assembled on the CPU from the oracle's
right and left eigenvectors (the reference's eigvecs(S) / eigvecs(S; left=true)).
"""
import numpy as np
import pytest

from common import randn_matrix
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
TAU = 0.1


def loss_and_gbar(w):
    x = w.real / TAU
    m = x.max()
    e = np.exp(x - m)
    L = m + np.log(e.sum())
    return L, (e / e.sum()) / TAU + 0j


def total_loss(mats):
    return sum(loss_and_gbar(po.gschur_cplx(A)[2])[0] for A in mats)


def gpu_grads(gs, mats):
    Ts, Zs, ws, st = gs.gschur_batched(mats)
    Tp, ns, offs, woffs = gs.pack_batch(Ts, np.complex128)
    Zp, _, _, _ = gs.pack_batch(Zs, np.complex128)
    gbar = np.concatenate([loss_and_gbar(w)[1] for w in ws])
    G = gs.eig_adjoint_batched(Tp, Zp, ns, offs, woffs, gbar)
    return gs.unpack_batch(G, ns, offs), Ts, Zs, ws


def oracle_grad(A):
    T, Z, w = po.gschur_cplx(A)
    X = po.eigvecs(T, Z)
    Y = po.eigvecs(T, Z, left=True)
    g = loss_and_gbar(w)[1]
    s = np.sum(Y.conj() * X, axis=0)
    return (Y * (g / s.conj())) @ X.conj().T


@pytest.mark.parametrize("n", [4, 16, 64])
def test_adjoint_matches_oracle_eigvec_gradient(gs, n):
    rng = np.random.default_rng(7000 + n)
    mats = [randn_matrix(rng, n, cplx=True) / np.sqrt(n) for _ in range(6)]
    grads, _, _, _ = gpu_grads(gs, mats)
    for A, G in zip(mats, grads):
        Gr = oracle_grad(A)
        assert np.linalg.norm(G - Gr) <= 1e-9 * max(np.linalg.norm(Gr), 1e-300)


@pytest.mark.parametrize("n", [8, 64])
def test_adjoint_matches_finite_differences(gs, n):
    rng = np.random.default_rng(8000 + n)
    mats = [randn_matrix(rng, n, cplx=True) / np.sqrt(n) for _ in range(3)]
    grads, _, _, _ = gpu_grads(gs, mats)
    h = 1e-6
    for _ in range(50 if n <= 8 else 10):
        E = [randn_matrix(rng, n, cplx=True) for _ in mats]
        fd = (total_loss([A + h * e for A, e in zip(mats, E)]) - total_loss([A - h * e for A, e in zip(mats, E)])) / (2 * h)
        an = sum(np.real(np.vdot(G, e)) for G, e in zip(grads, E))
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1.0), (fd, an)


def test_torch_autograd_function(gs):
    torch = pytest.importorskip("torch")
    from genericschur_gb300.autograd import eigvals_batched
    rng = np.random.default_rng(9)
    n, b = 16, 5
    A0 = np.stack([randn_matrix(rng, n, cplx=True) / np.sqrt(n) for _ in range(b)])
    A = torch.tensor(A0, dtype=torch.complex128, device="cuda", requires_grad=True)
    w = eigvals_batched(A)
    L = torch.logsumexp(w.real / TAU, dim=1).sum()
    L.backward()
    G = A.grad.cpu().numpy()
    for k in range(b):
        Gr = oracle_grad(A0[k])
        assert np.linalg.norm(G[k] - Gr) <= 1e-9 * np.linalg.norm(Gr)


def test_adjoint_differentiation_workload(gs):
    """The differentiation workload at full size: 4,096 complex 64 x 64 matrices (iid
    complex N(0, 1/2) / 8, seed 7), L = sum_b logsumexp(Re(l_b) / 0.1).  The GPU
    gradient (eigenvalue adjoint on the GPU Schur pairs) must match central finite
    differences (h = 1e-6, Richardson-combined with 2h, forward passes on the GPU) on 50
    random directions to 1e-6 relative, and the gradient assembled from the oracle's left/right eigenvectors on
    a sample of the matrices to 1e-9 relative."""
    from genericschur_gb300.workloads import adjoint_batch, logsumexp_loss
    n = 64
    packed, ns, offs, woffs = adjoint_batch(4096, n, seed=7)

    def forward(p):
        T, Z, w, st = gs.gschur_batched(packed=p, ns=ns, offs=offs, woffs=woffs)
        assert np.all(st == 0)
        return T, Z, w

    T, Z, w = forward(packed)
    L, gbar = logsumexp_loss(w, woffs, n)
    G = gs.eig_adjoint_batched(T, Z, ns, offs, woffs, gbar)
    rng = np.random.default_rng(70)
    for b in rng.choice(len(ns), size=8, replace=False):
        A = packed[offs[b]:offs[b] + n * n].reshape((n, n), order="F")
        Gb = G[offs[b]:offs[b] + n * n].reshape((n, n), order="F")
        Gr = oracle_grad(A)
        assert np.linalg.norm(Gb - Gr) <= 1e-9 * np.linalg.norm(Gr)
    # Central differences with h = 1e-6 along directions with iid complex N(0, 1) entries.
    # Over 262,144 eigenvalues the closest pairs make the h^2 truncation term of a single
    # central difference reach ~1e-5 relative, and shrinking the direction instead lets
    # the loss's rounding noise (~35 eps of L) dominate; the Richardson combination of
    # the steps h and 2h, (4 D(h) - D(2h)) / 3, removes the h^2 term and keeps both
    # errors near 1e-7.
    h = 1e-6
    worst = 0.0
    for _ in range(50):
        E = (rng.standard_normal(len(packed)) + 1j * rng.standard_normal(len(packed))) / np.sqrt(2.0)

        def cd(step):
            Lp = logsumexp_loss(forward(packed + step * E)[2], woffs, n)[0]
            Lm = logsumexp_loss(forward(packed - step * E)[2], woffs, n)[0]
            return (Lp - Lm) / (2 * step)

        fd = (4.0 * cd(h) - cd(2 * h)) / 3.0
        an = float(np.real(np.vdot(G, E)))
        worst = max(worst, abs(fd - an) / max(abs(an), 1.0))
    assert worst <= 1e-6, worst
