"""CPU check of the schedule of the tiled block Sylvester solve in the mixed batched
refinement (sylv_tiled in genericschur.jl_gb300/csrc/refine_bin_impl.cuh).

Each Newton step solves, for the block-lower W of a quasi-triangular T (1x1 and 2x2
diagonal blocks),

    T_pp W_pq - W_pq T_qq = R_pq - sum_{r>p} T_pr W_rq + sum_{r<q} W_pr T_rq,   p > q.

The kernel cuts the blocks into tiles of about kTile rows (never splitting a 2x2 block),
solves the tile pairs (P, Q), P >= Q, by waves D = P - Q from the bottom-left tile up, each
tile by local anti-diagonals of block pairs with only the within-tile sums, and after each
wave pushes the solved tiles' contributions into the right-hand sides of the tiles that
need them (R_PQ -= T_{P,S} W_{S,Q} for the solved tile below, R_PQ += W_{P,S} T_{S,Q} for the
solved tile to the left).  This test restates that schedule in FP64 with the kernel's index
rules and compares it with a direct solve of the whole equation, for block patterns that
put 2x2 blocks on tile boundaries, and for several tile sizes.  No GPU is used.
"""
import numpy as np
import pytest


def _blocks(n, pattern, rng):
    """Block starts bs[0..N] for a pattern: 'ones', 'twos', 'mixed' or 'random'."""
    bs, i = [0], 0
    while i < n:
        if pattern == "ones":
            w = 1
        elif pattern == "twos":
            w = 2
        elif pattern == "mixed":
            w = 2 if (len(bs) % 3) else 1
        else:
            w = int(rng.integers(1, 3))
        w = min(w, n - i)
        i += w
        bs.append(i)
    return bs


def _quasi_triangular(n, bs, rng):
    T = np.triu(rng.standard_normal((n, n)))
    for p in range(len(bs) - 1):
        i0, w = bs[p], bs[p + 1] - bs[p]
        T[i0, i0] = 3.0 * p + 1.0  # well separated diagonal blocks
        if w == 2:
            T[i0 + 1, i0 + 1] = T[i0, i0]
            T[i0, i0 + 1], T[i0 + 1, i0] = 1.5, -0.75
    return T


def _bid(n, bs):
    bid = np.zeros(n, dtype=int)
    for p in range(len(bs) - 1):
        bid[bs[p]:bs[p + 1]] = p
    return bid


def _direct(T, R, bs):
    """The block-lower unknowns of the whole equation by one dense solve."""
    n = T.shape[0]
    bid = _bid(n, bs)
    idx = [(i, j) for j in range(n) for i in range(n) if bid[i] > bid[j]]
    pos = {e: k for k, e in enumerate(idx)}
    K = np.zeros((len(idx), len(idx)))
    rhs = np.array([R[i, j] for i, j in idx])
    for k, (i, j) in enumerate(idx):
        # (T W - W T)_{ij} over block-lower W: sum_a T[i, a] W[a, j] - sum_b W[i, b] T[b, j]
        for a in range(n):
            if (a, j) in pos:
                K[k, pos[(a, j)]] += T[i, a]
        for b in range(n):
            if (i, b) in pos:
                K[k, pos[(i, b)]] -= T[b, j]
    w = np.linalg.solve(K, rhs)
    W = np.zeros_like(T)
    for k, (i, j) in enumerate(idx):
        W[i, j] = w[k]
    return W


def _pair_solve(T, i0, ip, j0, jq, r):
    m = ip * jq
    K = np.zeros((m, m))
    rv = np.zeros(m)
    for b in range(jq):
        for a in range(ip):
            row = a + ip * b
            rv[row] = r[a, b]
            for a2 in range(ip):
                K[row, a2 + ip * b] += T[i0 + a, i0 + a2]
            for b2 in range(jq):
                K[row, a + ip * b2] -= T[j0 + b2, j0 + b]
    x = np.linalg.solve(K, rv)
    out = np.zeros((2, 2))
    for b in range(jq):
        for a in range(ip):
            out[a, b] = x[a + ip * b]
    return out


def _tiled(T, R, bs, tile):
    """The kernel's schedule (sylv_tiled), in FP64."""
    n = T.shape[0]
    N = len(bs) - 1
    bid = _bid(n, bs)
    te, tbk = [0], [0]
    for p in range(N):
        if bs[p] - te[-1] >= tile:
            te.append(bs[p])
            tbk.append(p)
    te.append(n)
    tbk.append(N)
    nt = len(te) - 1
    assert all(te[t + 1] - te[t] <= tile + 1 for t in range(nt))
    R = R.copy()
    W = np.zeros_like(T)
    for D in range(nt - 1, -1, -1):
        ntl = nt - D
        rw = {Q: R[te[Q + D]:te[Q + D + 1], te[Q]:te[Q + 1]].copy() for Q in range(ntl)}
        maxw = max((tbk[Q + D + 1] - tbk[Q + D]) + (tbk[Q + 1] - tbk[Q]) - 1 for Q in range(ntl))
        for w in range(maxw):
            for Q in range(ntl):
                P = Q + D
                pb, pe, qb, qe = tbk[P], tbk[P + 1], tbk[Q], tbk[Q + 1]
                for a in range(w + 1):
                    p, q = pe - 1 - a, qb + (w - a)
                    if p < pb or q >= qe or (D == 0 and p <= q):
                        continue
                    tP, tQ = te[P], te[Q]
                    li0, ip, lj0, jq = bs[p] - tP, bs[p + 1] - bs[p], bs[q] - tQ, bs[q + 1] - bs[q]
                    lpe = te[P + 1] - tP
                    blk = rw[Q]
                    r = np.zeros((2, 2))
                    r[:ip, :jq] = blk[li0:li0 + ip, lj0:lj0 + jq]
                    for k in range(li0 + ip, lpe):  # - sum_{r>p} T_pr W_rq within tile P
                        r[:ip, :jq] -= np.outer(T[tP + li0:tP + li0 + ip, tP + k], blk[k, lj0:lj0 + jq])
                    for k in range(0, lj0):  # + sum_{r<q} W_pr T_rq within tile Q
                        r[:ip, :jq] += np.outer(blk[li0:li0 + ip, k], T[tQ + k, tQ + lj0:tQ + lj0 + jq])
                    x = _pair_solve(T, bs[p], ip, bs[q], jq, r)
                    blk[li0:li0 + ip, lj0:lj0 + jq] = x[:ip, :jq]
        for Q in range(ntl):
            P = Q + D
            for li in range(te[P + 1] - te[P]):
                for lj in range(te[Q + 1] - te[Q]):
                    i, j = te[P] + li, te[Q] + lj
                    if bid[i] > bid[j]:
                        W[i, j] = rw[Q][li, lj]
        if D == 0:
            break
        for Q in range(ntl):  # term 1: the solved tile (Q+D, Q) into tiles Q .. Q+D-1 of column Q
            k0, k1 = te[Q + D], te[Q + D + 1]
            R[te[Q]:te[Q + D], te[Q]:te[Q + 1]] -= T[te[Q]:te[Q + D], k0:k1] @ rw[Q]
        for P in range(D, nt):  # term 2: the solved tile (P, P-D) into tiles P-D+1 .. P of row P
            k0, k1 = te[P - D], te[P - D + 1]
            R[te[P]:te[P + 1], te[P - D + 1]:te[P + 1]] += rw[P - D] @ T[k0:k1, te[P - D + 1]:te[P + 1]]
    return W


@pytest.mark.parametrize("n", [1, 2, 7, 33, 61])
@pytest.mark.parametrize("pattern", ["ones", "twos", "mixed", "random"])
@pytest.mark.parametrize("tile", [4, 16])
def test_tiled_schedule_equals_direct_solve(n, pattern, tile):
    rng = np.random.default_rng(7 * n + len(pattern) + tile)
    bs = _blocks(n, pattern, rng)
    T = _quasi_triangular(n, bs, rng)
    R = rng.standard_normal((n, n))
    W_ref = _direct(T, R, bs)
    W = _tiled(T, R, bs, tile)
    scale = max(1.0, float(np.max(np.abs(W_ref))))
    assert np.max(np.abs(W - W_ref)) <= 1e-10 * scale
