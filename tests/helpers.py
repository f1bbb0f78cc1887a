"""Shared builders for the parity tests (random charge-conserving MPS, conversions)."""
import numpy as np

from oracle import tn_oracle as O


def random_qn_links(N, rng, maxsec_dim=4, target=0, qn=True):
    """Link charge arrays of an N-site spin-1/2 chain with total charge ``target``."""
    links = []
    for i in range(N + 1):
        if not qn:
            links.append(np.repeat([0], 1 if i in (0, N) else rng.integers(2, maxsec_dim * 3)))
            continue
        lo = max(-i, target - (N - i))
        hi = min(i, target + (N - i))
        qs = [q for q in range(lo, hi + 1) if (q - i) % 2 == 0]
        if i in (0, N):
            links.append(np.array([0 if i == 0 else target]))
            continue
        dims = rng.integers(1, maxsec_dim + 1, size=len(qs))
        links.append(np.repeat(np.array(qs), dims))
    return links


def random_qn_mps(N, rng, maxsec_dim=4, qn=True):
    links = random_qn_links(N, rng, maxsec_dim, qn=qn)
    pq = O.SPIN_HALF_Q if qn else np.zeros(2, dtype=np.int64)
    A = []
    for i in range(N):
        t = rng.standard_normal((len(links[i]), 2, len(links[i + 1])))
        t *= O.qn_mask3(links[i], pq, links[i + 1])
        A.append(t)
    return O.MPS(A, links, pq, center=0)


def upload_mps(tn, ctx, mps, center):
    return tn.MPS([a for a in mps.A], [q.astype(np.int32) for q in mps.links],
                  mps.phys_q.astype(np.int32), center, ctx)


def upload_mpo(tn, ctx, H):
    return tn.MPO(H.W, [d.astype(np.int32) for d in H.delta], H.phys_q.astype(np.int32), ctx)


def oracle_envs(mps, H, p):
    """L[p] and R[p+1] of the oracle for the two-site position p."""
    env = O.StateEnvs(mps, H)
    env.position(p, 2)
    return env.L[p], env.R[p + 1]


def dense_mpo(H):
    """Contract an MPO to a dense matrix (small N only)."""
    acc = H.W[0][0]  # (b, s', s)
    for W in H.W[1:]:
        b, Sp, S = acc.shape
        d = W.shape[2]
        acc = np.einsum("bxy,bcuv->cxuyv", acc, W).reshape(W.shape[1], Sp * d, S * d)
    return acc[0]
