"""Host-side model inputs: spin-1/2 site charges, MPOs of two-body Hamiltonians and
product states.  These build dense host arrays only; all sweep arithmetic runs in
libtennet_cuda.so.

Charges follow ITensors' S=1/2 convention with QN("Sz") in units of 1/2: Up = +1, Dn = -1.
"""
from __future__ import annotations

import numpy as np

SPIN_HALF_Q = np.array([1, -1], dtype=np.int32)


def _ops():
    eye = np.eye(2)
    sz = np.diag([0.5, -0.5])
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm = sp.T.copy()
    return {"Id": (eye, 0), "Sz": (sz, 0), "S+": (sp, 2), "S-": (sm, -2)}


def heisenberg_chain_terms(N: int, J: float = 1.0):
    """OpSum of the open S=1/2 Heisenberg chain: J Sz Sz + J/2 (S+S- + S-S+) per bond
    (the model of the reference tests, test/test_MPS_DMRG.jl:29-33)."""
    terms = []
    for i in range(N - 1):
        terms += [(J, "Sz", i, "Sz", i + 1), (0.5 * J, "S+", i, "S-", i + 1),
                  (0.5 * J, "S-", i, "S+", i + 1)]
    return terms


def j1j2_cylinder_terms(Lx: int, Ly: int, J1: float = 1.0, J2: float = 0.5):
    """J1-J2 Heisenberg model on an Lx x Ly cylinder (periodic in y, open in x), sites
    snaked column by column: site = Ly * x + y."""
    def site(x, y):
        return Ly * x + (y % Ly)

    bonds = {}
    for x in range(Lx):
        for y in range(Ly):
            a = site(x, y)
            cand = [((x, y + 1), J1)]
            if x + 1 < Lx:
                cand += [((x + 1, y), J1), ((x + 1, y + 1), J2), ((x + 1, y - 1), J2)]
            for (xx, yy), J in cand:
                b = site(xx, yy)
                if a != b:
                    bonds[(min(a, b), max(a, b))] = J
    terms = []
    for (i, j), J in sorted(bonds.items()):
        terms += [(J, "Sz", i, "Sz", j), (0.5 * J, "S+", i, "S-", j), (0.5 * J, "S-", i, "S+", j)]
    return terms


def mpo_from_terms(N: int, terms, conserve_qns: bool = True):
    """Finite-state-automaton MPO of a sum of two-body terms c * O_i O_j (i < j).

    Link k (left of site k) carries the states "start" (k < N), one pending state per
    (first operator, its site i) that is still waiting for its partner (i < k <= last j),
    and "done" (k > 0).  Returns (W, delta, phys_q) with W[k] of shape (w_k, w_{k+1}, 2, 2)
    as [a, b, s', s] and delta[k] the charges of MPO link k.
    """
    ops = _ops()
    eye = ops["Id"][0]
    by_first: dict = {}
    for c, o1, i, o2, j in terms:
        if not i < j:
            raise ValueError("two-body terms need i < j")
        by_first.setdefault((o1, i), []).append((c, o2, j))
    last = {k: max(j for _, _, j in v) for k, v in by_first.items()}
    order = sorted(by_first, key=lambda t: (t[1], t[0]))
    links = []
    for k in range(N + 1):
        keys = (["start"] if k < N else []) + [key for key in order if key[1] < k <= last[key]]
        if k > 0:
            keys.append("done")
        links.append(keys)
    W = []
    for s in range(N):
        li = {key: n for n, key in enumerate(links[s])}
        ri = {key: n for n, key in enumerate(links[s + 1])}
        w = np.zeros((len(li), len(ri), 2, 2))
        if "start" in li and "start" in ri:
            w[li["start"], ri["start"]] += eye
        if "done" in li and "done" in ri:
            w[li["done"], ri["done"]] += eye
        for key, lst in by_first.items():
            o1, i = key
            if i == s:
                w[li["start"], ri[key]] += ops[o1][0]
            if key in li and key in ri:
                w[li[key], ri[key]] += eye
            if key in li:
                for c, o2, j in lst:
                    if j == s:
                        w[li[key], ri["done"]] += c * ops[o2][0]
        W.append(w)
    delta = [np.array([0 if (not conserve_qns or key in ("start", "done")) else ops[key[0]][1]
                       for key in keys], dtype=np.int32) for keys in links]
    pq = SPIN_HALF_Q.copy() if conserve_qns else np.zeros(2, dtype=np.int32)
    return W, delta, pq


def mpo_direct_sum(mpos):
    """One MPO equal to the sum of several: ``[(W, delta), ...]`` with equal site counts,
    physical dimensions and edge charges, edge MPO bonds of dimension one.  The site tensors
    are block diagonal in the MPO bonds (the first concatenated along its right bond, the last
    along its left one), the bond charges concatenated, so its environments are those of the
    summands side by side and every H_eff product is the sum of theirs -- the product of
    ProjMPOSum2 (TenNetLib src/mps/projmposum2.jl:86-101).  Returns (W, delta)."""
    Ws = [[np.asarray(w, dtype=np.float64) for w in W] for W, _ in mpos]
    ds = [[np.asarray(x, dtype=np.int64) for x in delta] for _, delta in mpos]
    if not Ws:
        raise ValueError("no MPO to sum")
    N = len(Ws[0])
    d = Ws[0][0].shape[2]
    for W, delta in zip(Ws, ds):
        if len(W) != N or len(delta) != N + 1 or any(w.shape[2:] != (d, d) for w in W):
            raise ValueError("the MPOs of a sum need the same sites")
        if W[0].shape[0] != 1 or W[-1].shape[1] != 1:
            raise ValueError("the MPOs of a sum need edge bonds of dimension one")
        if not (np.array_equal(delta[0], ds[0][0]) and np.array_equal(delta[N], ds[0][N])):
            raise ValueError("the MPOs of a sum need the same edge charges")
    if N == 1:
        return [sum(W[0] for W in Ws)], [ds[0][0], ds[0][1]]
    out = []
    for i in range(N):
        rows = [1] if i == 0 else [W[i].shape[0] for W in Ws]
        cols = [1] if i == N - 1 else [W[i].shape[1] for W in Ws]
        T = np.zeros((sum(rows), sum(cols), d, d))
        r0 = c0 = 0
        for k, W in enumerate(Ws):
            a, b = W[i].shape[:2]
            T[r0:r0 + a, c0:c0 + b] = W[i]
            if i > 0:
                r0 += a
            if i < N - 1:
                c0 += b
        out.append(T)
    delta = [ds[0][0]] + [np.concatenate([x[i] for x in ds]) for i in range(1, N)] + [ds[0][N]]
    return out, delta


def neel_states(N: int):
    """Up on odd (1-based) sites, Dn on even ones (test/test_MPS_DMRG.jl:35)."""
    return [0 if i % 2 == 0 else 1 for i in range(N)]


def product_state(states, phys_q):
    """Dense site tensors and link charges of a product state of basis states."""
    tensors, links = [], [np.array([0], dtype=np.int32)]
    q = 0
    d = len(phys_q)
    for s in states:
        t = np.zeros((1, d, 1))
        t[0, s, 0] = 1.0
        tensors.append(t)
        q += int(phys_q[s])
        links.append(np.array([q], dtype=np.int32))
    return tensors, links


def random_product_state(N: int, d: int, seed: int):
    """Dense product state with random normalised site vectors (no charge conservation)."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((N, d))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    tensors = [v[i].reshape(1, d, 1).copy() for i in range(N)]
    links = [np.array([0], dtype=np.int32) for _ in range(N + 1)]
    return tensors, links
