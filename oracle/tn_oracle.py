"""CPU oracle for the two-site DMRG / TDVP sweep hot path (TEST INFRASTRUCTURE ONLY).

This module is the oracle, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py`` may import it.  The
product path (``libtennet_cuda.so``) never calls into it.

It restates, in plain numpy FP64 with dense arrays carrying U(1) charge labels, what the
reference computes on the sweep path:

* the step order of ``_update_two_site!``     -- TenNetLib ``src/mps/update_site.jl:27-90``
* the bond order and recorded data of ``fullsweep!`` -- ``src/mps/sweep.jl:94-196``
* the stage/noise schedule of ``dmrg!``       -- ``src/mps/dmrg.jl:148-227``
* the solver defaults of ``eig_solver``       -- ``src/base/solver.jl:23-43``
* the entropy of the mid-bond spectrum        -- ``src/mps/measure.jl:4-20``

The arithmetic of those steps lives in packages that are not part of the reference tree
(ITensorMPS.jl 0.3 ``ProjMPO``/``replacebond!``, ITensors.jl 0.9 block-sparse ``svd`` and
``truncate!``, KrylovKit.jl 0.9/0.10 ``eigsolve``; versions are compat ranges only, no
Manifest).  They are restated here from their published behaviour:

* ProjMPO product: contract v with L, W_b, W_{b+1}, R (the order does not change the result).
* ITensors truncation: global sort of all blocks' S^2, maxdim first, then discard the
  smallest while the accumulated discarded weight stays <= cutoff * sum(S^2) and more than
  mindim remain; a cut value halfway between the last kept and the first discarded weight,
  raised by 1e-3 of the last kept weight when those two are within 1e-3 relative of each
  other (degenerate multiplets are cut as a whole); every block keeps its values whose
  S^2 exceeds the cut value.
* KrylovKit Lanczos eigsolve: thick-restart Lanczos (Wu & Simon 2000) with full
  re-orthogonalisation, ``keep = (3*krylovdim + 2*converged) // 5`` Ritz vectors on restart,
  convergence when |beta * U[K-1, j]| <= tol.

Parity status: the reference ships no golden vectors (its tests assert nothing), so this
oracle is pinned against exact diagonalisation of the Heisenberg chain (tests/golden) and
against invariants; agreement with the reference itself is "parity unpinned".

Conventions (shared with the engine):
* physical charges q_s: S=1/2 with q = 2*Sz, state 0 = Up (+1), state 1 = Dn (-1);
* a link is an int array of per-basis-state charges sorted ascending, so each charge
  sector is a contiguous range;
* MPS tensor A[l, s, r] is nonzero only when q_r = q_l + q_s;
* MPO tensor W[a, b, s', s] is nonzero only when q_s' - q_s = delta_b - delta_a;
* environments L[l', a, l] / R[r', c, r] are nonzero only when q_l' = q_l + delta_a.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

FLOAT64_THRESHOLD = 1e-15  # src/base/global_variables.jl:10


# --------------------------------------------------------------------------------------
# models
# --------------------------------------------------------------------------------------

SPIN_HALF_Q = np.array([1, -1], dtype=np.int64)  # Up, Dn in units of 2*Sz


def spin_half_ops():
    sz = np.array([[0.5, 0.0], [0.0, -0.5]])
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])  # |Up><Dn|
    sm = sp.T.copy()
    eye = np.eye(2)
    return eye, sz, sp, sm


@dataclass
class MPO:
    """Dense MPO with U(1) labels.  W[i] has shape (w_{i-1}, w_i, d, d) as [a, b, s', s]."""

    W: list
    delta: list  # delta[i] = charges of MPO link i (i = 0..N), int arrays
    phys_q: np.ndarray

    @property
    def N(self):
        return len(self.W)


def heisenberg_mpo(N: int, J: float = 1.0, Jz: float | None = None, qn: bool = True) -> MPO:
    """H = sum_i J (S^x S^x + S^y S^y) + Jz S^z S^z on an open chain (five-state MPO).

    MPO states: 0 = nothing placed yet, 1 = S+ placed, 2 = S- placed, 3 = Sz placed,
    4 = term complete.  Same operator content as the OpSum built in the reference test
    ``test/test_MPS_DMRG.jl:29-33``.
    """
    if Jz is None:
        Jz = J
    eye, sz, sp, sm = spin_half_ops()
    w = 5
    bulk = np.zeros((w, w, 2, 2))
    bulk[0, 0] = eye
    bulk[0, 1] = 0.5 * J * sp
    bulk[1, 4] = sm
    bulk[0, 2] = 0.5 * J * sm
    bulk[2, 4] = sp
    bulk[0, 3] = Jz * sz
    bulk[3, 4] = sz
    bulk[4, 4] = eye
    dq = np.array([0, 2, -2, 0, 0]) if qn else np.zeros(5, dtype=np.int64)
    Ws = []
    deltas = [np.array([0])]
    for i in range(N):
        lo = [0] if i == 0 else list(range(w))
        hi = [4] if i == N - 1 else list(range(w))
        Ws.append(bulk[np.ix_(lo, hi)].copy())
        deltas.append(np.array([0]) if i == N - 1 else dq.copy())
    return MPO(Ws, deltas, SPIN_HALF_Q.copy() if qn else np.zeros(2, dtype=np.int64))


def mpo_from_terms(N: int, terms, qn: bool = True) -> MPO:
    """Finite-state-automaton MPO for a sum of two-body terms c * O_i O_j (i < j).

    ``terms``: list of (coef, opname_i, i, opname_j, j), opnames in {"Sz", "S+", "S-"}.
    Automaton states on link k (between site k-1 and site k): "start" (nothing placed,
    k < N), one pending state per (first operator, its site i) for i < k <= max j of its
    terms, and "done" (k > 0).  A pending state is carried by identities and closed into
    "done" by c * O_j at every site j of its terms.  The bond dimension is exact for this
    construction (no compression); the J1-J2 cylinder gets a few dozen states.
    """
    eye, sz, sp, sm = spin_half_ops()
    ops = {"Sz": (sz, 0), "S+": (sp, 2), "S-": (sm, -2)}
    by_first = {}
    for c, o1, i, o2, j in terms:
        if not i < j:
            raise ValueError("terms must have i < j")
        by_first.setdefault((o1, i), []).append((c, o2, j))
    jmax = {key: max(j for _, _, j in lst) for key, lst in by_first.items()}
    order = sorted(by_first, key=lambda t: (t[1], t[0]))
    links = []
    for k in range(N + 1):
        keys = []
        if k < N:
            keys.append("start")
        keys += [key for key in order if key[1] < k <= jmax[key]]
        if k > 0:
            keys.append("done")
        links.append(keys)
    Ws = []
    for s in range(N):
        li = {key: n for n, key in enumerate(links[s])}
        ri = {key: n for n, key in enumerate(links[s + 1])}
        W = np.zeros((len(li), len(ri), 2, 2))
        if "start" in li and "start" in ri:
            W[li["start"], ri["start"]] += eye
        if "done" in li and "done" in ri:
            W[li["done"], ri["done"]] += eye
        for key, lst in by_first.items():
            o1, i = key
            if i == s:
                W[li["start"], ri[key]] += ops[o1][0]
            if key in li and key in ri:
                W[li[key], ri[key]] += eye
            if key in li:
                for c, o2, j in lst:
                    if j == s:
                        W[li[key], ri["done"]] += c * ops[o2][0]
        Ws.append(W)
    deltas = []
    for keys in links:
        deltas.append(np.array([0 if (key in ("start", "done") or not qn) else ops[key[0]][1]
                                for key in keys], dtype=np.int64))
    return MPO(Ws, deltas, SPIN_HALF_Q.copy() if qn else np.zeros(2, dtype=np.int64))


def j1j2_cylinder_terms(Lx: int, Ly: int, J1: float = 1.0, J2: float = 0.5):
    """Bonds of the J1-J2 model on an Lx x Ly cylinder (periodic in y, open in x),
    snaked column-major: site = Ly * x + y.  Returns OpSum-like two-body terms."""
    def site(x, y):
        return Ly * x + (y % Ly)

    bonds = set()
    for x in range(Lx):
        for y in range(Ly):
            a = site(x, y)
            nn = [(x, y + 1)] + ([(x + 1, y)] if x + 1 < Lx else [])
            nnn = ([(x + 1, y + 1), (x + 1, y - 1)] if x + 1 < Lx else [])
            for (xx, yy) in nn:
                b = site(xx, yy)
                if a != b:
                    bonds.add((min(a, b), max(a, b), J1))
            for (xx, yy) in nnn:
                b = site(xx, yy)
                if a != b:
                    bonds.add((min(a, b), max(a, b), J2))
    terms = []
    for i, j, J in sorted(bonds):
        terms.append((J, "Sz", i, "Sz", j))
        terms.append((0.5 * J, "S+", i, "S-", j))
        terms.append((0.5 * J, "S-", i, "S+", j))
    return terms


# --------------------------------------------------------------------------------------
# MPS construction
# --------------------------------------------------------------------------------------

@dataclass
class MPS:
    A: list  # A[i] of shape (D_{i}, d, D_{i+1}) for i = 0..N-1
    links: list  # links[i] = charges of link i (i = 0..N)
    phys_q: np.ndarray
    center: int = 0  # orthogonality center (0-based site); -1 unknown

    @property
    def N(self):
        return len(self.A)

    def maxlinkdim(self):
        return max(len(q) for q in self.links)


def product_mps(states, phys_q, vectors=None) -> MPS:
    """Product-state MPS.  ``states`` are basis indices (QN case) or None when
    ``vectors`` (N x d, normalised per site) give a dense product state."""
    N = len(states) if states is not None else len(vectors)
    A = []
    links = [np.array([0])]
    q = 0
    for i in range(N):
        d = len(phys_q)
        t = np.zeros((1, d, 1))
        if vectors is not None:
            t[0, :, 0] = vectors[i]
            qn = q  # all charges equal in the no-QN case
        else:
            t[0, states[i], 0] = 1.0
            qn = q + int(phys_q[states[i]])
        A.append(t)
        q = qn
        links.append(np.array([q]))
    return MPS(A, links, np.asarray(phys_q), center=0)


def random_product_vectors(N: int, d: int, seed: int):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((N, d))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


# --------------------------------------------------------------------------------------
# environments and the effective Hamiltonian (ProjMPO restated)
# --------------------------------------------------------------------------------------

def left_env_update(L, A, W):
    """L_new[r', b, r] = sum conj(A[l', s', r']) L[l', a, l] W[a, b, s', s] A[l, s, r]."""
    t = np.tensordot(L, A, axes=([2], [0]))          # [l', a, s, r]
    t = np.tensordot(t, W, axes=([1, 2], [0, 3]))    # [l', r, b, s']
    out = np.tensordot(A.conj(), t, axes=([0, 1], [0, 3]))  # [r', r, b]
    return out.transpose(0, 2, 1).copy()


def right_env_update(R, B, W):
    """R_new[l', a, l] = sum conj(B[l', s', r']) R[r', c, r] W[a, c, s', s] B[l, s, r]."""
    t = np.tensordot(R, B, axes=([2], [2]))          # [r', c, l, s]
    t = np.tensordot(t, W, axes=([1, 3], [1, 3]))    # [r', l, a, s']
    out = np.tensordot(B.conj(), t, axes=([1, 2], [3, 0]))  # [l', l, a]
    return out.transpose(0, 2, 1).copy()


def heff2_apply(L, W1, W2, R, phi):
    """Two-site H_eff * phi, phi[l, s1, s2, r] (ProjMPO product restated)."""
    t = np.tensordot(L, phi, axes=([2], [0]))            # [l', a, s1, s2, r]
    t = np.tensordot(t, W1, axes=([1, 2], [0, 3]))       # [l', s2, r, b, s1']
    t = np.tensordot(t, W2, axes=([3, 1], [0, 3]))       # [l', r, s1', c, s2']
    t = np.tensordot(t, R, axes=([1, 3], [2, 1]))        # [l', s1', s2', r']
    return t


def heff1_apply(L, W, R, phi):
    t = np.tensordot(L, phi, axes=([2], [0]))            # [l', a, s, r]
    t = np.tensordot(t, W, axes=([1, 2], [0, 3]))        # [l', r, b, s']
    t = np.tensordot(t, R, axes=([1, 2], [2, 1]))        # [l', s', r']
    return t


def heff0_apply(L, R, C):
    """Zero-site H_eff * C for the bond matrix C[x, y] between the environments L (sites left
    of the bond) and R (sites right of it): y[x', y'] = sum L[x', a, x] C[x, y] R[y', a, y]
    (ProjMPO with nsite = 0, the reverse step of one-site TDVP)."""
    t = np.tensordot(L, C, axes=([2], [0]))               # [x', a, y]
    return np.tensordot(t, R, axes=([1, 2], [1, 2]))      # [x', y']


def heff2_flops(L_shape, W1, W2, R_shape, phi_shape):
    """Dense multiply-add count of the four-step contraction above (x2 = flops)."""
    Dl, w0, _ = L_shape
    _, d1, d2, Dr = phi_shape
    w1 = W1.shape[1]
    w2 = W2.shape[1]
    f = Dl * w0 * Dl * d1 * d2 * Dr
    f += Dl * d2 * Dr * w1 * d1 * w0 * d1
    f += Dl * Dr * d1 * w2 * d2 * w1 * d2
    f += Dl * d1 * d2 * Dr * Dr * w2
    return 2 * f


# --------------------------------------------------------------------------------------
# Lanczos eigensolver (KrylovKit eigsolve semantics restated)
# --------------------------------------------------------------------------------------

@dataclass
class EigInfo:
    matvecs: int = 0
    converged: int = 0
    numiter: int = 0
    residual: float = float("nan")


def _gs2(V, w):
    """Classical Gram-Schmidt, applied twice; returns coefficients and the residual."""
    if not V:
        return np.zeros(0, dtype=w.dtype), w
    M = np.stack(V, axis=0)
    h = M.conj() @ w
    w = w - h @ M
    h2 = M.conj() @ w
    w = w - h2 @ M
    return h + h2, w


def eigsolve_lowest(apply, x0, krylovdim=5, maxiter=2, tol=1e-14, eager=False):
    """Lowest eigenpair of a Hermitian operator by thick-restart Lanczos.

    Follows ``eig_solver`` (``src/base/solver.jl:23-43``): howmany = 1, :SR, Hermitian.
    Returns (energy, vector, EigInfo).
    """
    info = EigInfo()
    x = x0 / np.linalg.norm(x0)
    V = [x]
    w = apply(x)
    info.matvecs += 1
    h, r = _gs2(V, w)
    H = np.zeros((krylovdim + 1, krylovdim + 1), dtype=np.result_type(x0, np.float64))
    H[0, 0] = h[0].real
    beta = np.linalg.norm(r)
    numiter = 1
    D = U = None
    converged = 0
    while True:
        K = len(V)
        # K >= n: the Krylov space spans the whole vector space, the Ritz pair is exact
        exhausted = K >= x.size
        if K == krylovdim or beta <= tol or (eager and K >= 1) or exhausted:
            Hk = H[:K, :K]
            Hk = 0.5 * (Hk + Hk.conj().T)
            D, U = np.linalg.eigh(Hk)
            f = beta * U[K - 1, :]
            converged = 0
            while converged < K and abs(f[converged]) <= tol:
                converged += 1
            info.residual = abs(f[0])
            if converged >= 1 or exhausted:
                break
        if K < krylovdim:
            v = r / beta
            V.append(v)
            w = apply(v)
            info.matvecs += 1
            h, r = _gs2(V, w)
            H[: K + 1, K] = h
            H[K, : K + 1] = h.conj()
            H[K, K] = h[K].real
            beta = np.linalg.norm(r)
        else:
            if numiter == maxiter:
                break
            keep = (3 * krylovdim + 2 * converged) // 5
            M = np.stack(V, axis=0)
            V = [U[:, j] @ M for j in range(keep)]
            f = beta * U[K - 1, :]
            H = np.zeros_like(H)
            for j in range(keep):
                H[j, j] = D[j]
            # the residual r is unchanged; its coupling to Ritz vector j is f[j], which the
            # explicit Gram-Schmidt of the next expansion recomputes.
            numiter += 1
    info.converged = converged
    info.numiter = numiter
    M = np.stack(V, axis=0)
    vec = U[:, 0] @ M
    vec = vec / np.linalg.norm(vec)
    return float(D[0]), vec, info


def exponentiate(apply, t, x0, krylovdim=30, maxiter=100, tol=1e-12):
    """exp(t A) x0 for Hermitian A (``exp_solver``, ``src/base/solver.jl:66-88``, restating
    KrylovKit's ``exponentiate`` with eager Lanczos and full re-orthogonalisation).

    Step control of this restatement: the Krylov space grows one vector at a time; after
    each expansion y = exp(dt T) e1 is formed from the projected matrix T and the step is
    accepted when |dt| * beta * |y[K-1]| <= tol (or beta <= tol, or the space is
    exhausted).  If krylovdim vectors do not reach the tolerance, the largest step dt/2^j
    that does is taken and the iteration restarts from the evolved vector for the rest of
    t; at most maxiter restarts.  Returns (vector, info) with info = number of matvecs.
    """
    x = np.array(x0, dtype=np.result_type(x0, t, np.float64))
    remaining = t
    matvecs = 0
    for _ in range(maxiter):
        if remaining == 0:
            break
        nrm = np.linalg.norm(x)
        if nrm == 0:
            break
        V = [x / nrm]
        H = np.zeros((krylovdim + 1, krylovdim + 1), dtype=V[0].dtype)
        w = apply(V[0])
        matvecs += 1
        h, r = _gs2(V, w)
        H[0, 0] = h[0].real
        beta = np.linalg.norm(r)
        dt = remaining
        while True:
            K = len(V)
            Hk = H[:K, :K]
            Hk = 0.5 * (Hk + Hk.conj().T)
            lam, U = np.linalg.eigh(Hk)
            y = U @ (np.exp(dt * lam) * U[0, :].conj())
            err = abs(dt) * beta * abs(y[K - 1])
            if err <= tol or beta <= tol or K >= x.size:
                x = nrm * (y @ np.stack(V, axis=0))
                remaining = remaining - dt
                break
            if K == krylovdim:
                while err > tol and abs(dt) > 1e-300:
                    dt = dt / 2
                    y = U @ (np.exp(dt * lam) * U[0, :].conj())
                    err = abs(dt) * beta * abs(y[K - 1])
                x = nrm * (y @ np.stack(V, axis=0))
                remaining = remaining - dt
                break
            v = r / beta
            V.append(v)
            w = apply(v)
            matvecs += 1
            h, r = _gs2(V, w)
            H[: K + 1, K] = h
            H[K, : K + 1] = h.conj()
            H[K, K] = h[K].real
            beta = np.linalg.norm(r)
    return x, matvecs


# --------------------------------------------------------------------------------------
# SVD with ITensors-style global truncation
# --------------------------------------------------------------------------------------

@dataclass
class Spectrum:
    eigs: np.ndarray
    truncerr: float


def truncation_rule(P, maxdim, mindim, cutoff):
    """ITensors ``truncate!`` restated.  P: all S^2, sorted descending.

    Returns (n_kept_by_rank, truncerr, docut).  Per block, values with S^2 > docut are kept.
    """
    P = np.array(P, dtype=np.float64)
    origm = len(P)
    for n in range(origm - 1, -1, -1):
        if P[n] >= 0:
            break
        P[n] = 0.0
    n = origm
    truncerr = 0.0
    while n > maxdim:
        truncerr += P[n - 1]
        n -= 1
    scale = float(np.sum(P))
    if scale == 0.0:
        scale = 1.0
    while n > mindim and truncerr + P[n - 1] <= cutoff * scale:
        truncerr += P[n - 1]
        n -= 1
    truncerr /= scale
    if n < 1:
        n = 1
    docut = 0.0
    if n < origm:
        docut = 0.5 * (P[n - 1] + P[n])
        if abs(P[n - 1] - P[n]) < 1e-3 * P[n - 1]:
            docut += 1e-3 * P[n - 1]
    return n, truncerr, docut


def svd_blocks_truncate(blocks, maxdim, mindim, cutoff):
    """SVD of a list of dense blocks, global truncation.

    Returns per block (U_k, S_k, Vh_k) truncated, the Spectrum, and kept dims.
    """
    svds = []
    allP = []
    for M in blocks:
        if M.size == 0:
            svds.append((np.zeros((M.shape[0], 0)), np.zeros(0), np.zeros((0, M.shape[1]))))
            continue
        U, S, Vh = np.linalg.svd(M, full_matrices=False)
        svds.append((U, S, Vh))
        allP.append(S * S)
    P = np.sort(np.concatenate(allP))[::-1] if allP else np.zeros(0)
    n, truncerr, docut = truncation_rule(P, maxdim, mindim, cutoff)
    out = []
    kept = []
    for (U, S, Vh) in svds:
        k = int(np.sum(S * S > docut))
        kept.append(k)
        out.append((U[:, :k], S[:k], Vh[:k, :]))
    if sum(kept) == 0:
        # every value fell under the cut (fully degenerate spectrum at maxdim): keep the
        # largest value so that the link never becomes empty.
        best = int(np.argmax([s[1][0] if len(s[1]) else -1 for s in svds]))
        U, S, Vh = svds[best]
        out[best] = (U[:, :1], S[:1], Vh[:1, :])
        kept[best] = 1
    eigs = np.sort(np.concatenate([o[1] ** 2 for o in out]))[::-1]
    return out, Spectrum(eigs=eigs, truncerr=truncerr), kept


def split_two_site(phi, ql, qs, qr, maxdim, mindim, cutoff, ortho, normalize=True):
    """``replacebond!`` restated: SVD phi[l, s1, s2, r] per middle charge, truncate.

    Returns (A_left, A_right, qmid, spec).  ortho == "left": left tensor is U (left
    isometry), right tensor is S V^H.  ortho == "right": left is U S, right is V^H.
    The new link basis is sorted by charge ascending, then by singular value descending.
    """
    Dl, d1, d2, Dr = phi.shape
    M = phi.reshape(Dl * d1, d2 * Dr)
    qrow = (ql[:, None] + qs[None, :]).reshape(-1)
    qcol = (qr[None, :] - qs[:, None]).reshape(-1)
    charges = sorted(set(qrow.tolist()) & set(qcol.tolist()))
    blocks, rows, cols = [], [], []
    for m in charges:
        ri = np.nonzero(qrow == m)[0]
        ci = np.nonzero(qcol == m)[0]
        rows.append(ri)
        cols.append(ci)
        blocks.append(M[np.ix_(ri, ci)])
    res, spec, kept = svd_blocks_truncate(blocks, maxdim, mindim, cutoff)
    chi = sum(kept)
    Lm = np.zeros((Dl * d1, chi), dtype=phi.dtype)
    Rm = np.zeros((chi, d2 * Dr), dtype=phi.dtype)
    qmid = []
    norm = math.sqrt(sum(float(np.sum(s ** 2)) for _, s, _ in res)) if normalize else 1.0
    off = 0
    for m, ri, ci, (U, S, Vh), k in zip(charges, rows, cols, res, kept):
        if k == 0:
            continue
        Sn = S / norm
        if ortho == "left":
            Lm[np.ix_(ri, range(off, off + k))] = U
            Rm[np.ix_(range(off, off + k), ci)] = Sn[:, None] * Vh
        else:
            Lm[np.ix_(ri, range(off, off + k))] = U * Sn[None, :]
            Rm[np.ix_(range(off, off + k), ci)] = Vh
        qmid.extend([m] * k)
        off += k
    A = Lm.reshape(Dl, d1, chi)
    B = Rm.reshape(chi, d2, Dr)
    return A, B, np.array(qmid, dtype=np.int64), spec


def entropy(p):
    """von Neumann entropy of a probability vector (``src/mps/measure.jl:4-20``)."""
    p = np.asarray(p, dtype=np.float64)
    s = float(np.sum(p))
    if abs(s - 1.0) > 100 * FLOAT64_THRESHOLD:
        p = p / s
    return float(-sum(a * math.log(a) for a in p if a > 0.0))


# --------------------------------------------------------------------------------------
# sweeps (StateEnvs + fullsweep! + dmrg! restated)
# --------------------------------------------------------------------------------------

@dataclass
class SweepData:
    """Per-sweep history (``src/mps/sweep.jl:26-35``)."""

    sweepcount: int = 0
    maxchi: list = field(default_factory=list)
    energy: list = field(default_factory=list)
    entropy: list = field(default_factory=list)
    maxtruncerr: list = field(default_factory=list)
    lasteigs: list = field(default_factory=list)


def overlap_left_update(E, A, M):
    """ProjMPS2 ``_makeL!`` step (``src/mps/projmps2.jl:76-91``): E_new[r, r_M] =
    sum A[l, s, r] E[l, l_M] conj(M[l_M, s, r_M]) (psi on the first index, M on the second)."""
    t = np.tensordot(E, M.conj(), axes=([1], [0]))         # [l, s, r_M]
    return np.tensordot(A, t, axes=([0, 1], [0, 1]))       # [r, r_M]


def overlap_right_update(E, A, M):
    """ProjMPS2 ``_makeR!`` step (``src/mps/projmps2.jl:106-122``): E_new[l, l_M] =
    sum A[l, s, r] E[r, r_M] conj(M[l_M, s, r_M])."""
    t = np.tensordot(A, E, axes=([2], [0]))                # [l, s, r_M]
    return np.tensordot(t, M.conj(), axes=([1, 2], [1, 2]))  # [l, l_M]


class StateEnvs:
    """MPS + MPO environments.  ``L[i]`` contracts sites < i, ``R[i]`` sites > i.

    With ``Ms`` (``StateEnvs(psi, H, Ms; weight)``, ``src/mps/state_envs.jl:88-105``) the
    effective Hamiltonian is ProjMPO_MPS2's (``src/mps/projmpo_mps2.jl:94-101``):
    H_eff v + weight sum_k m_k <m_k|v>, with m_k the projection of M_k onto the sites being
    optimised through the overlap environments ``LM[k][i]`` / ``RM[k][i]`` (sites < i / > i)."""

    def __init__(self, psi: MPS, H: MPO, Ms=None, weight=None):
        assert psi.N == H.N
        self.psi = MPS([a.copy() for a in psi.A], [q.copy() for q in psi.links],
                       psi.phys_q.copy(), psi.center)
        self.H = H
        N = psi.N
        self.L = [None] * (N + 1)
        self.R = [None] * (N + 1)
        self.L[0] = np.ones((1, 1, 1))
        self.R[N - 1] = np.ones((1, 1, 1))
        self.lpos = 0       # L[0..lpos] valid
        self.rpos = N - 1   # R[rpos..N-1] valid
        self.matvec_flops = 0
        self.Ms = []
        self.weight = 0.0
        if Ms:
            if weight is None or weight <= 0.0:
                raise ValueError("`weight` parameter should be > 0.0 (value passed was "
                                 f"`weight={weight}`)")
            self.Ms = [[a.copy() for a in M.A] for M in Ms]
            self.weight = float(weight)
            self.LM = [[None] * (N + 1) for _ in Ms]
            self.RM = [[None] * (N + 1) for _ in Ms]
            for k, M in enumerate(Ms):
                same_l = M.links[0][0] == psi.links[0][0]
                same_r = M.links[N][0] == psi.links[N][0]
                self.LM[k][0] = np.ones((1, 1)) * float(same_l)
                self.RM[k][N - 1] = np.ones((1, 1)) * float(same_r)

    @property
    def N(self):
        return self.psi.N

    def update_h(self, H: MPO, recalc_env=True):
        """``updateH!(sysenv, H; recalcEnv)`` (``src/mps/state_envs.jl:181-212``): with
        recalc_env a new ProjMPO, every MPO environment dropped; without it (single MPO, left
        environments unset, same MPO link indices) H takes the old MPO's place and the right
        environments already built stay, so the next half sweep reads environments of the old
        MPO."""
        assert H.N == self.N
        N = self.N
        if recalc_env:
            self.H = H
            self.L = [None] * (N + 1)
            self.R = [None] * (N + 1)
            self.L[0] = np.ones((1, 1, 1))
            self.R[N - 1] = np.ones((1, 1, 1))
            self.lpos, self.rpos = 0, N - 1
            return
        assert not self.Ms and self.lpos == 0 and self.psi.center == 0
        assert all(a.shape[:2] == b.shape[:2] for a, b in zip(H.W, self.H.W))
        self.H = H

    def position(self, pos, nsite):
        """Make L[pos] and R[pos+nsite-1] valid (ProjMPO ``position!`` restated; the
        projector environments follow the same positions)."""
        while self.lpos < pos:
            i = self.lpos
            self.L[i + 1] = left_env_update(self.L[i], self.psi.A[i], self.H.W[i])
            for k, M in enumerate(self.Ms):
                self.LM[k][i + 1] = overlap_left_update(self.LM[k][i], self.psi.A[i], M[i])
            self.lpos += 1
        self.lpos = pos
        last = pos + nsite - 1
        while self.rpos > last:
            i = self.rpos
            self.R[i - 1] = right_env_update(self.R[i], self.psi.A[i], self.H.W[i])
            for k, M in enumerate(self.Ms):
                self.RM[k][i - 1] = overlap_right_update(self.RM[k][i], self.psi.A[i], M[i])
            self.rpos -= 1
        self.rpos = last

    def proj_vectors(self, pos, nsite):
        """``proj_mps`` (``src/mps/projmps2.jl:168-184``) of every M_k at the sites
        pos..pos+nsite-1: LM M_pos (M_pos+1) RM^T, in the shape of the local tensor."""
        out = []
        for k, M in enumerate(self.Ms):
            t = np.tensordot(self.LM[k][pos], M[pos].conj(), axes=([1], [0]))
            if nsite == 2:
                t = np.tensordot(t, M[pos + 1].conj(), axes=([-1], [0]))
            out.append(np.tensordot(t, self.RM[k][pos + nsite - 1], axes=([-1], [1])))
        return out

    def _add_proj(self, pos, nsite, phi, out):
        for m in self.proj_vectors(pos, nsite):
            out = out + self.weight * m * float(np.vdot(m, phi))
        return out

    def product2(self, pos, phi):
        out = heff2_apply(self.L[pos], self.H.W[pos], self.H.W[pos + 1], self.R[pos + 1], phi)
        return self._add_proj(pos, 2, phi, out) if self.Ms else out

    def product1(self, pos, phi):
        out = heff1_apply(self.L[pos], self.H.W[pos], self.R[pos], phi)
        return self._add_proj(pos, 1, phi, out) if self.Ms else out


def noise_factor(env: StateEnvs, pos):
    """Noise tensors of ``noiseterm(P, phi, ortho)`` (ITensorMPS ProjMPO; TenNetLib's own
    ProjCouplingModel version at src/mps/projcouplingmodel.jl:391-492 has the same form):
    returns functions phi -> N with drho = N N^T on the rows (ortho "left", N indexed
    [(l', s1'), (b, s2, r)]) or on the columns (ortho "right", [(s2', r'), (l, s1, b)]) of the
    two-site matrix phi.reshape(Dl d, d Dr)."""
    L, R = env.L[pos], env.R[pos + 1]
    W1, W2 = env.H.W[pos], env.H.W[pos + 1]

    def left(phi):
        Dl, d1, d2, Dr = phi.shape
        t = np.tensordot(L, phi, axes=([2], [0]))           # [l', a, s1, s2, r]
        t = np.tensordot(t, W1, axes=([1, 2], [0, 3]))      # [l', s2, r, b, s1']
        return t.transpose(0, 4, 3, 1, 2).reshape(Dl * d1, -1)

    def right(phi):
        Dl, d1, d2, Dr = phi.shape
        t = np.tensordot(phi, W2, axes=([2], [3]))          # [l, s1, r, b, c, s2']
        t = np.tensordot(t, R, axes=([2, 4], [2, 1]))       # [l, s1, b, s2', r']
        return t.transpose(3, 4, 0, 1, 2).reshape(d2 * Dr, -1)

    return left, right


def split_two_site_noise(phi, Nmat, noise, ql, qs, qr, maxdim, mindim, cutoff, ortho,
                         normalize=True):
    """``replacebond!`` with ``eigen_perturbation = noise * noiseterm`` (ITensors
    ``factorize_eigen``): per charge block the density matrix rho = M M^T + noise N N^T of the
    kept side (rows for ortho "left", columns for "right") is diagonalised, its eigenvalues
    truncated like S^2 (ITensors truncate!), the eigenvectors kept on that side and the other
    factor is U^T M (resp. M V), normalised (ITensorMPS replacebond!)."""
    Dl, d1, d2, Dr = phi.shape
    M = phi.reshape(Dl * d1, d2 * Dr)
    qrow = (ql[:, None] + qs[None, :]).reshape(-1)
    qcol = (qr[None, :] - qs[:, None]).reshape(-1)
    side = qrow if ortho == "left" else qcol
    # every charge of the kept side: rho has blocks where only the noise term reaches, and
    # those sectors may enter the new link (that is how the perturbation grows the basis)
    charges = sorted(set(side.tolist()))
    Ms = M if ortho == "left" else M.T
    evs, vecs, idx = [], [], []
    for m in charges:
        ii = np.nonzero(side == m)[0]
        rho = Ms[ii] @ Ms[ii].T + noise * (Nmat[ii] @ Nmat[ii].T)
        w, U = np.linalg.eigh(0.5 * (rho + rho.T))
        order = np.argsort(-w, kind="stable")
        evs.append(np.maximum(w[order], 0.0))
        vecs.append(U[:, order])
        idx.append(ii)
    P = np.sort(np.concatenate(evs))[::-1]
    _, truncerr, docut = truncation_rule(P, maxdim, mindim, cutoff)
    kept = [int(np.sum(e > docut)) for e in evs]
    if sum(kept) == 0:
        kept[int(np.argmax([e[0] if len(e) else -1 for e in evs]))] = 1
    chi = sum(kept)
    Ke = np.zeros((Ms.shape[0], chi))
    qmid, eigs, off = [], [], 0
    for m, ii, U, e, k in zip(charges, idx, vecs, evs, kept):
        if k == 0:
            continue
        Ke[np.ix_(ii, range(off, off + k))] = U[:, :k]
        qmid.extend([m] * k)
        eigs.extend(e[:k])
        off += k
    other = Ke.T @ Ms                      # k x (other side)
    if normalize:
        other = other / np.linalg.norm(other)
    if ortho == "left":
        A = Ke.reshape(Dl, d1, chi)
        B = other.reshape(chi, d2, Dr)
    else:
        A = other.T.reshape(Dl, d1, chi)
        B = Ke.T.reshape(chi, d2, Dr)
    spec = Spectrum(eigs=np.sort(np.array(eigs))[::-1], truncerr=truncerr)
    return A, B, np.array(qmid, dtype=np.int64), spec


def update_two_site(env: StateEnvs, pos, ortho, maxdim, mindim, cutoff, krylovdim, maxiter,
                    tol, normalize=True, noise=0.0):
    """``_update_two_site!`` (``src/mps/update_site.jl:27-90``) for the eigensolver, with the
    density-matrix noise term when noise > 0 (``:59-62``)."""
    psi = env.psi
    phi = np.tensordot(psi.A[pos], psi.A[pos + 1], axes=([2], [0]))
    env.position(pos, 2)
    shape = phi.shape

    def apply(v):
        return env.product2(pos, v.reshape(shape)).reshape(-1)

    energy, vec, info = eigsolve_lowest(apply, phi.reshape(-1), krylovdim, maxiter, tol)
    phi = vec.reshape(shape)
    if normalize:
        phi = phi / np.linalg.norm(phi)
    if abs(noise) > FLOAT64_THRESHOLD:
        left, right = noise_factor(env, pos)
        Nmat = left(phi) if ortho == "left" else right(phi)
        A, B, qmid, spec = split_two_site_noise(phi, Nmat, noise, psi.links[pos], psi.phys_q,
                                                psi.links[pos + 2], maxdim, mindim, cutoff,
                                                ortho, normalize)
    else:
        A, B, qmid, spec = split_two_site(phi, psi.links[pos], psi.phys_q, psi.links[pos + 2],
                                          maxdim, mindim, cutoff, ortho, normalize)
    psi.A[pos] = A
    psi.A[pos + 1] = B
    psi.links[pos + 1] = qmid
    psi.center = pos + 1 if ortho == "left" else pos
    # environments that contain the changed sites become invalid
    env.lpos = min(env.lpos, pos)
    env.rpos = max(env.rpos, pos + 1)
    return energy, spec, info


def halfsweep_done(N, pos, nsite, ortho):
    """``halfsweep_done`` (``src/mps/update_site.jl:13-23``), 0-based positions."""
    if pos == 0 and ortho == "right":
        return True
    if pos == N - 1 and ortho == "left" and nsite == 1:
        return True
    if pos == N - 2 and ortho == "left" and nsite == 2:
        return True
    return False


def update_two_site_tdvp(env: StateEnvs, pos, ortho, time_step, maxdim, mindim, cutoff,
                         krylovdim=30, maxiter=100, tol=1e-12, normalize=True):
    """``_update_two_site!`` with ``exp_solver`` and ``reverse_step = true``
    (``src/mps/update_site.jl:27-90``): forward two-site evolution by ``time_step``,
    ``replacebond!``, then the one-site backward evolution by ``-time_step`` on the new
    orthogonality center unless the half sweep is done."""
    psi = env.psi
    N = psi.N
    phi = np.tensordot(psi.A[pos], psi.A[pos + 1], axes=([2], [0]))
    env.position(pos, 2)
    shape = phi.shape

    def apply2(v):
        return env.product2(pos, v.reshape(shape)).reshape(-1)

    vec, _ = exponentiate(apply2, time_step, phi.reshape(-1), krylovdim, maxiter, tol)
    if normalize:
        vec = vec / np.linalg.norm(vec)
    energy = float(np.real(np.vdot(vec, apply2(vec))))
    phi = vec.reshape(shape)
    A, B, qmid, spec = split_two_site(phi, psi.links[pos], psi.phys_q, psi.links[pos + 2],
                                      maxdim, mindim, cutoff, ortho, normalize)
    psi.A[pos] = A
    psi.A[pos + 1] = B
    psi.links[pos + 1] = qmid
    psi.center = pos + 1 if ortho == "left" else pos
    env.lpos = min(env.lpos, pos)
    env.rpos = max(env.rpos, pos + 1)
    if not halfsweep_done(N, pos, 2, ortho):
        p1 = pos + 1 if ortho == "left" else pos
        env.position(p1, 1)
        t1 = psi.A[p1]
        sh1 = t1.shape

        def apply1(v):
            return heff1_apply(env.L[p1], env.H.W[p1], env.R[p1], v.reshape(sh1)).reshape(-1)

        v1, _ = exponentiate(apply1, -time_step, t1.reshape(-1), krylovdim, maxiter, tol)
        if normalize:
            v1 = v1 / np.linalg.norm(v1)
        energy = float(np.real(np.vdot(v1, apply1(v1))))
        psi.A[p1] = v1.reshape(sh1)
        env.lpos = min(env.lpos, p1)
        env.rpos = max(env.rpos, p1)
    return energy, spec


def tdvp_sweep(env: StateEnvs, swdata: SweepData, tau, maxdim, cutoff, mindim=1, krylovdim=30,
               maxiter=100, tol=1e-12, normalize=True, nsite=2):
    """``tdvpsweep!`` (``src/mps/tdvp.jl:247-277``): a full sweep with ``exp_solver`` at time
    step tau/2 and reverse steps, two-site (nsite = 2) or one-site (nsite = 1: the sweep
    order of ``fullsweep1``, the one-site update with its zero-site reverse step)."""
    N = env.N
    assert env.psi.center == 0
    if nsite == 1:
        swdata.sweepcount += 1
        energy = float("nan")
        maxtruncerr = 0.0
        lasteigs = [None] * (N - 1)
        for q in range(N):
            energy, spec, _ = update_one_site(env, q, "left", maxdim, mindim, cutoff, krylovdim,
                                              maxiter, tol, normalize, 0.0, 0.5 * tau)
            maxtruncerr = max(spec.truncerr, maxtruncerr)
        for q in range(N - 1, -1, -1):
            energy, spec, _ = update_one_site(env, q, "right", maxdim, mindim, cutoff, krylovdim,
                                              maxiter, tol, normalize, 0.0, 0.5 * tau)
            if q >= 1:
                lasteigs[q - 1] = spec.eigs
            maxtruncerr = max(spec.truncerr, maxtruncerr)
        swdata.maxchi.append(env.psi.maxlinkdim())
        swdata.energy.append(energy)
        mid = lasteigs[N // 2 - 1]
        swdata.entropy.append(entropy(mid / np.sum(mid)))
        swdata.maxtruncerr.append(maxtruncerr)
        swdata.lasteigs = lasteigs
        return energy
    swdata.sweepcount += 1
    energy = float("nan")
    maxtruncerr = 0.0
    lasteigs = [None] * (N - 1)
    for b in range(N - 1):
        energy, spec = update_two_site_tdvp(env, b, "left", 0.5 * tau, maxdim, mindim, cutoff,
                                            krylovdim, maxiter, tol, normalize)
        maxtruncerr = max(maxtruncerr, spec.truncerr)
    for b in range(N - 2, -1, -1):
        energy, spec = update_two_site_tdvp(env, b, "right", 0.5 * tau, maxdim, mindim, cutoff,
                                            krylovdim, maxiter, tol, normalize)
        lasteigs[b] = spec.eigs
        maxtruncerr = max(maxtruncerr, spec.truncerr)
    swdata.maxchi.append(env.psi.maxlinkdim())
    swdata.energy.append(energy)
    mid = lasteigs[N // 2 - 1]
    swdata.entropy.append(entropy(mid / np.sum(mid)))
    swdata.maxtruncerr.append(maxtruncerr)
    swdata.lasteigs = lasteigs
    return energy


def expect_local(psi: MPS, op):
    """<psi| op_i |psi> for every site i (``measure(T, psi, opstr)``, restated by moving the
    orthogonality center with dense QR; ``src/mps/measure.jl:150-177``)."""
    N = psi.N
    # left-canonicalise a copy site by site; the center then runs left to right
    A = [a.copy() for a in psi.A]
    # bring to right-canonical form first (copy may already be, be safe)
    for i in range(N - 1, 0, -1):
        Dl, d, Dr = A[i].shape
        M = A[i].reshape(Dl, d * Dr)
        Q, R = np.linalg.qr(M.T.conj())
        A[i] = Q.T.conj().reshape(-1, d, Dr)
        A[i - 1] = np.tensordot(A[i - 1], R.T.conj(), axes=([2], [0]))
    out = np.zeros(N)
    for i in range(N):
        c = A[i]
        out[i] = float(np.real(np.einsum("lsr,ts,ltr->", c.conj(), op, c)))
        if i < N - 1:
            Dl, d, Dr = c.shape
            Q, R = np.linalg.qr(c.reshape(Dl * d, Dr))
            A[i] = Q.reshape(Dl, d, -1)
            A[i + 1] = np.tensordot(R, A[i + 1], axes=([1], [0]))
    return out


def inner(a: MPS, b: MPS):
    """<a|b> of two MPS on the same sites by dense transfer matrices, left to right (the
    ITensorMPS ``inner(a, b)`` that users of TenNetLib call on its states; the library itself
    calls no overlap on the sweep path).  A float for real states, else a complex."""
    E = np.ones((1, 1))
    for x, y in zip(a.A, b.A):
        E = np.einsum("ab,asc,bsd->cd", E, x.conj(), y)
    v = E[0, 0]
    return complex(v) if np.iscomplexobj(E) else float(v)


def fullsweep(env: StateEnvs, swdata: SweepData, maxdim, cutoff, mindim=1, krylovdim=5,
              maxiter=2, tol=1e-14, normalize=True, noise=0.0):
    """``fullsweep!`` with nsite = 2 (``src/mps/sweep.jl:94-196``)."""
    N = env.N
    assert env.psi.center == 0, "sweep starts with the orthogonality center on site 1"
    swdata.sweepcount += 1
    energy = float("nan")
    maxtruncerr = 0.0
    lasteigs = [None] * (N - 1)
    for b in range(N - 1):
        energy, spec, _ = update_two_site(env, b, "left", maxdim, mindim, cutoff, krylovdim,
                                          maxiter, tol, normalize, noise)
        maxtruncerr = max(spec.truncerr, maxtruncerr)
    for b in range(N - 2, -1, -1):
        energy, spec, _ = update_two_site(env, b, "right", maxdim, mindim, cutoff, krylovdim,
                                          maxiter, tol, normalize, noise)
        lasteigs[b] = spec.eigs
        maxtruncerr = max(spec.truncerr, maxtruncerr)
    swdata.maxchi.append(env.psi.maxlinkdim())
    swdata.energy.append(energy)
    mid = lasteigs[N // 2 - 1]
    swdata.entropy.append(entropy(mid / np.sum(mid)))
    swdata.maxtruncerr.append(maxtruncerr)
    swdata.lasteigs = lasteigs
    if swdata.sweepcount > 1:
        return swdata.energy[-1] - swdata.energy[-2], swdata.entropy[-1] - swdata.entropy[-2]
    return float("nan"), float("nan")


def update_one_site(env: StateEnvs, pos, ortho, maxdim, mindim, cutoff, krylovdim, maxiter,
                    tol, normalize=True, noise=0.0, time_step=None):
    """``_update_one_site!`` (``src/mps/update_site.jl:94-190``): solve the one-site problem
    at the orthogonality center (time_step None: the eigensolver; else ``exp_solver``,
    exp(time_step H_eff) phi); unless the half sweep is done, SVD the tensor with the link
    toward the next site on the V side (ITensors truncation), keep U at pos and multiply S V
    into the next site -- with a time step after evolving that bond matrix by -time_step
    under the zero-site H_eff (``reverse_step``, ``:175-182``).  With noise > 0
    (``:135-152``) the solved tensor times the next site is split as a two-site tensor at
    pos0 (pos for "left", pos - 1 for "right") with the density-matrix perturbation of that
    bond."""
    psi = env.psi
    N = psi.N
    assert psi.center == pos
    env.position(pos, 1)
    phi = psi.A[pos]
    shape = phi.shape

    def apply(v):
        return env.product1(pos, v.reshape(shape)).reshape(-1)

    if time_step is None:
        energy, vec, info = eigsolve_lowest(apply, phi.reshape(-1), krylovdim, maxiter, tol)
    else:
        if abs(noise) > FLOAT64_THRESHOLD:
            raise ValueError("`updatePosition()` :: `noise` cannot be greater than zero for "
                             "`reverse_step=true` !!")
        vec, info = exponentiate(apply, time_step, phi.reshape(-1), krylovdim, maxiter, tol)
    phi = vec.reshape(shape)
    if normalize:
        phi = phi / np.linalg.norm(phi)
    if time_step is not None:
        energy = float(np.real(np.vdot(phi.reshape(-1), apply(phi.reshape(-1)))))
    if halfsweep_done(N, pos, 1, ortho):
        psi.A[pos] = phi
        env.lpos = min(env.lpos, pos)
        env.rpos = max(env.rpos, pos)
        return energy, Spectrum(eigs=np.zeros(0), truncerr=0.0), info
    if abs(noise) > FLOAT64_THRESHOLD:
        if ortho == "left":
            pos0 = pos
            phi2 = np.tensordot(phi, psi.A[pos + 1], axes=([2], [0]))
        else:
            pos0 = pos - 1
            phi2 = np.tensordot(psi.A[pos - 1], phi, axes=([2], [0]))
        env.position(pos0, 2)
        left, right = noise_factor(env, pos0)
        Nmat = left(phi2) if ortho == "left" else right(phi2)
        A, B, qmid, spec = split_two_site_noise(phi2, Nmat, noise, psi.links[pos0], psi.phys_q,
                                                psi.links[pos0 + 2], maxdim, mindim, cutoff,
                                                ortho, normalize)
        psi.A[pos0] = A
        psi.A[pos0 + 1] = B
        psi.links[pos0 + 1] = qmid
        psi.center = pos0 + 1 if ortho == "left" else pos0
        env.lpos = min(env.lpos, pos0)
        env.rpos = max(env.rpos, pos0 + 1)
        return energy, spec, info
    ql, qs, qr = psi.links[pos], psi.phys_q, psi.links[pos + 1]
    Dl, d, Dr = shape
    if ortho == "left":
        # (l, s) | r blocked by the charge of r
        M = phi.reshape(Dl * d, Dr)
        qrow = (ql[:, None] + qs[None, :]).reshape(-1)
        qcol = qr
    else:
        # l | (s, r) blocked by the charge of l
        M = phi.reshape(Dl, d * Dr)
        qrow = ql
        qcol = (qr[None, :] - qs[:, None]).reshape(-1)
    charges = sorted(set(qrow.tolist()) & set(qcol.tolist()))
    rows = [np.nonzero(qrow == m)[0] for m in charges]
    cols = [np.nonzero(qcol == m)[0] for m in charges]
    blocks = [M[np.ix_(ri, ci)] for ri, ci in zip(rows, cols)]
    res, spec, kept = svd_blocks_truncate(blocks, maxdim, mindim, cutoff)
    chi = sum(kept)
    norm = math.sqrt(sum(float(np.sum(S ** 2)) for _, S, _ in res)) if normalize else 1.0
    Lm = np.zeros((M.shape[0], chi), dtype=M.dtype)
    Rm = np.zeros((chi, M.shape[1]), dtype=M.dtype)
    qnew = []
    off = 0
    for m, ri, ci, (U, S, Vh), k in zip(charges, rows, cols, res, kept):
        if k == 0:
            continue
        Sn = S / norm
        if ortho == "left":
            Lm[np.ix_(ri, range(off, off + k))] = U
            Rm[np.ix_(range(off, off + k), ci)] = Sn[:, None] * Vh
        else:
            Lm[np.ix_(ri, range(off, off + k))] = U * Sn[None, :]
            Rm[np.ix_(range(off, off + k), ci)] = Vh
        qnew.extend([m] * k)
        off += k
    qnew = np.array(qnew, dtype=np.int64)
    if time_step is not None:
        # reverse step: the bond matrix C evolves by -time_step under the zero-site H_eff;
        # the environment on the side of the new site includes it
        W = env.H.W[pos]
        if ortho == "left":
            Lx = left_env_update(env.L[pos], Lm.reshape(Dl, d, chi), W)
            Rx = env.R[pos]
            C = Rm
        else:
            Lx = env.L[pos]
            Rx = right_env_update(env.R[pos], Rm.reshape(chi, d, Dr), W)
            C = Lm

        def apply0(v):
            return heff0_apply(Lx, Rx, v.reshape(C.shape)).reshape(-1)

        c, nmv = exponentiate(apply0, -time_step, C.reshape(-1), krylovdim, maxiter, tol)
        info += nmv
        if normalize:
            c = c / np.linalg.norm(c)
        energy = float(np.real(np.vdot(c, apply0(c))))
        if ortho == "left":
            Rm = c.reshape(C.shape)
        else:
            Lm = c.reshape(C.shape)
    if ortho == "left":
        psi.A[pos] = Lm.reshape(Dl, d, chi)
        psi.A[pos + 1] = np.tensordot(Rm, psi.A[pos + 1], axes=([1], [0]))
        psi.links[pos + 1] = qnew
        psi.center = pos + 1
        nxt = pos + 1
    else:
        psi.A[pos] = Rm.reshape(chi, d, Dr)
        psi.A[pos - 1] = np.tensordot(psi.A[pos - 1], Lm, axes=([2], [0]))
        psi.links[pos] = qnew
        psi.center = pos - 1
        nxt = pos - 1
    env.lpos = min(env.lpos, pos, nxt)
    env.rpos = max(env.rpos, pos, nxt)
    return energy, spec, info


def fullsweep1(env: StateEnvs, swdata: SweepData, maxdim, cutoff, mindim=1, krylovdim=5,
               maxiter=2, tol=1e-14, normalize=True, noise=0.0):
    """``fullsweep!`` with nsite = 1 (``src/mps/sweep.jl:94-196``): sites 1..N moving right,
    then N..1 moving left; lasteigs[bond] from the left-moving update at site bond + 1."""
    N = env.N
    assert env.psi.center == 0
    swdata.sweepcount += 1
    energy = float("nan")
    maxtruncerr = 0.0
    lasteigs = [None] * (N - 1)
    for q in range(N):
        energy, spec, _ = update_one_site(env, q, "left", maxdim, mindim, cutoff, krylovdim,
                                          maxiter, tol, normalize, noise)
        maxtruncerr = max(spec.truncerr, maxtruncerr)
    for q in range(N - 1, -1, -1):
        energy, spec, _ = update_one_site(env, q, "right", maxdim, mindim, cutoff, krylovdim,
                                          maxiter, tol, normalize, noise)
        if q >= 1:
            lasteigs[q - 1] = spec.eigs
        maxtruncerr = max(spec.truncerr, maxtruncerr)
    swdata.maxchi.append(env.psi.maxlinkdim())
    swdata.energy.append(energy)
    mid = lasteigs[N // 2 - 1]
    swdata.entropy.append(entropy(mid / np.sum(mid)))
    swdata.maxtruncerr.append(maxtruncerr)
    swdata.lasteigs = lasteigs
    if swdata.sweepcount > 1:
        return swdata.energy[-1] - swdata.energy[-2], swdata.entropy[-1] - swdata.entropy[-2]
    return float("nan"), float("nan")


def dynamic_sweep(env: StateEnvs, swdata: SweepData, maxdim, cutoff, eigthreshold=1e-12,
                  tau=None, mindim=1, krylovdim=None, maxiter=None, tol=None, normalize=True):
    """The sweep of ``dynamic_fullsweep!`` after its first one (``src/mps/sweep.jl:284-355``;
    the first sweep and every extendat-th open with ``krylov_extend!``, not restated here):
    bond b (0-based, between sites b and b + 1) takes a one-site update when the smallest
    kept eigenvalue of swdata.lasteigs[b] is below eigthreshold or its link dimension is at
    maxdim, else a two-site update, left to right and back; a one-site update at the end bond
    adds the update of the end site (``:314-316``, ``:333-335``).  ``lasteigs`` is shared
    between the halves, so the right half decides on the left half's spectra.  tau None: the
    eigensolver; else ``exp_solver`` at tau/2 with reverse steps (``tdvpsweep!``,
    ``src/mps/tdvp.jl:256-260``).  Returns the choices (left half, right half by bond)."""
    N = env.N
    assert env.psi.center == 0
    if krylovdim is None:
        krylovdim = 5 if tau is None else 30
    if maxiter is None:
        maxiter = 2 if tau is None else 100
    if tol is None:
        tol = 1e-14 if tau is None else 1e-12
    step = None if tau is None else 0.5 * tau

    def update(pos, nsite, ortho):
        if nsite == 1:
            e, spec, _ = update_one_site(env, pos, ortho, maxdim, mindim, cutoff, krylovdim,
                                         maxiter, tol, normalize, 0.0, step)
        elif tau is None:
            e, spec, _ = update_two_site(env, pos, ortho, maxdim, mindim, cutoff, krylovdim,
                                         maxiter, tol, normalize)
        else:
            e, spec = update_two_site_tdvp(env, pos, ortho, step, maxdim, mindim, cutoff,
                                           krylovdim, maxiter, tol, normalize)
        return e, spec

    def pick(b):
        return 1 if (swdata.lasteigs[b][-1] < eigthreshold
                     or len(env.psi.links[b + 1]) >= maxdim) else 2

    swdata.sweepcount += 1
    energy = float("nan")
    maxtruncerr = 0.0
    lasteigs = [None] * (N - 1)
    left, right = [0] * (N - 1), [0] * (N - 1)
    for b in range(N - 1):
        ns = left[b] = pick(b)
        energy, spec = update(b, ns, "left")
        lasteigs[b] = spec.eigs
        maxtruncerr = max(spec.truncerr, maxtruncerr)
        if ns == 1 and b == N - 2:
            energy, _ = update(N - 1, 1, "left")
    swdata.lasteigs = lasteigs
    for b in range(N - 2, -1, -1):
        ns = right[b] = pick(b)
        energy, spec = update(b + 1 if ns == 1 else b, ns, "right")
        lasteigs[b] = spec.eigs
        maxtruncerr = max(spec.truncerr, maxtruncerr)
        if ns == 1 and b == 0:
            energy, _ = update(0, 1, "right")
    swdata.maxchi.append(env.psi.maxlinkdim())
    swdata.energy.append(energy)
    mid = lasteigs[N // 2 - 1]
    swdata.entropy.append(entropy(mid / np.sum(mid)))
    swdata.maxtruncerr.append(maxtruncerr)
    swdata.lasteigs = lasteigs
    return left, right


def dmrg(psi0: MPS, H: MPO, maxdim, nsweeps, cutoff, krylovdim=5, maxiter=2, tol=1e-14,
         mindim=1):
    """``dmrg!`` stage loop without noise (``src/mps/dmrg.jl:148-227``)."""
    env = StateEnvs(psi0, H)
    sw = SweepData()
    if np.isscalar(cutoff):
        cutoff = [cutoff] * len(nsweeps)
    for ii in range(len(nsweeps)):
        for _ in range(nsweeps[ii]):
            fullsweep(env, sw, maxdim[ii], cutoff[ii], mindim, krylovdim, maxiter, tol)
    return sw, env


# --------------------------------------------------------------------------------------
# dense <-> charge-sector helpers used by the tests
# --------------------------------------------------------------------------------------

def sectors(q):
    """(charges, dims, offsets) of a sorted link charge array."""
    q = np.asarray(q)
    ch, idx, cnt = np.unique(q, return_index=True, return_counts=True)
    return ch, cnt, idx


def random_qn_link(charges, dims):
    return np.repeat(np.asarray(charges, dtype=np.int64), np.asarray(dims, dtype=np.int64))


def qn_mask3(ql, qs, qr):
    return (ql[:, None, None] + qs[None, :, None]) == qr[None, None, :]


def qn_mask_env(qb, delta, qk):
    return qb[:, None, None] == (qk[None, None, :] + delta[None, :, None])


def random_qn_tensor(rng, ql, qs, qr, dtype=np.float64):
    t = rng.standard_normal((len(ql), len(qs), len(qr)))
    if dtype == np.complex128:
        t = t + 1j * rng.standard_normal(t.shape)
    return t * qn_mask3(ql, qs, qr)


def random_env(rng, qlink, delta, hermitian=True):
    """Random environment tensor E[x', a, x] respecting charges; each a-slice symmetric
    when the MPO state is its own conjugate partner is not required for tests."""
    D = len(qlink)
    w = len(delta)
    t = rng.standard_normal((D, w, D))
    return t * qn_mask_env(qlink, delta, qlink)
