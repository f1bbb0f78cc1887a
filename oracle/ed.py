"""Exact diagonalisation used to pin the oracle (TEST INFRASTRUCTURE ONLY).

Builds sparse spin-1/2 Hamiltonians from two-body terms in a fixed total-S^z sector and
returns the lowest eigenvalue with scipy's ARPACK Lanczos.  Independent of every
tensor-network routine, so agreement with it pins the DMRG oracle's arithmetic.
"""
from __future__ import annotations

import itertools

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla


def heisenberg_chain_terms(N, J=1.0):
    terms = []
    for i in range(N - 1):
        terms.append((J, "Sz", i, "Sz", i + 1))
        terms.append((0.5 * J, "S+", i, "S-", i + 1))
        terms.append((0.5 * J, "S-", i, "S+", i + 1))
    return terms


def sector_basis(N, nup):
    states = []
    for ups in itertools.combinations(range(N), nup):
        s = 0
        for u in ups:
            s |= 1 << u
        states.append(s)
    return np.array(sorted(states), dtype=np.int64)


def sector_hamiltonian(N, terms, nup):
    """(basis, H): the sparse Hamiltonian in the sector with ``nup`` up spins.

    Bit i of a basis state is 1 when site i is Up.  S+ S- style terms conserve S^z.
    """
    basis = sector_basis(N, nup)
    index = {int(s): n for n, s in enumerate(basis)}
    rows, cols, vals = [], [], []
    diag = np.zeros(len(basis))
    for c, o1, i, o2, j in terms:
        for n, s in enumerate(basis):
            s = int(s)
            bi = (s >> i) & 1
            bj = (s >> j) & 1
            if o1 == "Sz" and o2 == "Sz":
                diag[n] += c * (0.5 if bi else -0.5) * (0.5 if bj else -0.5)
            elif o1 == "S+" and o2 == "S-":
                if bi == 0 and bj == 1:
                    t = s | (1 << i)
                    t &= ~(1 << j)
                    rows.append(index[t]); cols.append(n); vals.append(c)
            elif o1 == "S-" and o2 == "S+":
                if bi == 1 and bj == 0:
                    t = s & ~(1 << i)
                    t |= 1 << j
                    rows.append(index[t]); cols.append(n); vals.append(c)
            else:
                raise ValueError((o1, o2))
    H = sp.coo_matrix((vals, (rows, cols)), shape=(len(basis), len(basis))).tocsr()
    return basis, H + sp.diags(diag)


def ground_energy(N, terms, nup=None, k=1):
    """Lowest eigenvalue(s) in the sector with ``nup`` up spins (default N//2)."""
    if nup is None:
        nup = N // 2
    basis, H = sector_hamiltonian(N, terms, nup)
    if len(basis) < 400:
        w = np.linalg.eigvalsh(H.toarray())
        return w[:k] if k > 1 else float(w[0])
    w = sla.eigsh(H, k=max(k, 1), which="SA", tol=1e-14, return_eigenvectors=False)
    w = np.sort(w)
    return w[:k] if k > 1 else float(w[0])


def quench_sz(N, terms, up_sites, times):
    """<S^z_i(t)> after a quench from the product state with the given sites Up, by exact
    real-time evolution exp(-i H t) (scipy expm_multiply) in its S^z sector.  Returns one
    list of N values per time."""
    up = set(int(i) for i in up_sites)
    basis, H = sector_hamiltonian(N, terms, len(up))
    s0 = sum(1 << i for i in up)
    v = np.zeros(len(basis), dtype=np.complex128)
    v[int(np.searchsorted(basis, s0))] = 1.0
    sz = np.array([[0.5 if (int(b) >> i) & 1 else -0.5 for b in basis] for i in range(N)])
    out = []
    t_prev = 0.0
    for t in times:
        v = sla.expm_multiply(-1j * (t - t_prev) * H.tocsc(), v)
        t_prev = t
        p = np.abs(v) ** 2
        out.append([float(sz[i] @ p) for i in range(N)])
    return out
