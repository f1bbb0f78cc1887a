"""TTN measurements (measure(T, psi, opstr[, pos]; sites) and the multi-site product form,
src/ttn/measure_ttn.jl:12-170) against the dense state of the oracle's TTN.

Tolerance 1e-12 (single- and multi-site expectation values of a normalised state).  A
three-body Hamiltonian term (factors on three legs of a node) is swept against the oracle
and the dense spectrum: per sweep energies 1e-10, ground energy 1e-10."""
import numpy as np
import pytest

from oracle import ttn_oracle as T

pytestmark = pytest.mark.gpu
N = 12
SZ = np.diag([0.5, -0.5])
SX = np.array([[0.0, 0.5], [0.5, 0.0]])


def _dense_expect(psi_o, ops):
    v = T.ttn_to_dense(psi_o)
    v = v / np.linalg.norm(v)
    H = T.dense_hamiltonian(N, [(1.0, [(s, m) for s, m in sorted(ops.items())])])
    return float(v @ H @ v)


def test_local_and_product_expectations_match_dense(tn, ctx):
    po = T.random_ttn(N, 8, 3)
    pg = tn.ttn.TTN(po.adj, po.site_nodes, 2, po.tensors, po.center, ctx)
    sz = tn.ttn.measure(pg, "Sz")
    ref = [_dense_expect(po, {i: SZ}) for i in range(N)]
    assert np.abs(np.array(sz) - np.array(ref)).max() < 1e-12
    assert abs(tn.ttn.measure(pg, "Sx", pos=3) - _dense_expect(po, {3: SX})) < 1e-12
    assert np.allclose(tn.ttn.measure(pg, SX, sites=[0, 7]),
                       [_dense_expect(po, {0: SX}), _dense_expect(po, {7: SX})], atol=1e-12)
    for pairs in ([("Sz", 1), ("Sz", 10)], [("Sx", 0), ("Sx", 11)], [("S+", 2), ("S-", 3)],
                  [("S+", 4), ("S-", 4), ("Sz", 9)], [("Sz", 6)]):
        ops = {}
        for name, site in pairs:
            m = {"Sz": SZ, "Sx": SX, "S+": np.array([[0.0, 1.0], [0.0, 0.0]]),
                 "S-": np.array([[0.0, 0.0], [1.0, 0.0]])}[name]
            ops[site] = ops[site] @ m if site in ops else m
        assert abs(tn.ttn.measure(pg, pairs) - _dense_expect(po, ops)) < 1e-12, pairs
    with pytest.raises(ValueError):
        tn.ttn.measure(pg, "Q")
    # strings over three and more subtrees of a node (chained factors)
    for pairs in ([("Sx", 0), ("Sz", 5), ("Sx", 11)],
                  [("Sz", 0), ("Sz", 3), ("Sz", 6), ("Sz", 9)]):
        ops = {site: {"Sz": SZ, "Sx": SX}[name] for name, site in pairs}
        assert abs(tn.ttn.measure(pg, pairs) - _dense_expect(po, ops)) < 1e-12, pairs


def test_three_body_terms_sweep_to_exact(tn, ctx):
    """Heisenberg chain plus three-body terms 0.3 Sz_i Sz_{i+1} Sz_{i+2} (and a four-body
    one): products whose factors sit on three and more legs of a node."""
    terms = T.heisenberg_terms(N)
    terms += [(0.3, [(i, SZ), (i + 1, SZ), (i + 2, SZ)]) for i in range(N - 2)]
    terms += [(0.2, [(0, SX), (4, SX), (8, SX), (11, SX)])]
    ev = np.linalg.eigvalsh(T.dense_hamiltonian(N, terms))
    path = tn.ttn.default_sweeppath(N)
    po = T.random_ttn(N, 64, 5)
    eo = T.StateEnvsTTN(po, terms)
    eg = tn.ttn.StateEnvsTTN(tn.ttn.TTN(po.adj, po.site_nodes, 2, po.tensors, po.center, ctx),
                             tn.ttn.CouplingModel(terms, N))
    x = np.random.default_rng(1).standard_normal(po.tensors[po.center].shape)
    ref = eo.product(x)
    assert np.linalg.norm(eg.product(x) - ref) <= 1e-12 * np.linalg.norm(ref)
    so, sg = T.SweepDataTTN(), tn.ttn.SweepDataTTN()
    for _ in range(6):
        T.fullsweep(eo, path, so, maxdim=64)
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, maxdim=64, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
    assert abs(sg.energy[-1] - ev[0]) < 1e-9
