"""TTN measurements (measure(T, psi, opstr[, pos]; sites) and the multi-site product form,
src/ttn/measure_ttn.jl:12-170) against the dense state of the oracle's TTN.

Tolerance 1e-12 (single- and two-point expectation values of a normalised state).  Strings
whose sites span more than two subtrees of a node are refused (TenNetError): the engine's
term groups act with at most two factors at a node."""
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
    # a string over more than two subtrees of a node is outside the engine's term groups
    with pytest.raises(tn.TenNetError):
        tn.ttn.measure(pg, [("Sx", 0), ("Sz", 5), ("Sx", 11)])
