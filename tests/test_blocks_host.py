"""Host helpers of the block-sparse MPS boundary: dense_to_blocks / blocks_to_dense round
trip on random charge-conserving site tensors, and the block count equals the number of
entries the charges allow."""
import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import random_qn_mps


def test_dense_blocks_round_trip(tn):
    mps = random_qn_mps(7, np.random.default_rng(11), maxsec_dim=3)
    for i, t in enumerate(mps.A):
        ql, qr = mps.links[i], mps.links[i + 1]
        b = tn.dense_to_blocks(t, ql, mps.phys_q, qr)
        assert b.size == int(O.qn_mask3(ql, mps.phys_q, qr).sum())
        assert np.array_equal(tn.blocks_to_dense(b, ql, mps.phys_q, qr), t)


def test_mpo_direct_sum_is_the_sum_of_the_mpos(tn):
    """models.mpo_direct_sum (the MPO of StateEnvs(psi, Vector{MPO}), ProjMPOSum2): its dense
    matrix is the sum of the summands' (the XY and the Ising parts of the Heisenberg chain,
    plus a next-nearest-neighbour Ising term), its bond charges keep the U(1) rule, and
    mismatched summands are refused."""
    from tests.helpers import dense_mpo
    N = 6
    parts = [O.heisenberg_mpo(N, 1.0, Jz=0.0),
             O.mpo_from_terms(N, [(1.0, "Sz", i, "Sz", i + 1) for i in range(N - 1)]),
             O.mpo_from_terms(N, [(0.3, "Sz", i, "Sz", i + 2) for i in range(N - 2)])]
    W, delta = tn.models.mpo_direct_sum([(h.W, h.delta) for h in parts])
    total = O.MPO(W, [np.asarray(x) for x in delta], parts[0].phys_q)
    ref = sum(dense_mpo(h) for h in parts)
    assert np.abs(dense_mpo(total) - ref).max() < 1e-14
    dense_h = dense_mpo(O.heisenberg_mpo(N))
    two = O.MPO(*tn.models.mpo_direct_sum([(h.W, h.delta) for h in parts[:2]]),
                parts[0].phys_q)
    assert np.abs(dense_mpo(two) - dense_h).max() < 1e-14
    q = parts[0].phys_q
    for i, w in enumerate(W):
        a, b, sp, s = np.nonzero(w)
        assert np.all(q[sp] - q[s] == delta[i + 1][b] - delta[i][a])
    with pytest.raises(ValueError, match="same sites"):
        tn.models.mpo_direct_sum([(parts[0].W, parts[0].delta),
                                  (O.heisenberg_mpo(N + 1).W, O.heisenberg_mpo(N + 1).delta)])


def test_mpo_direct_sum_edge_cases(tn):
    """One site: the summands' 1 x 1 site matrices add up; a summand whose edge bond is
    wider than one, or whose edge charges differ, is refused."""
    s = tn.models.mpo_direct_sum
    q = np.zeros(2, dtype=np.int64)
    a = np.arange(4.0).reshape(1, 1, 2, 2)
    b = np.ones((1, 1, 2, 2))
    W, delta = s([([a], [q[:1], q[:1]]), ([b], [q[:1], q[:1]])])
    assert len(W) == 1 and np.array_equal(W[0], a + b)
    wide = [np.ones((2, 1, 2, 2)), np.ones((1, 1, 2, 2))]
    with pytest.raises(ValueError, match="dimension one"):
        s([(wide, [np.zeros(2), np.zeros(1), np.zeros(1)])])
    ok = [np.ones((1, 1, 2, 2)), np.ones((1, 1, 2, 2))]
    with pytest.raises(ValueError, match="edge charges"):
        s([(ok, [np.zeros(1), np.zeros(1), np.zeros(1)]),
           (ok, [np.ones(1), np.zeros(1), np.ones(1)])])
