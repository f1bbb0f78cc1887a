"""Host helpers of the block-sparse MPS boundary: dense_to_blocks / blocks_to_dense round
trip on random charge-conserving site tensors, and the block count equals the number of
entries the charges allow."""
import numpy as np

from oracle import tn_oracle as O
from tests.helpers import random_qn_mps


def test_dense_blocks_round_trip(tn):
    mps = random_qn_mps(7, np.random.default_rng(11), maxsec_dim=3)
    for i, t in enumerate(mps.A):
        ql, qr = mps.links[i], mps.links[i + 1]
        b = tn.dense_to_blocks(t, ql, mps.phys_q, qr)
        assert b.size == int(O.qn_mask3(ql, mps.phys_q, qr).sum())
        assert np.array_equal(tn.blocks_to_dense(b, ql, mps.phys_q, qr), t)
