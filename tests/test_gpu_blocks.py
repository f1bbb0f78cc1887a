"""Block-sparse MPS boundary (tn_mps_create_blocks / tn_mps_site_blocks): only the charge
blocks cross the C ABI, in the block order of an ITensors QN MPS.

The same random state uploaded dense and as blocks gives identical device states (sites
read back dense and as blocks, bit-exact), for centres in the middle and at the ends (left-
and right-grouped sites); a DMRG sweep from either upload gives the same energy; wrong block
lengths are rejected."""
import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import random_qn_mps

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("center", [0, 3, 6])
def test_blocks_and_dense_uploads_agree(tn, ctx, center):
    mps = random_qn_mps(7, np.random.default_rng(12), maxsec_dim=4)
    pq = mps.phys_q.astype(np.int32)
    links = [q.astype(np.int32) for q in mps.links]
    blocks = [tn.dense_to_blocks(t, mps.links[i], mps.phys_q, mps.links[i + 1])
              for i, t in enumerate(mps.A)]
    a = tn.MPS(mps.A, links, pq, center, ctx)
    b = tn.MPS.from_blocks(blocks, links, pq, center, ctx)
    assert b.center == center
    for i in range(7):
        assert np.array_equal(b.site(i), mps.A[i]), i
        assert np.array_equal(a.site_blocks(i), blocks[i]), i
        assert np.array_equal(b.site_blocks(i), blocks[i]), i
    assert abs(a.inner(b) - O.inner(mps, mps)) <= 1e-12 * abs(O.inner(mps, mps))


def test_sweep_from_blocks_equals_sweep_from_dense(tn, ctx):
    N = 12
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    env = tn.StateEnvs(tn.MPS.product(tn.models.neel_states(N), pq, ctx), H)
    sw = tn.SweepData()
    for md in (8, 16):
        tn.fullsweep_(env, tn.eig_solver, 2, sw, maxdim=md, cutoff=1e-12, outputlevel=0)
    psi = env.getpsi()
    links = [psi.link_charges(i) for i in range(N + 1)]
    dense = [psi.site(i) for i in range(N)]
    blocks = [psi.site_blocks(i) for i in range(N)]
    assert sum(b.size for b in blocks) < sum(t.size for t in dense)
    e = []
    for p in (tn.MPS(dense, links, pq, 0, ctx), tn.MPS.from_blocks(blocks, links, pq, 0, ctx)):
        s = tn.SweepData()
        tn.fullsweep_(tn.StateEnvs(p, H), tn.eig_solver, 2, s, maxdim=32, cutoff=1e-12,
                      outputlevel=0)
        e.append(s.energy[-1])
    assert e[0] == e[1]
    with pytest.raises(tn.TenNetError):
        tn.MPS.from_blocks([blocks[0][:-1]] + blocks[1:], links, pq, 0, ctx)
