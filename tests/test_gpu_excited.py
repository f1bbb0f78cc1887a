"""Excited-state DMRG on the GPU: ProjMPS2 / ProjMPO_MPS2 (TenNetLib src/mps/projmps2.jl,
src/mps/projmpo_mps2.jl:94-101, StateEnvs(psi, H, Ms; weight) of src/mps/state_envs.jl:88-105)
against the oracle's restatement, as in the reference's own excited-state test
(test/test_MPS_DMRG.jl:71-96: the ground state as M, weight 10).

Tolerances: the product H_eff v + w m (m . v) 1e-12 relative; per sweep |dE/E| <= 1e-10 and
identical largest bond dimension; at the end the second-lowest energy of the S^z = 0 sector
(dense diagonalisation) to 1e-8 and an overlap with M below 1e-6."""
import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import dense_mpo, upload_mps, upload_mpo

pytestmark = pytest.mark.gpu
N = 10


def _setup(tn, prec):
    H = O.heisenberg_mpo(N)
    D = dense_mpo(H)
    sz = np.array([sum(0.5 - ((k >> (N - 1 - i)) & 1) for i in range(N)) for k in range(2 ** N)])
    sec = np.nonzero(sz == 0)[0]
    ev = np.linalg.eigvalsh(D[np.ix_(sec, sec)])
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    sw, env = O.dmrg(O.product_mps(start, O.SPIN_HALF_Q), H, maxdim=[16, 32], nsweeps=[3, 4],
                     cutoff=1e-14)
    gr = env.psi
    ctx = tn.Context(0, precision=prec, slices=5)
    return H, ev, start, gr, ctx


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_excited_state_sweeps_match_oracle(tn, prec):
    H, ev, start, gr, ctx = _setup(tn, prec)
    Hg = upload_mpo(tn, ctx, H)
    grg = upload_mps(tn, ctx, gr, gr.center)
    pq = H.phys_q.astype(np.int32)
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H, [gr], weight=10.0)
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), Hg, [grg], weight=10.0)
    so, sg = O.SweepData(), tn.SweepData()
    for md in (8, 16, 32, 32, 32, 32):
        O.fullsweep(eo, so, md, 1e-14, 1, 5, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-14, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), md
        assert sg.maxchi[-1] == so.maxchi[-1], md
    # one-site sweeps from the grown state (ProjMPS2 with nsite = 1)
    for _ in range(2):
        O.fullsweep1(eo, so, 32, 1e-14, 1, 5, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 1, sg, maxdim=32, cutoff=1e-14, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1]
    assert abs(sg.energy[-1] - ev[1]) < 1e-8
    psi = eg.getpsi()
    assert abs(psi.inner(grg)) < 1e-6
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i


def test_projected_product_matches_oracle(tn):
    H, ev, start, gr, ctx = _setup(tn, "fp64")
    Hg = upload_mpo(tn, ctx, H)
    # psi: a random charge-conserving state at bond dimension of the ground state's links
    rng = np.random.default_rng(5)
    A = [rng.standard_normal(a.shape) * O.qn_mask3(gr.links[i], gr.phys_q, gr.links[i + 1])
         for i, a in enumerate(gr.A)]
    M2 = O.MPS([a.copy() for a in gr.A], [q.copy() for q in gr.links], gr.phys_q.copy(),
               gr.center)
    Ms = [upload_mps(tn, ctx, gr, gr.center), upload_mps(tn, ctx, M2, M2.center)]
    for p in (0, 3, 7):
        # environments are plain contractions: the state need not be orthonormal
        psi = O.MPS(A, [q.copy() for q in gr.links], gr.phys_q.copy(), center=p)
        eo = O.StateEnvs(psi, H, [gr, M2], weight=3.5)
        eg = tn.StateEnvs(upload_mps(tn, ctx, psi, p), Hg, Ms, weight=3.5)
        eo.position(p, 2)
        eg.position_(p, 2)
        v = rng.standard_normal((len(psi.links[p]), 2, 2, len(psi.links[p + 2])))
        v *= (psi.links[p][:, None, None, None] + psi.phys_q[None, :, None, None] +
              psi.phys_q[None, None, :, None] == psi.links[p + 2][None, None, None, :])
        ref = eo.product2(p, v)
        got = eg.product(v)
        assert np.allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max()), p


def test_dmrg_api_with_projectors(tn):
    H, ev, start, gr, ctx = _setup(tn, "fp64")
    Hg = upload_mpo(tn, ctx, H)
    grg = upload_mps(tn, ctx, gr, gr.center)
    pq = H.phys_q.astype(np.int32)
    params = tn.DMRGParams(nsweeps=[4, 4], maxdim=[16, 32], cutoff=1e-14)
    e, psi = tn.dmrg2(tn.MPS.product(start, pq, ctx), Hg, [grg], params, weight=10.0,
                      outputlevel=0)
    assert abs(e - ev[1]) < 1e-8
    assert abs(psi.inner(grg)) < 1e-6
    with pytest.raises(tn.TenNetError):
        tn.dmrg2(tn.MPS.product(start, pq, ctx), Hg, [grg], params, outputlevel=0)
    with pytest.raises(tn.TenNetError):
        tn.StateEnvs(tn.MPS.product(start, pq, ctx), Hg, [grg], weight=0.0)
