"""One-site DMRG on the GPU (dmrg1, fullsweep! with nsite = 1, _update_one_site! of
TenNetLib src/mps/update_site.jl:94-190) against the oracle's restatement.

Both start from the same two-site warm-up; then one-site sweeps on both sides.  Per sweep:
|dE/E| <= 1e-10, identical largest bond dimension; at the end every link's charge sectors
are bit-exact and the energy is within 1e-8 of exact diagonalisation where the bond
dimension is complete."""
import json
import os

import numpy as np
import pytest

from oracle import tn_oracle as O

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))


@pytest.mark.parametrize("prec,svd_split", [("fp64", 96), ("split", 96), ("fp64", 0)])
def test_dmrg1_sweeps_match_oracle(tn, prec, svd_split):
    N = 12
    ctx = tn.Context(0, precision=prec, slices=5, svd_split=svd_split)
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), tn.MPO(W, delta, pq, ctx))
    sg = tn.SweepData()
    for md in (8, 32, 64):
        O.fullsweep(eo, so, md, 1e-14, 1, 4, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-14, solver_krylovdim=4,
                      outputlevel=0)
    for _ in range(3):
        O.fullsweep1(eo, so, 64, 1e-14, 1, 4, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 1, sg, maxdim=64, cutoff=1e-14, solver_krylovdim=4,
                      outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1]
        assert abs(sg.entropy[-1] - so.entropy[-1]) <= 1e-9
    psi = eg.getpsi()
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert abs(sg.energy[-1] - GOLD["heisenberg_chain"][str(N)]) < 1e-8


def test_dmrg1_update_position_truncates_and_moves_center(tn):
    # one update at a time through update_position!(..., 1, ortho): the kept spectrum and
    # truncation error agree with the oracle, also when maxdim cuts the link
    N = 10
    ctx = tn.Context(0)
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), tn.MPO(W, delta, pq, ctx))
    sg = tn.SweepData()
    for md in (8, 32):
        O.fullsweep(eo, so, md, 1e-14, 1, 4, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-14, solver_krylovdim=4,
                      outputlevel=0)
    for q in range(N - 1):
        e_g, err_g, eigs_g = tn.update_position_(eg, tn.eig_solver, q, 1, "left", maxdim=12,
                                                 cutoff=1e-14, solver_krylovdim=4)
        e_o, spec, _ = O.update_one_site(eo, q, "left", 12, 1, 1e-14, 4, 2, 1e-14)
        assert abs(e_g - e_o) <= 1e-10 * abs(e_o), q
        assert len(eigs_g) == len(spec.eigs), q
        assert np.allclose(eigs_g, spec.eigs, rtol=0, atol=1e-12), q
        assert abs(err_g - spec.truncerr) <= 1e-14 + 1e-8 * spec.truncerr, q
    assert eg.getpsi().center == N - 1
