"""Density-matrix noise term of the two-site update (noiseterm + replacebond! with an
eigen perturbation, TenNetLib src/mps/update_site.jl:59-76) and of the one-site update
(:135-152) against the oracle's restatement, through dmrg!'s noise schedule
(src/mps/dmrg.jl:212-223).

Per sweep: |dE/E| <= 1e-10 and identical largest bond dimension; at the end the charge
sectors of every link bit-exact and the energy at the exact ground energy (1e-8)."""
import json
import os

import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import upload_mpo

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))


@pytest.mark.parametrize("prec,svd_split", [("fp64", 96), ("split", 96), ("fp64", 0)])
def test_noise_sweeps_match_oracle(tn, prec, svd_split):
    N = 12
    ctx = tn.Context(0, precision=prec, slices=5, svd_split=svd_split)
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    # the same MPO on both sides: the noise tensor L W phi carries the MPO link between the
    # two sites, so the perturbation depends on the MPO's basis of that link
    pq = H.phys_q.astype(np.int32)
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), upload_mpo(tn, ctx, H))
    sg = tn.SweepData()
    # maxdim 4 then 8 with noise 1e-3 halving each sweep, then noise off
    sched = [(4, 1e-3), (8, 5e-4), (16, 2.5e-4), (32, 1.25e-4), (64, 0.0), (64, 0.0)]
    for md, nz in sched:
        O.fullsweep(eo, so, md, 1e-14, 1, 4, 2, 1e-14, noise=nz)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-14, solver_krylovdim=4,
                      noise=nz, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), (md, nz)
        assert sg.maxchi[-1] == so.maxchi[-1], (md, nz)
    psi = eg.getpsi()
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert abs(sg.energy[-1] - GOLD["heisenberg_chain"][str(N)]) < 1e-8


def test_noise_update_matches_oracle_both_directions(tn):
    # single updates with noise in both sweep directions: kept spectra (eigenvalues of the
    # perturbed density matrix) and truncation errors
    N = 10
    ctx = tn.Context(0)
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    # the same MPO on both sides: the noise tensor L W phi carries the MPO link between the
    # two sites, so the perturbation depends on the MPO's basis of that link
    pq = H.phys_q.astype(np.int32)
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), upload_mpo(tn, ctx, H))
    sg = tn.SweepData()
    for md in (4, 8):
        O.fullsweep(eo, so, md, 1e-14, 1, 4, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-14, solver_krylovdim=4,
                      outputlevel=0)
    for b, ortho in [(q, "left") for q in range(N - 1)] + [(q, "right") for q in range(N - 2, -1, -1)]:
        e_g, err_g, eigs_g = tn.update_position_(eg, tn.eig_solver, b, 2, ortho, maxdim=12,
                                                 cutoff=1e-12, solver_krylovdim=4, noise=1e-2)
        e_o, spec, _ = O.update_two_site(eo, b, ortho, 12, 1, 1e-12, 4, 2, 1e-14, noise=1e-2)
        assert abs(e_g - e_o) <= 1e-10 * abs(e_o), (b, ortho)
        assert len(eigs_g) == len(spec.eigs), (b, ortho)
        # the updates chain 17 noisy bond splits: 1e-10 on the density-matrix eigenvalues
        assert np.allclose(eigs_g, spec.eigs, rtol=0, atol=1e-10), (b, ortho)
        assert abs(err_g - spec.truncerr) <= 1e-14 + 1e-8 * spec.truncerr, (b, ortho)


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_one_site_noise_sweeps_match_oracle(tn, prec):
    # one-site DMRG from a product state: only the noise term can grow the bonds (the
    # reference's own test runs dmrg1 this way, test/test_MPS_DMRG.jl:50-65)
    N = 12
    ctx = tn.Context(0, precision=prec, slices=5)
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    pq = H.phys_q.astype(np.int32)
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), upload_mpo(tn, ctx, H))
    sg = tn.SweepData()
    sched = [(8, 1e-3), (16, 5e-4), (32, 2.5e-4), (64, 1.25e-4), (64, 0.0), (64, 0.0)]
    # cutoff 1e-10: the density-matrix eigenvalues come from eigh(rho) in the oracle (as in
    # ITensors' factorize_eigen), accurate to ~1e-16 absolute, so near a 1e-14 cutoff the
    # kept count is decided by rounding; at 1e-10 both sides resolve it
    for md, nz in sched:
        O.fullsweep1(eo, so, md, 1e-10, 1, 4, 2, 1e-14, noise=nz)
        tn.fullsweep_(eg, tn.eig_solver, 1, sg, maxdim=md, cutoff=1e-10, solver_krylovdim=4,
                      noise=nz, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), (md, nz)
        assert sg.maxchi[-1] == so.maxchi[-1], (md, nz)
    assert so.maxchi[-1] > 8
    psi = eg.getpsi()
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
