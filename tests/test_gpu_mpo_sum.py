"""StateEnvs(psi, Vector{MPO}) (ProjMPOSum2, TenNetLib src/mps/state_envs.jl:70-78,
src/mps/projmposum2.jl:86-101) on the GPU through the direct-sum MPO: DMRG and real-time
TDVP with H given as its XY and Ising parts, against the oracle's sweeps with the single
Heisenberg MPO (the same Hamiltonian).

Tolerances: per sweep energies 1e-10 relative and bond dimensions exact; <S^z_i> 1e-8; the
DMRG ground energy against exact diagonalisation 1e-8."""
import json
import os

import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import upload_mpo

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))
SZ = np.diag([0.5, -0.5])


def test_mpo_sum_sweeps_match_single_mpo_oracle(tn, ctx):
    N = 12
    H = O.heisenberg_mpo(N)
    parts = [upload_mpo(tn, ctx, O.heisenberg_mpo(N, 1.0, Jz=0.0)),
             upload_mpo(tn, ctx, O.mpo_from_terms(
                 N, [(1.0, "Sz", i, "Sz", i + 1) for i in range(N - 1)]))]
    pq = np.array([1, -1], dtype=np.int32)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), parts)
    sg = tn.SweepData()
    for md in (8, 16, 16, 32, 32):
        O.fullsweep(eo, so, md, 1e-12, 1, 3, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-12, solver_krylovdim=3,
                      outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), md
        assert sg.maxchi[-1] == so.maxchi[-1], md
    assert abs(sg.energy[-1] - GOLD["heisenberg_chain"]["12"]) < 1e-8
    # real-time TDVP with the sum (TDVPEngine(psi, Vector{MPO}), src/mps/tdvp.jl:45-49)
    po = O.product_mps(start, O.SPIN_HALF_Q)
    po.A = [a.astype(np.complex128) for a in po.A]
    e2, s2 = O.StateEnvs(po, H), O.SweepData()
    eng = tn.TDVPEngine(tn.MPS.product(start, pq, ctx), parts)
    for _ in range(3):
        O.tdvp_sweep(e2, s2, -0.05j, 16, 1e-12, krylovdim=30)
        tn.tdvpsweep_(eng, -0.05j, maxdim=16, cutoff=1e-12, solver_krylovdim=30)
        assert abs(eng.getenergy() - s2.energy[-1]) <= 1e-10 * abs(s2.energy[-1])
        assert eng.maxchi() == s2.maxchi[-1]
        sz = np.array(tn.measure(eng.getpsi(), "Sz"))
        assert np.abs(sz - O.expect_local(e2.psi, SZ)).max() < 1e-8
    # updateH! of a sum: recalcEnv = false is refused as for ProjMPOSum2 (state_envs.jl:227-229)
    with pytest.raises(ValueError, match="ProjMPOSum2"):
        tn.updateH_(eng, parts, recalcEnv=False)
    tn.updateH_(eng, parts, recalcEnv=True)
    tn.tdvpsweep_(eng, -0.05j, maxdim=16, cutoff=1e-12, solver_krylovdim=30)
    O.tdvp_sweep(e2, s2, -0.05j, 16, 1e-12, krylovdim=30)
    assert abs(eng.getenergy() - s2.energy[-1]) <= 1e-10 * abs(s2.energy[-1])
