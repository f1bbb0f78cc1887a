"""updateH! on the GPU (TenNetLib src/mps/state_envs.jl:181-212 through updateH!(engine, H;
recalcEnv) of src/mps/tdvp.jl:182-196): a quench that changes the Hamiltonian between TDVP
sweeps, with the environments rebuilt (recalcEnv = true) or reused (recalcEnv = false: the
first half sweep after the change reads right environments of the old MPO), against the
oracle's restatement.

The workload: the N = 10 Heisenberg chain evolved from the Néel state by four sweeps of
tau = -0.2i, then H -> 0.5 (S^x S^x + S^y S^y) + 2 S^z S^z for three more sweeps.  The two
recalcEnv choices differ by 1.7e-7 in the energy and 8.6e-8 in <S^z_i> there, far above the
tolerances, so each run pins its own semantics.  Tolerances: per sweep energies 1e-10
relative, <S^z_i> 1e-8, bond dimensions and link charges exact."""
import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import upload_mpo

pytestmark = pytest.mark.gpu
SZ = np.diag([0.5, -0.5])
N = 10


@pytest.mark.parametrize("recalc", [True, False])
def test_update_h_quench_matches_oracle(tn, ctx, recalc):
    H1, H2 = O.heisenberg_mpo(N), O.heisenberg_mpo(N, 0.5, Jz=2.0)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    po = O.product_mps(start, O.SPIN_HALF_Q)
    po.A = [a.astype(np.complex128) for a in po.A]
    eo = O.StateEnvs(po, H1)
    so = O.SweepData()
    eng = tn.TDVPEngine(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx),
                        upload_mpo(tn, ctx, H1))
    kw = dict(maxdim=16, cutoff=1e-12, solver_krylovdim=30)
    for _ in range(4):
        O.tdvp_sweep(eo, so, -0.2j, 16, 1e-12, krylovdim=30)
        tn.tdvpsweep_(eng, -0.2j, **kw)
    eo.update_h(H2, recalc)
    tn.updateH_(eng, upload_mpo(tn, ctx, H2), recalcEnv=recalc)
    for _ in range(3):
        O.tdvp_sweep(eo, so, -0.2j, 16, 1e-12, krylovdim=30)
        tn.tdvpsweep_(eng, -0.2j, **kw)
        assert abs(eng.getenergy() - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert eng.maxchi() == so.maxchi[-1]
        sz = np.array(tn.measure(eng.getpsi(), "Sz"))
        assert np.abs(sz - O.expect_local(eo.psi, SZ)).max() < 1e-8
    psi = eng.getpsi()
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i


def test_update_h_argument_errors(tn, ctx):
    H1 = O.heisenberg_mpo(N)
    pq = np.array([1, -1], dtype=np.int32)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eng = tn.TDVPEngine(tn.MPS.product(start, pq, ctx), upload_mpo(tn, ctx, H1))
    tn.tdvpsweep_(eng, -0.1, maxdim=8)
    # other MPO link indices (a next-nearest-neighbour term widens the MPO)
    terms = [(1.0, "Sz", i, "Sz", i + 1) for i in range(N - 1)]
    terms += [(0.5, "Sz", i, "Sz", i + 2) for i in range(N - 2)]
    wide = O.mpo_from_terms(N, terms)
    assert max(w.shape[1] for w in wide.W) != max(w.shape[1] for w in H1.W)
    with pytest.raises(tn.TenNetError, match="link indices"):
        tn.updateH_(eng, upload_mpo(tn, ctx, wide), recalcEnv=False)
    tn.updateH_(eng, upload_mpo(tn, ctx, wide), recalcEnv=True)
    tn.tdvpsweep_(eng, -0.1, maxdim=8)
    assert np.isfinite(eng.getenergy())
    # left environments built (two left-moving updates): reuse is refused, as the reference
    # asserts lpos == 0
    for b in range(2):
        tn.update_position_(eng.sysenv, tn.eig_solver, b, 2, "left", maxdim=8)
    with pytest.raises(tn.TenNetError, match="lpos"):
        tn.updateH_(eng, upload_mpo(tn, ctx, H1), recalcEnv=False)
    # site indices must match
    with pytest.raises(tn.TenNetError, match="site indices"):
        tn.updateH_(eng, upload_mpo(tn, ctx, O.heisenberg_mpo(N + 2)), recalcEnv=True)
    with pytest.raises(ValueError, match="projector"):
        tn.updateH_(eng, upload_mpo(tn, ctx, H1), [eng.getpsi()], weight=1.0)
