"""The mixed one-/two-site sweep of dynamic_fullsweep! on the GPU (TenNetLib
src/mps/sweep.jl:284-355; tdvpsweep! with nsite = "dynamic", src/mps/tdvp.jl:256-260)
against the oracle's restatement: per bond a one-site update when the bond's last kept
spectrum ends below eigthreshold or its link is at maxdim, else two sites.

Both branches of the choice are exercised (bonds at maxdim and bonds whose smallest kept
eigenvalue is below the threshold; the thresholds sit at least 6 % away from every decided
value of the oracle).  Tolerances: the per-bond choices of both halves exact, energies per
sweep 1e-10 relative, entropy 1e-9, bond dimensions and link charges exact, <S^z_i> 1e-8
(TDVP), norm 1e-12."""
import copy

import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import upload_mpo, upload_mps

pytestmark = pytest.mark.gpu
SZ = np.diag([0.5, -0.5])


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("tau,thr", [(-0.1, 1e-6), (-0.05j, 1e-8)])
def test_dynamic_tdvp_matches_oracle(tn, tau, thr, precision):
    ctx = tn.Context(0, precision=precision, slices=5)
    N, md = 10, 6
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    po = O.product_mps(start, O.SPIN_HALF_Q)
    if isinstance(tau, complex):
        po.A = [a.astype(np.complex128) for a in po.A]
    eo = O.StateEnvs(po, H)
    so = O.SweepData()
    eng = tn.TDVPEngine(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx),
                        upload_mpo(tn, ctx, H))
    kw = dict(maxdim=md, cutoff=1e-12, solver_krylovdim=30)
    for _ in range(2):
        O.tdvp_sweep(eo, so, tau, md, 1e-12, krylovdim=30)
        tn.tdvpsweep_(eng, tau, **kw)
    for i, e in enumerate(eng.swdata.lasteigs):
        np.testing.assert_allclose(e, so.lasteigs[i], rtol=1e-7, atol=1e-13)
    seen = set()
    for _ in range(5):
        lo, ro = O.dynamic_sweep(eo, so, md, 1e-12, thr, tau)
        tn.tdvpsweep_(eng, tau, nsite="dynamic", eigthreshold=thr, **kw)
        st = eng.swdata.stats[-1]
        assert list(st["nsite_left"]) == lo and list(st["nsite_right"]) == ro
        seen.update(lo + ro)
        assert abs(eng.getenergy() - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert eng.maxchi() == so.maxchi[-1]
        assert abs(eng.getentropy() - so.entropy[-1]) < 1e-9
        psi = eng.getpsi()
        sz = np.array(tn.measure(psi, "Sz"))
        assert np.abs(sz - O.expect_local(eo.psi, SZ)).max() < 1e-8
    assert seen == {1, 2}
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert abs(psi.inner(psi) - 1.0) < 1e-12
    assert eng.sweepcount() == 7
    assert eng.abstime == pytest.approx(7 * abs(tau))


def test_dynamic_dmrg_matches_oracle(tn, ctx):
    """dynamic_fullsweep! with eig_solver after two two-site sweeps from the Néel state:
    bonds at maxdim 16 and bonds below eigthreshold 1e-5 (smallest kept eigenvalues
    ~1e-7 and ~1e-10 against ~2e-4 on the two-site bonds) take one-site updates."""
    N, md, thr = 10, 16, 1e-5
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    eg = tn.StateEnvs(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx),
                      upload_mpo(tn, ctx, H))
    sg = tn.SweepData()
    kw = dict(maxdim=md, cutoff=1e-12, solver_krylovdim=3, outputlevel=0)
    for _ in range(2):
        O.fullsweep(eo, so, md, 1e-12, 1, 3)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, **kw)
    seen = set()
    for _ in range(3):
        lo, ro = O.dynamic_sweep(eo, so, md, 1e-12, thr, krylovdim=3)
        tn.dynamic_fullsweep_(eg, tn.eig_solver, sg, eigthreshold=thr, **kw)
        assert list(sg.stats[-1]["nsite_left"]) == lo
        assert list(sg.stats[-1]["nsite_right"]) == ro
        seen.update(lo + ro)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1]
        assert abs(sg.entropy[-1] - so.entropy[-1]) < 1e-9
    assert seen == {1, 2}
    psi = eg.getpsi()
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    # a single MPO: the first sweep (and every extendat-th) would be global subspace
    # expansion, which is not built
    fresh = tn.StateEnvs(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx),
                         upload_mpo(tn, ctx, H))
    with pytest.raises(NotImplementedError, match="krylov_extend"):
        tn.dynamic_fullsweep_(fresh, tn.eig_solver, tn.SweepData(), maxdim=md)
    with pytest.raises(NotImplementedError, match="krylov_extend"):
        tn.dynamic_fullsweep_(eg, tn.eig_solver, sg, extendat=1, maxdim=md)


def test_dynamic_dmrg_with_projector_matches_oracle(tn, ctx):
    """With an excited-state projector (ProjMPO_MPS2) the first dynamic sweep is a plain
    two-site sweep (sweep.jl:266-272: subspace expansion only for a single MPO), then the
    mixed sweeps, with one-site updates on the projected H_eff; the ground state of a DMRG
    run is M, weight 10.  Against the oracle: choices exact, energies 1e-10."""
    N, md, thr = 10, 16, 1e-5
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    _, env = O.dmrg(O.product_mps(start, O.SPIN_HALF_Q), H, maxdim=[16, 32], nsweeps=[3, 4],
                    cutoff=1e-14)
    gr = env.psi
    pq = H.phys_q.astype(np.int32)
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H, [gr], weight=10.0)
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), upload_mpo(tn, ctx, H),
                      [upload_mps(tn, ctx, gr, gr.center)], weight=10.0)
    so, sg = O.SweepData(), tn.SweepData()
    kw = dict(maxdim=md, cutoff=1e-14, outputlevel=0)
    O.fullsweep(eo, so, md, 1e-14, 1, 5, 2, 1e-14)
    tn.dynamic_fullsweep_(eg, tn.eig_solver, sg, eigthreshold=thr, **kw)
    assert sg.sweepcount == 1 and "nsite_left" not in sg.stats[-1]
    assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
    seen = set()
    for _ in range(3):
        lo, ro = O.dynamic_sweep(eo, so, md, 1e-14, thr)
        tn.dynamic_fullsweep_(eg, tn.eig_solver, sg, eigthreshold=thr, **kw)
        assert list(sg.stats[-1]["nsite_left"]) == lo
        assert list(sg.stats[-1]["nsite_right"]) == ro
        seen.update(lo + ro)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1]
    assert seen == {1, 2}


def test_dynamic_fullsweep_exp_solver_is_the_tdvp_sweep(tn, ctx):
    """dynamic_fullsweep!(sysenv, exp_solver, swdata; time_step = tau / 2, reverse_step =
    true) is the sweep tdvpsweep!(engine, tau; nsite = "dynamic") runs (tdvp.jl:256-260):
    the same choices and energies (1e-11) from copies of one state."""
    N = 8
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    eng = tn.TDVPEngine(tn.MPS.product(tn.models.neel_states(N), pq, ctx), H)
    kw = dict(maxdim=6, cutoff=1e-12)
    for _ in range(2):
        tn.tdvpsweep_(eng, -0.1, **kw)
    se = tn.StateEnvs(eng.getpsi(), H)
    sw = copy.deepcopy(eng.swdata)
    for _ in range(3):
        tn.tdvpsweep_(eng, -0.1, nsite="dynamic", eigthreshold=1e-6, **kw)
        tn.dynamic_fullsweep_(se, tn.exp_solver, sw, eigthreshold=1e-6, time_step=-0.05,
                              reverse_step=True, outputlevel=0, **kw)
        st = eng.swdata.stats[-1]
        assert list(sw.stats[-1]["nsite_left"]) == list(st["nsite_left"])
        assert list(sw.stats[-1]["nsite_right"]) == list(st["nsite_right"])
        assert abs(sw.energy[-1] - eng.getenergy()) <= 1e-11 * abs(eng.getenergy())
    with pytest.raises(ValueError, match="reverse_step"):
        tn.dynamic_fullsweep_(se, tn.exp_solver, sw, time_step=-0.05, **kw)
