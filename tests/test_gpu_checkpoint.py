"""Checkpoint / resume of a DMRG run (the reference restarts from a serialised StateEnvs,
docs/src/mps/example_dmrg.md:76-78): two sweeps, save, load into a new StateEnvs, one more
sweep; the result equals three uninterrupted sweeps and the sweep history continues."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_checkpoint_resume_matches_uninterrupted(tn, tmp_path):
    ctx = tn.Context(0)
    N = 12
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    start = tn.models.neel_states(N)
    kw = dict(cutoff=1e-12, solver_krylovdim=4, outputlevel=0)
    ea = tn.StateEnvs(tn.MPS.product(start, pq, ctx), H)
    sa = tn.SweepData()
    for md in (8, 16, 32):
        tn.fullsweep_(ea, tn.eig_solver, 2, sa, maxdim=md, **kw)
    eb = tn.StateEnvs(tn.MPS.product(start, pq, ctx), H)
    sb = tn.SweepData()
    for md in (8, 16):
        tn.fullsweep_(eb, tn.eig_solver, 2, sb, maxdim=md, **kw)
    path = str(tmp_path / "dmrg.npz")
    tn.save_checkpoint(path, eb, sb)
    del eb
    psi, sw = tn.load_checkpoint(path, ctx)
    assert sw.sweepcount == 2 and sw.energy == sb.energy
    ec = tn.StateEnvs(psi, H)
    tn.fullsweep_(ec, tn.eig_solver, 2, sw, maxdim=32, **kw)
    assert sw.sweepcount == 3
    assert abs(sw.energy[-1] - sa.energy[-1]) <= 1e-12 * abs(sa.energy[-1])
    assert sw.maxchi[-1] == sa.maxchi[-1]
    pa, pc = ea.getpsi(), ec.getpsi()
    assert abs(abs(pa.inner(pc)) - 1.0) < 1e-10


def test_checkpoint_resume_of_a_complex_tdvp_run(tn, tmp_path):
    """Real-time TDVP (ComplexF64 state): two sweeps, save, load, one more sweep equals three
    uninterrupted sweeps."""
    ctx = tn.Context(0)
    N = 10
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    start = tn.models.neel_states(N)
    kw = dict(maxdim=16, cutoff=1e-12)
    ea = tn.TDVPEngine(tn.MPS.product(start, pq, ctx), H)
    for _ in range(3):
        tn.tdvpsweep_(ea, -0.1j, **kw)
    eb = tn.TDVPEngine(tn.MPS.product(start, pq, ctx), H)
    for _ in range(2):
        tn.tdvpsweep_(eb, -0.1j, **kw)
    path = str(tmp_path / "tdvp.npz")
    tn.save_checkpoint(path, eb.sysenv, eb.swdata)
    psi, sw = tn.load_checkpoint(path, ctx)
    assert psi.is_complex
    ec = tn.TDVPEngine(psi, H)
    ec.swdata = sw
    tn.tdvpsweep_(ec, -0.1j, **kw)
    assert ec.sweepcount() == 3
    assert abs(ec.getenergy() - ea.getenergy()) <= 1e-12 * abs(ea.getenergy())
    pa, pc = ea.getpsi(), ec.getpsi()
    assert abs(abs(pa.inner(pc)) - 1.0) < 1e-10
    assert np.abs(np.array(tn.measure(pa, "Sz")) - np.array(tn.measure(pc, "Sz"))).max() < 1e-10
