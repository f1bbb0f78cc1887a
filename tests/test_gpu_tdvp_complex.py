"""Real-time (complex) two-site TDVP on the GPU: tdvpsweep! with tau = -0.05i
(TenNetLib src/mps/tdvp.jl:247-277, exp_solver of src/base/solver.jl:66-88, the reverse step
of src/mps/update_site.jl:78-87) on ComplexF64 states, against the oracle's complex
restatement and the exact quench (tests/golden/quench_sz.json).

Tolerances: the complex H_eff product 1e-12 relative (5e-11 in split precision, as for real
states); complex overlaps and local expectation
values 1e-12; per sweep <S^z_i(t)> within 1e-8 of the oracle (the TDVP observable bound),
energies 1e-10 relative, bond dimensions and link charges bit-exact; against the exact
evolution 1e-6 (the TDVP projection error of the small bond dimensions, as for the oracle).
One-site TDVP (nsite = 1, zero-site reverse step), real and complex steps: per sweep energies
1e-10, entropy 1e-9, <S^z_i> 1e-8, bond dimensions and link charges exact.  At the scale of
the real-time workload (N = 64, chi ~ 60, one sweep from a GPU-evolved state): energy
1e-10, <S^z_i> 1e-8, link charges exact."""
import json
import os

import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import random_qn_mps, upload_mpo, upload_mps

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "quench_sz.json")))
SZ = np.diag([0.5, -0.5])


def _complex_mps(N, seed, maxsec_dim=3):
    rng = np.random.default_rng(seed)
    m = random_qn_mps(N, rng, maxsec_dim)
    m.A = [a + 1j * rng.standard_normal(a.shape) * (a != 0) for a in m.A]
    return m


def test_complex_product_overlap_and_expectation(tn, ctx):
    N = 8
    H = O.heisenberg_mpo(N)
    Hg = upload_mpo(tn, ctx, H)
    for p in (0, 3, 6):
        m = _complex_mps(N, 10 + p)
        m.center = p
        eo = O.StateEnvs(m, H)
        eg = tn.StateEnvs(upload_mps(tn, ctx, m, p), Hg)
        assert eg.is_complex
        eo.position(p, 2)
        eg.position_(p, 2)
        rng = np.random.default_rng(p)
        shape = (len(m.links[p]), 2, 2, len(m.links[p + 2]))
        v = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        v *= (m.links[p][:, None, None, None] + m.phys_q[None, :, None, None] +
              m.phys_q[None, None, :, None] == m.links[p + 2][None, None, None, :])
        ref = eo.product2(p, v)
        got = eg.product(v)
        assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), p
        # the split-precision complex product (bf16-slice tensor-core GEMMs, unsigned form)
        cs = tn.Context(0, precision="split", slices=5)
        es = tn.StateEnvs(upload_mps(tn, cs, m, p), upload_mpo(tn, cs, H))
        es.position_(p, 2)
        got = es.product(v)
        assert np.linalg.norm(got - ref) <= 5e-11 * np.linalg.norm(ref), p
    # overlap of two complex states on the same links (a conjugated)
    rng = np.random.default_rng(7)
    a = _complex_mps(N, 1)
    b = O.MPS([x + 0.3 * (rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape)) *
               (x != 0) for x in a.A], [q.copy() for q in a.links], a.phys_q.copy(), 0)
    ag, bg = upload_mps(tn, ctx, a, 0), upload_mps(tn, ctx, b, 0)
    ref = O.inner(a, b)
    assert abs(ag.inner(bg) - ref) <= 1e-12 * abs(ref)
    for i in range(N):
        assert np.array_equal(ag.site(i), a.A[i])
    # <S^z_i> of a normalised complex state (transfer matrices) against the oracle's
    a.A[0] = a.A[0] / np.sqrt(abs(O.inner(a, a)))
    ag = upload_mps(tn, ctx, a, 0)
    assert np.abs(ag.expect_local(SZ) - O.expect_local(a, SZ)).max() < 1e-12
    # a real state is read with zero imaginary parts once made complex
    r = random_qn_mps(N, np.random.default_rng(3))
    rg = upload_mps(tn, ctx, r, 0)
    assert not rg.is_complex
    rg.to_complex_()
    assert rg.is_complex
    assert np.array_equal(rg.site(2), r.A[2].astype(np.complex128))


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_real_time_quench_matches_oracle_and_exact(tn, precision):
    ctx = tn.Context(0, precision=precision, slices=5)
    N = GOLD["N"]
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    po = O.product_mps(start, O.SPIN_HALF_Q)
    po.A = [a.astype(np.complex128) for a in po.A]
    eo = O.StateEnvs(po, H)
    so = O.SweepData()
    eng = tn.TDVPEngine(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx),
                        upload_mpo(tn, ctx, H))
    t = 0.0
    for tk, exact in zip(GOLD["times"], GOLD["sz"]):
        while t < tk - 1e-12:
            O.tdvp_sweep(eo, so, -0.05j, maxdim=64, cutoff=1e-12, krylovdim=30)
            tn.tdvpsweep_(eng, -0.05j, maxdim=64, cutoff=1e-12, solver_krylovdim=30)
            t += 0.05
            psi = eng.getpsi()
            assert psi.is_complex
            sz_g = np.array(tn.measure(psi, "Sz"))
            sz_o = O.expect_local(eo.psi, SZ)
            assert np.abs(sz_g - sz_o).max() < 1e-8, t
            assert eng.maxchi() == so.maxchi[-1], t
            assert abs(eng.getenergy() - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), t
        assert np.abs(sz_g - np.array(exact)).max() < 1e-6
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert abs(psi.inner(psi) - 1.0) < 1e-12
    assert eng.abstime == pytest.approx(1.0)


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("tau", [-0.1, -0.05j])
def test_one_site_tdvp_matches_oracle(tn, tau, precision):
    """tdvpsweep! with nsite = 1 (one-site updates with the zero-site reverse step) after
    three two-site sweeps that grow the bonds, real and complex steps, against the oracle."""
    ctx = tn.Context(0, precision=precision, slices=5)
    N = 10
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    po = O.product_mps(start, O.SPIN_HALF_Q)
    if isinstance(tau, complex):
        po.A = [a.astype(np.complex128) for a in po.A]
    eo = O.StateEnvs(po, H)
    so = O.SweepData()
    eng = tn.TDVPEngine(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx),
                        upload_mpo(tn, ctx, H))
    for nsite in (2, 2, 2, 1, 1, 1, 1):
        O.tdvp_sweep(eo, so, tau, 16, 1e-12, krylovdim=30, nsite=nsite)
        tn.tdvpsweep_(eng, tau, nsite=nsite, maxdim=16, cutoff=1e-12, solver_krylovdim=30)
        assert abs(eng.getenergy() - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), nsite
        assert eng.maxchi() == so.maxchi[-1]
        assert abs(eng.getentropy() - so.entropy[-1]) < 1e-9
        psi = eng.getpsi()
        sz = np.array(tn.measure(psi, "Sz"))
        assert np.abs(sz - O.expect_local(eo.psi, SZ)).max() < 1e-8
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert abs(psi.inner(psi) - 1.0) < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_quench_at_scale_matches_oracle(tn, precision):
    """The real-time quench workload (N = 64 chain, maxdim 512, cutoff 1e-9, krylovdim 30):
    a state evolved on the GPU to t = 2.5 (10 sweeps of tau = -0.25i), copied to the oracle,
    then the same sweep of tau = -0.05i on both."""
    ctx = tn.Context(0, precision=precision, slices=5)
    N = 64
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    eng = tn.TDVPEngine(tn.MPS.product(tn.models.neel_states(N), pq, ctx), H)
    kw = dict(maxdim=512, cutoff=1e-9, solver_krylovdim=30)
    for _ in range(10):
        tn.tdvpsweep_(eng, -0.25j, **kw)
    psi0 = eng.getpsi()
    assert psi0.maxlinkdim() >= 16
    po = O.MPS([psi0.site(i) for i in range(N)],
               [psi0.link_charges(i).astype(np.int64) for i in range(N + 1)],
               O.SPIN_HALF_Q.copy(), center=0)
    eo = O.StateEnvs(po, O.heisenberg_mpo(N))
    so = O.SweepData()
    O.tdvp_sweep(eo, so, -0.05j, 512, 1e-9, 1, 30, 100, 1e-12)
    e2 = tn.TDVPEngine(psi0, H)
    tn.tdvpsweep_(e2, -0.05j, **kw)
    psi = e2.getpsi()
    assert abs(e2.getenergy() - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
    assert np.abs(np.array(tn.measure(psi, "Sz")) - O.expect_local(eo.psi, SZ)).max() < 1e-8
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
