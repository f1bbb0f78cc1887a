"""Parity of the CUDA sweep path (through the C ABI) with the CPU oracle.

Tolerances: FP64 path, relative 1e-12 for single products and block SVDs, 1e-10 relative
for DMRG energies (the accuracy bound of the sweep); bond dimensions and charge sectors bit-exact.
"""
import json
import os

import numpy as np
import pytest

from oracle import ed
from oracle import tn_oracle as O
from tests.helpers import oracle_envs, random_qn_mps, upload_mpo, upload_mps

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))


def _mask2(ql, pq, qr):
    return (ql[:, None, None, None] + pq[None, :, None, None] + pq[None, None, :, None]) == \
        qr[None, None, None, :]


@pytest.mark.parametrize("qn", [True, False])
@pytest.mark.parametrize("p", [0, 3, 6])
def test_heff_product_matches_oracle(tn, ctx, qn, p):
    rng = np.random.default_rng(100 + p + 10 * qn)
    N = 8
    mps = random_qn_mps(N, rng, maxsec_dim=3, qn=qn)
    H = O.heisenberg_mpo(N, qn=qn)
    env = tn.StateEnvs(upload_mps(tn, ctx, mps, center=p), upload_mpo(tn, ctx, H))
    env.position_(p, 2)
    Lp, Rp = oracle_envs(mps, H, p)
    v = rng.standard_normal((len(mps.links[p]), 2, 2, len(mps.links[p + 2])))
    v *= _mask2(mps.links[p], mps.phys_q, mps.links[p + 2])
    ref = O.heff2_apply(Lp, H.W[p], H.W[p + 1], Rp, v)
    got = env.product(v)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
    assert env.product_flops() > 0


def test_heff_product_long_range_mpo(tn, ctx):
    # a J1-J2 cylinder MPO (automaton with a few dozen states) on a random state
    rng = np.random.default_rng(5)
    Lx, Ly = 3, 4
    N = Lx * Ly
    H = O.mpo_from_terms(N, O.j1j2_cylinder_terms(Lx, Ly, 1.0, 0.5))
    mps = random_qn_mps(N, rng, maxsec_dim=3)
    for p in (2, 5):
        env = tn.StateEnvs(upload_mps(tn, ctx, mps, center=p), upload_mpo(tn, ctx, H))
        env.position_(p, 2)
        Lp, Rp = oracle_envs(mps, H, p)
        v = rng.standard_normal((len(mps.links[p]), 2, 2, len(mps.links[p + 2])))
        v *= _mask2(mps.links[p], mps.phys_q, mps.links[p + 2])
        ref = O.heff2_apply(Lp, H.W[p], H.W[p + 1], Rp, v)
        got = env.product(v)
        assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


def test_block_svd_truncation_matches_oracle(tn, ctx):
    rng = np.random.default_rng(9)
    blocks = []
    for (r, c) in [(1, 1), (5, 3), (3, 7), (40, 40), (64, 17), (9, 100), (33, 33)]:
        # graded singular values so that the cutoff falls inside the spectrum
        U, _ = np.linalg.qr(rng.standard_normal((r, r)))
        V, _ = np.linalg.qr(rng.standard_normal((c, c)))
        k = min(r, c)
        s = np.exp(-rng.uniform(0, 14, size=k))
        blocks.append((U[:, :k] * s) @ V[:k, :])
    for maxdim, cutoff in [(1000, 1e-12), (40, 1e-12), (7, 1e-15), (1000, 1e-6)]:
        kept, sv, err = tn.svd_truncate(blocks, maxdim=maxdim, cutoff=cutoff, ctx=ctx)
        _, spec, kept_ref = O.svd_blocks_truncate(blocks, maxdim, 1, cutoff)
        assert list(kept) == kept_ref
        assert abs(err - spec.truncerr) <= 1e-14 + 1e-10 * spec.truncerr
        for b, s in zip(blocks, sv):
            ref = np.linalg.svd(b, compute_uv=False)
            assert np.allclose(s, ref, rtol=0, atol=1e-13 * ref[0])


def test_block_svd_degenerate_multiplets(tn, ctx):
    # SU(2)-like multiplets split over charge blocks: the cut is taken whole
    s = np.sqrt(np.array([0.4, 0.2]))
    blocks = [np.diag(s), np.diag([np.sqrt(0.2)]), np.diag([np.sqrt(0.2)]), np.diag([0.1])]
    kept, _, _ = tn.svd_truncate(blocks, maxdim=2, cutoff=1e-15, ctx=ctx)
    _, _, kept_ref = O.svd_blocks_truncate(blocks, 2, 1, 1e-15)
    assert list(kept) == kept_ref == [1, 0, 0, 0]


def _dmrg_both(tn, ctx, N, H, start, maxdims, cutoff, krylovdim, maxiter=2, qn=True):
    """Run the same sweeps on the oracle and on the engine; yield per-sweep pairs."""
    if qn:
        po = O.product_mps(start, O.SPIN_HALF_Q)
        pg = tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx)
    else:
        po = O.product_mps(None, np.zeros(2, dtype=np.int64), vectors=start)
        t = [start[i].reshape(1, 2, 1) for i in range(N)]
        lk = [np.array([0], dtype=np.int32)] * (N + 1)
        pg = tn.MPS(t, lk, np.zeros(2, dtype=np.int32), 0, ctx)
    eo = O.StateEnvs(po, H)
    so = O.SweepData()
    eg = tn.StateEnvs(pg, upload_mpo(tn, ctx, H))
    sg = tn.SweepData()
    for md in maxdims:
        O.fullsweep(eo, so, md, cutoff, 1, krylovdim, maxiter, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=cutoff,
                      solver_krylovdim=krylovdim, solver_maxiter=maxiter, outputlevel=0)
        yield so, sg, eo, eg


def _same_links(eo, eg):
    psi = eg.getpsi()
    for i in range(len(eo.psi.links)):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), f"link {i}"


def test_dmrg_sweeps_match_oracle_qn(tn, ctx):
    N = 12
    H = O.heisenberg_mpo(N)
    for so, sg, eo, eg in _dmrg_both(tn, ctx, N, H, [0 if i % 2 == 0 else 1 for i in range(N)],
                                     [8, 16, 16, 32, 32], 1e-12, krylovdim=3):
        e_o, e_g = so.energy[-1], sg.energy[-1]
        assert abs(e_g - e_o) <= 1e-10 * abs(e_o)
        assert sg.maxchi[-1] == so.maxchi[-1]
        assert abs(sg.entropy[-1] - so.entropy[-1]) < 1e-9
        _same_links(eo, eg)
    assert abs(sg.energy[-1] - GOLD["heisenberg_chain"]["12"]) < 1e-8
    # state overlap with the oracle's ground state, on the GPU (both normalised)
    pg = eg.getpsi()
    po = upload_mps(tn, ctx, eo.psi, center=eo.psi.center)
    f = abs(pg.inner(po)) / np.sqrt(pg.inner(pg) * po.inner(po))
    assert abs(f - 1.0) < 1e-9


def test_dmrg_config1_random_product_no_qn(tn, ctx):
    # Heisenberg N=20, no QN, random product start (seed 1234), 10 sweeps, maxdim 16 -> 64,
    # cutoff 1e-10, Lanczos krylovdim 3, maxiter 2.
    N = 20
    H = O.heisenberg_mpo(N, qn=False)
    v = O.random_product_vectors(N, 2, 1234)
    sched = [16, 16, 32, 32, 48, 48, 64, 64, 64, 64]
    for so, sg, eo, eg in _dmrg_both(tn, ctx, N, H, v, sched, 1e-10, krylovdim=3, qn=False):
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1]
    assert abs(sg.energy[-1] - GOLD["heisenberg_chain"]["20"]) < 1e-7


def test_dmrg_j1j2_cylinder_matches_ed(tn, ctx):
    Lx, Ly = 3, 4
    N = Lx * Ly
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.j1j2_cylinder_terms(Lx, Ly, 1.0, 0.5))
    Hg = tn.MPO(W, delta, pq, ctx)
    psi = tn.MPS.product(tn.models.neel_states(N), pq, ctx)
    params = tn.DMRGParams(maxdim=[32, 64, 64], nsweeps=[2, 2, 3], cutoff=1e-14)
    e, psi2 = tn.dmrg2(psi, Hg, params, solver_krylovdim=5, outputlevel=0)
    assert abs(e - GOLD["j1j2_cylinder"]["3x4"]) < 1e-9
    assert psi2.link(N)[0][0] == 0


def test_update_position_errors(tn, ctx):
    N = 6
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    env = tn.StateEnvs(tn.MPS.product(tn.models.neel_states(N), pq, ctx), tn.MPO(W, delta, pq, ctx))
    with pytest.raises(tn.TenNetError):
        tn.update_position_(env, tn.eig_solver, 2, 2, "left")  # center is at site 0
    with pytest.raises(tn.TenNetError):  # negative noise
        tn.update_position_(env, tn.eig_solver, 0, 1, "left", noise=-1e-3)
    e, err, eigs = tn.update_position_(env, tn.eig_solver, 0, 2, "left", maxdim=4)
    assert np.isfinite(e) and len(eigs) >= 1


def test_environments_match_oracle(tn, ctx):
    rng = np.random.default_rng(21)
    N, p = 10, 5
    mps = random_qn_mps(N, rng, maxsec_dim=3)
    H = O.mpo_from_terms(N, ed.heisenberg_chain_terms(N))
    env = tn.StateEnvs(upload_mps(tn, ctx, mps, center=p), upload_mpo(tn, ctx, H))
    env.position_(p, 2)
    eo = O.StateEnvs(mps, H)
    eo.position(p, 2)
    for i in range(1, p + 1):
        ref = eo.L[i]
        got = env.environment("left", i)
        assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), f"L[{i}]"
    for i in range(p + 1, N - 1):
        ref = eo.R[i]
        got = env.environment("right", i)
        assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), f"R[{i}]"


def test_block_svd_large_blocks_global_path(tn, ctx):
    # blocks whose work matrices exceed shared memory run on the global-memory path
    rng = np.random.default_rng(13)
    blocks = []
    for (r, c) in [(150, 150), (300, 120), (90, 260), (20, 20)]:
        U, _ = np.linalg.qr(rng.standard_normal((r, r)))
        V, _ = np.linalg.qr(rng.standard_normal((c, c)))
        k = min(r, c)
        s = np.exp(-np.linspace(0, 30, k)) * rng.uniform(0.5, 1.5, size=k)
        blocks.append((U[:, :k] * s) @ V[:k, :])
    kept, sv, err = tn.svd_truncate(blocks, maxdim=200, cutoff=1e-12, ctx=ctx)
    _, spec, kept_ref = O.svd_blocks_truncate(blocks, 200, 1, 1e-12)
    assert list(kept) == kept_ref
    for b, s in zip(blocks, sv):
        ref = np.linalg.svd(b, compute_uv=False)
        # LAPACK's gesdd is accurate to ~1e-16 of the largest value (absolute), so that is
        # the scale of the comparison
        assert np.allclose(s, ref, rtol=0, atol=1e-13 * ref[0])
