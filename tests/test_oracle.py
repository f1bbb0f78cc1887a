"""The oracle pinned against exact results (CPU only).

The reference's own tests assert nothing (test/*.jl contain no @test), so the oracle is
pinned against exact diagonalisation (tests/golden/ed_energies.json), against dense
linear algebra and against invariants.
"""
import json
import os

import numpy as np
import pytest

from oracle import ed
from oracle import tn_oracle as O

GOLD_DIR = os.path.join(os.path.dirname(__file__), "golden")
GOLD = json.load(open(os.path.join(GOLD_DIR, "ed_energies.json")))


@pytest.mark.parametrize("N", [6, 8, 10, 12])
def test_ed_fixture_reproduces(N):
    e = ed.ground_energy(N, ed.heisenberg_chain_terms(N))
    assert abs(e - GOLD["heisenberg_chain"][str(N)]) < 1e-12


def test_ed_known_values():
    # literature values of the open S=1/2 Heisenberg chain
    assert abs(GOLD["heisenberg_chain"]["12"] - (-5.142090632840)) < 1e-11
    assert abs(GOLD["heisenberg_chain"]["20"] - (-8.682473334398)) < 1e-11


@pytest.mark.parametrize("N", [8, 12])
def test_oracle_dmrg_matches_ed(N):
    H = O.heisenberg_mpo(N)
    psi = O.product_mps([0 if i % 2 == 0 else 1 for i in range(N)], O.SPIN_HALF_Q)
    sw, env = O.dmrg(psi, H, maxdim=[16, 32, 64], nsweeps=[2, 2, 3], cutoff=1e-14,
                     krylovdim=5)
    assert abs(sw.energy[-1] - GOLD["heisenberg_chain"][str(N)]) < 1e-10
    # the state stays in the S^z = 0 sector, right-canonical at the end
    assert env.psi.links[N][0] == 0 and env.psi.center == 0


def test_oracle_dmrg_no_qn_random_start():
    N = 10
    H = O.heisenberg_mpo(N, qn=False)
    v = O.random_product_vectors(N, 2, 1234)
    psi = O.product_mps(None, np.zeros(2, dtype=np.int64), vectors=v)
    sw, _ = O.dmrg(psi, H, maxdim=[16, 32], nsweeps=[3, 3], cutoff=1e-12, krylovdim=3)
    assert abs(sw.energy[-1] - GOLD["heisenberg_chain"]["10"]) < 1e-9


def test_oracle_j1j2_cylinder_matches_ed():
    Lx, Ly = 3, 4
    N = Lx * Ly
    H = O.mpo_from_terms(N, O.j1j2_cylinder_terms(Lx, Ly, 1.0, 0.5))
    psi = O.product_mps([0 if i % 2 == 0 else 1 for i in range(N)], O.SPIN_HALF_Q)
    sw, _ = O.dmrg(psi, H, maxdim=[32, 64, 64], nsweeps=[2, 2, 3], cutoff=1e-14, krylovdim=5)
    assert abs(sw.energy[-1] - GOLD["j1j2_cylinder"]["3x4"]) < 1e-9


def _dense_h(H):
    """Contract an MPO to a dense matrix (small N only)."""
    acc = H.W[0][0]  # (b, s', s)
    for W in H.W[1:]:
        # acc: (b, S', S) with S multi-index; W: (b, c, s', s)
        b, Sp, S = acc.shape
        acc = np.einsum("bxy,bcuv->cxuyv", acc, W).reshape(W.shape[1], Sp * 2, S * 2)
    return acc[0]


def test_mpo_builders_agree_with_exact_hamiltonian():
    N = 6
    H1 = O.heisenberg_mpo(N)
    H2 = O.mpo_from_terms(N, ed.heisenberg_chain_terms(N))
    D1, D2 = _dense_h(H1), _dense_h(H2)
    assert np.allclose(D1, D2, atol=1e-14)
    e = np.linalg.eigvalsh(D1)[0]
    assert abs(e - GOLD["heisenberg_chain"]["6"]) < 1e-12


def test_mpo_charges_conserved():
    N = 12
    H = O.mpo_from_terms(N, O.j1j2_cylinder_terms(3, 4))
    for i, W in enumerate(H.W):
        a, b, sp, s = np.nonzero(W)
        assert np.all(H.phys_q[sp] - H.phys_q[s] == H.delta[i + 1][b] - H.delta[i][a])


def test_truncation_rule_maxdim_and_cutoff():
    P = np.array([0.5, 0.3, 0.1, 0.05, 0.03, 0.02])
    n, err, docut = O.truncation_rule(P, maxdim=3, mindim=1, cutoff=1e-12)
    assert n == 3 and abs(err - 0.1) < 1e-15 and 0.05 < docut < 0.1
    n, err, docut = O.truncation_rule(P, maxdim=10, mindim=1, cutoff=0.06)
    # discard 0.02 + 0.03 = 0.05 <= 0.06, adding 0.05 would exceed
    assert n == 4 and abs(err - 0.05) < 1e-15
    n, err, docut = O.truncation_rule(P, maxdim=10, mindim=5, cutoff=0.5)
    assert n == 5
    n, err, docut = O.truncation_rule(P, maxdim=10, mindim=1, cutoff=0.0)
    assert n == 6 and docut == 0.0


def test_truncation_rule_degenerate_multiplet_is_cut_whole():
    P = np.array([0.4, 0.2, 0.2, 0.2])
    n, err, docut = O.truncation_rule(P, maxdim=2, mindim=1, cutoff=1e-15)
    # cut falls inside a degenerate triplet: the cut value is raised above it
    assert docut > 0.2
    blocks = [np.diag(np.sqrt([0.4, 0.2])), np.diag(np.sqrt([0.2])), np.diag(np.sqrt([0.2]))]
    _, spec, kept = O.svd_blocks_truncate(blocks, 2, 1, 1e-15)
    assert kept == [1, 0, 0]


def test_lanczos_restart_matches_eigh():
    rng = np.random.default_rng(7)
    n = 60
    A = rng.standard_normal((n, n))
    A = A + A.T
    x0 = rng.standard_normal(n)
    e, v, info = O.eigsolve_lowest(lambda x: A @ x, x0, krylovdim=20, maxiter=30, tol=1e-12)
    w, U = np.linalg.eigh(A)
    assert abs(e - w[0]) < 1e-9
    assert abs(abs(v @ U[:, 0]) - 1.0) < 1e-8


def test_lanczos_matvec_count_follows_restart_schedule():
    rng = np.random.default_rng(3)
    n = 200
    A = rng.standard_normal((n, n))
    A = A + A.T
    x0 = rng.standard_normal(n)
    _, _, info = O.eigsolve_lowest(lambda x: A @ x, x0, krylovdim=3, maxiter=2, tol=1e-14)
    # 3 vectors, restart keeping (3*3+0)//5 = 1 Ritz vector, 2 more expansions
    assert info.matvecs == 5 and info.numiter == 2


def test_heff_is_hermitian():
    rng = np.random.default_rng(11)
    N = 6
    H = O.heisenberg_mpo(N)
    psi = O.product_mps([0, 1, 0, 1, 0, 1], O.SPIN_HALF_Q)
    sw, env = O.dmrg(psi, H, maxdim=[8], nsweeps=[1], cutoff=1e-14)
    env.position(2, 2)
    sh = (len(env.psi.links[2]), 2, 2, len(env.psi.links[4]))
    mask = (env.psi.links[2][:, None, None, None] + O.SPIN_HALF_Q[None, :, None, None]
            + O.SPIN_HALF_Q[None, None, :, None]) == env.psi.links[4][None, None, None, :]
    x = rng.standard_normal(sh) * mask
    y = rng.standard_normal(sh) * mask
    assert abs(np.vdot(x, env.product2(2, y)) - np.vdot(env.product2(2, x), y)) < 1e-12


def test_entropy():
    assert O.entropy([1.0]) == 0.0
    assert abs(O.entropy([0.5, 0.5]) - np.log(2)) < 1e-15


def test_exponentiate_matches_expm():
    import scipy.linalg as sla
    rng = np.random.default_rng(0)
    A = rng.standard_normal((40, 40))
    A = A + A.T
    x = rng.standard_normal(40)
    for t, kd in ((-0.3, 30), (-0.3, 10), (-2.0, 8)):   # the last two restart
        y, mv = O.exponentiate(lambda v: A @ v, t, x, krylovdim=kd)
        ref = sla.expm(t * A) @ x
        assert np.linalg.norm(y - ref) <= 1e-11 * np.linalg.norm(ref)


def test_oracle_tdvp_imaginary_time_lowers_energy():
    N = 8
    H = O.heisenberg_mpo(N)
    env = O.StateEnvs(O.product_mps([0, 1] * 4, O.SPIN_HALF_Q), H)
    sw = O.SweepData()
    es = [O.tdvp_sweep(env, sw, -1.0, 16, 1e-14) for _ in range(40)]
    assert all(b <= a + 1e-12 for a, b in zip(es, es[1:]))
    assert abs(es[-1] - GOLD["heisenberg_chain"]["8"]) < 1e-8


def test_inner_matches_dense():
    from tests.helpers import random_qn_mps
    a = random_qn_mps(7, np.random.default_rng(3), maxsec_dim=3)
    b = random_qn_mps(7, np.random.default_rng(4), maxsec_dim=2)

    def dense(m):
        v = m.A[0]
        for t in m.A[1:]:
            v = np.tensordot(v, t, axes=([-1], [0]))
        return v.reshape(-1)

    assert O.inner(a, b) == pytest.approx(dense(a) @ dense(b), rel=1e-12, abs=1e-12)
    assert O.inner(a, a) == pytest.approx(dense(a) @ dense(a), rel=1e-12)


def test_real_time_tdvp_quench_matches_exact():
    """Two-site TDVP with complex steps tau = -0.05i (the real-time workload's step) from the
    Neel state of the N = 12 chain: <S^z_i(t)> against exact evolution (quench_sz.json) at
    t = 0.5 and 1.0.  The difference is the TDVP projection error of the small bond
    dimensions the sweep grows from a product state (7e-8 and 4e-7 here), bounded by 1e-6."""
    with open(os.path.join(GOLD_DIR, "quench_sz.json")) as f:
        q = json.load(f)
    N = q["N"]
    psi = O.product_mps([0 if i % 2 == 0 else 1 for i in range(N)], O.SPIN_HALF_Q)
    psi.A = [a.astype(np.complex128) for a in psi.A]
    env = O.StateEnvs(psi, O.heisenberg_mpo(N))
    sw = O.SweepData()
    t = 0.0
    for tk, ref in zip(q["times"], q["sz"]):
        while t < tk - 1e-12:
            O.tdvp_sweep(env, sw, -0.05j, maxdim=64, cutoff=1e-12, krylovdim=30)
            t += 0.05
        sz = O.expect_local(env.psi, np.diag([0.5, -0.5]))
        assert np.abs(sz - np.array(ref)).max() < 1e-6
        assert abs(O.inner(env.psi, env.psi) - 1.0) < 1e-12


def test_oracle_one_site_sweeps_reach_ed():
    """fullsweep! with nsite = 1 (src/mps/sweep.jl:94-196, _update_one_site! of
    src/mps/update_site.jl:94-190): after a two-site warm-up the one-site sweeps keep the
    bond dimensions, lower the energy monotonically, keep every site but the centre an
    isometry, and at full bond dimension (N = 8, chi = 16) reach the exact ground energy."""
    N = 8
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    env = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    sw = O.SweepData()
    for md in (4, 16):
        O.fullsweep(env, sw, md, 1e-14, 1, 4, 2, 1e-14)
    chi = env.psi.maxlinkdim()
    for _ in range(3):
        O.fullsweep1(env, sw, 16, 1e-14, 1, 4, 2, 1e-14)
        assert sw.energy[-1] <= sw.energy[-2] + 1e-12
        assert env.psi.maxlinkdim() == chi
    for i in range(1, N):
        A = env.psi.A[i].reshape(env.psi.A[i].shape[0], -1)
        assert np.allclose(A @ A.T, np.eye(A.shape[0]), atol=1e-12)


def test_oracle_one_site_noise():
    """One-site DMRG with noise (src/mps/update_site.jl:135-152) grows the bonds of a product
    state and reaches the exact ground energy; without noise the bonds stay at 1."""
    N = 10
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    env = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    sw = O.SweepData()
    O.fullsweep1(env, sw, 8, 1e-14, 1, 4, 2, 1e-14)
    assert sw.maxchi[-1] == 1
    for md, nz in [(8, 1e-3), (16, 5e-4), (32, 2.5e-4), (32, 0.0), (32, 0.0)]:
        O.fullsweep1(env, sw, md, 1e-14, 1, 4, 2, 1e-14, noise=nz)
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))
    assert sw.maxchi[-1] > 8
    assert abs(sw.energy[-1] - gold["heisenberg_chain"][str(N)]) < 1e-10

    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))
    assert abs(sw.energy[-1] - gold["heisenberg_chain"][str(N)]) < 1e-10


def test_checkpoint_arrays_round_trip():
    """save_checkpoint / load_checkpoint host format: charge blocks, links, centre and the
    sweep history come back unchanged (CPU only: the arrays, not the device MPS)."""
    import __graft_entry__ as g
    tn = g.load_package()
    rng = np.random.default_rng(3)
    N = 6
    links = [np.array([0])] + [np.repeat(np.array([q for q in range(-i, i + 1, 2)
                                                   if abs(q) <= N - i]),
                                         rng.integers(1, 4, size=len([q for q in range(-i, i + 1, 2)
                                                                      if abs(q) <= N - i])))
                               for i in range(1, N)] + [np.array([0])]
    pq = O.SPIN_HALF_Q
    tensors = [rng.standard_normal((len(links[i]), 2, len(links[i + 1])))
               * O.qn_mask3(links[i], pq, links[i + 1]) for i in range(N)]
    sw = tn.SweepData(sweepcount=2, maxchi=[4, 8], energy=[-1.0, -1.5], entropy=[0.1, 0.2],
                      maxtruncerr=[1e-9, 1e-10], lasteigs=[np.array([0.7, 0.3]), np.array([1.0])],
                      stats=[{"sweep_ms": 1.0}])
    z = tn.checkpoint_arrays(tensors, links, pq, 0, sw)
    t2, l2, pq2, c2, sw2 = tn.arrays_from_checkpoint(z)
    assert c2 == 0 and np.array_equal(pq2, pq)
    for a, b in zip(tensors, t2):
        assert np.array_equal(a, b)
    for a, b in zip(links, l2):
        assert np.array_equal(a, b)
    assert sw2.sweepcount == 2 and sw2.maxchi == [4, 8] and sw2.energy == [-1.0, -1.5]
    assert all(np.array_equal(a, b) for a, b in zip(sw.lasteigs, sw2.lasteigs))
    assert sw2.stats == [{"sweep_ms": 1.0}]
    # only the allowed entries are stored
    assert sum(v.size for k, v in z.items() if k.startswith("blocks_")) < sum(t.size for t in tensors)
    # a complex state (real-time evolution) keeps its imaginary parts
    ct = [t + 1j * rng.standard_normal(t.shape) * (t != 0) for t in tensors]
    t3 = tn.arrays_from_checkpoint(tn.checkpoint_arrays(ct, links, pq, 0, None))[0]
    for a, b in zip(ct, t3):
        assert b.dtype == np.complex128 and np.array_equal(a, b)


def test_oracle_noise_term():
    """noiseterm + replacebond! with an eigen perturbation (src/mps/update_site.jl:59-76):
    a noise below the threshold reproduces the plain SVD split, a real noise schedule reaches
    the exact ground energy and leaves right isometries behind."""
    N = 10
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]

    def run(sched):
        env = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
        sw = O.SweepData()
        for md, nz in sched:
            O.fullsweep(env, sw, md, 1e-14, 1, 4, 2, 1e-14, noise=nz)
        return sw, env

    sw0, _ = run([(4, 0.0), (8, 0.0), (16, 0.0)])
    sw1, _ = run([(4, 1e-14), (8, 1e-14), (16, 1e-14)])
    assert max(abs(a - b) for a, b in zip(sw0.energy, sw1.energy)) < 1e-12
    sw2, env = run([(4, 1e-3), (8, 5e-4), (16, 2.5e-4), (32, 0.0), (32, 0.0)])
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))
    assert abs(sw2.energy[-1] - gold["heisenberg_chain"][str(N)]) < 1e-10
    for i in range(1, N):
        A = env.psi.A[i].reshape(env.psi.A[i].shape[0], -1)
        assert np.allclose(A @ A.T, np.eye(A.shape[0]), atol=1e-12)


@pytest.mark.parametrize("nsite", [1, 2])
def test_oracle_excited_state_projector(nsite):
    """ProjMPO_MPS2 (src/mps/projmpo_mps2.jl:94-101) with the ground state as M and weight 10
    (the reference's own excited-state test, test/test_MPS_DMRG.jl:71-96): DMRG reaches the
    second-lowest energy of the S^z = 0 sector, and the result is orthogonal to M."""
    N = 8
    H = O.heisenberg_mpo(N)
    D = _dense_h(H)
    sz = np.array([sum(0.5 - ((k >> (N - 1 - i)) & 1) for i in range(N)) for k in range(2 ** N)])
    sec = np.nonzero(sz == 0)[0]
    ev = np.linalg.eigvalsh(D[np.ix_(sec, sec)])
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    sw, env = O.dmrg(O.product_mps(start, O.SPIN_HALF_Q), H, maxdim=[16, 32], nsweeps=[3, 4],
                     cutoff=1e-14)
    assert abs(sw.energy[-1] - ev[0]) < 1e-10
    gr = env.psi
    with pytest.raises(ValueError):
        O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H, [gr], weight=0.0)
    ex = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H, [gr], weight=10.0)
    sx = O.SweepData()
    # two-site sweeps grow the bonds; one-site ones then run from the grown state
    for md in (16, 32, 32, 32, 32, 32):
        O.fullsweep(ex, sx, md, 1e-14, 1, 5, 2, 1e-14)
    if nsite == 1:
        for _ in range(3):
            O.fullsweep1(ex, sx, 32, 1e-14, 1, 5, 2, 1e-14)
    assert abs(sx.energy[-1] - ev[1]) < 1e-8
    assert abs(O.inner(ex.psi, gr)) < 1e-6


def test_oracle_one_site_tdvp_is_exact_at_full_rank():
    """One-site TDVP (tdvpsweep! with nsite = 1: _update_one_site! with exp_solver and the
    zero-site reverse step, src/mps/update_site.jl:94-190) has no projection error when every
    bond has full rank: from a full-rank N = 6 state (two-site real-time sweeps) five sweeps of
    tau = -0.1i and of tau = -0.1 reproduce exp(-i H t) psi and exp(-H t) psi / |.| of the
    dense Hamiltonian (t = 0.5) to 1e-11, and the real-time sweeps conserve the energy."""
    import scipy.linalg as sl
    from tests.helpers import dense_mpo
    N = 6
    H = O.heisenberg_mpo(N)
    D = dense_mpo(H)
    psi = O.product_mps([0 if i % 2 == 0 else 1 for i in range(N)], O.SPIN_HALF_Q)
    psi.A = [a.astype(np.complex128) for a in psi.A]
    env = O.StateEnvs(psi, H)
    sw = O.SweepData()
    for _ in range(6):
        O.tdvp_sweep(env, sw, -0.3j, 8, 1e-14)
    assert [len(q) for q in env.psi.links] == [1, 2, 4, 8, 4, 2, 1]

    def dense(m):
        v = m.A[0]
        for a in m.A[1:]:
            v = np.tensordot(v, a, axes=([-1], [0]))
        return v.reshape(-1)

    psi0 = dense(env.psi)
    for tau, ref in ((-0.1j, sl.expm(-0.5j * D) @ psi0), (-0.1, sl.expm(-0.5 * D) @ psi0)):
        e = O.StateEnvs(env.psi, H)
        s = O.SweepData()
        for _ in range(5):
            O.tdvp_sweep(e, s, tau, 64, 1e-14, nsite=1)
        ref = ref / np.linalg.norm(ref)
        assert np.abs(dense(e.psi) - ref).max() < 1e-11
        if isinstance(tau, complex):
            assert np.ptp(s.energy) < 1e-12


@pytest.mark.parametrize("tau", [None, -0.1, -0.1j])
def test_oracle_dynamic_sweep_limits_are_the_fixed_sweeps(tau):
    """dynamic_fullsweep!'s mixed sweep (src/mps/sweep.jl:284-355) with every bond choosing
    two sites (threshold 0, no link at maxdim) is the two-site sweep, and with every bond
    choosing one site (threshold inf) the one-site sweep (sweep.jl:94-196), bit for bit, with
    the eigensolver and with real and complex TDVP steps; at maxdim every bond takes one site
    whatever the threshold."""
    N = 8
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]

    def prepared():
        psi = O.product_mps(start, O.SPIN_HALF_Q)
        if isinstance(tau, complex):
            psi.A = [a.astype(np.complex128) for a in psi.A]
        env, sw = O.StateEnvs(psi, H), O.SweepData()
        for _ in range(2):
            if tau is None:
                O.fullsweep(env, sw, 64, 1e-12)
            else:
                O.tdvp_sweep(env, sw, tau, 64, 1e-12)
        return env, sw

    for thr, nsite in ((0.0, 2), (np.inf, 1)):
        a, sa = prepared()
        b, sb = prepared()
        left, right = O.dynamic_sweep(a, sa, 64, 1e-12, thr, tau)
        assert left == right == [nsite] * (N - 1)
        if tau is None:
            (O.fullsweep if nsite == 2 else O.fullsweep1)(b, sb, 64, 1e-12)
        else:
            O.tdvp_sweep(b, sb, tau, 64, 1e-12, nsite=nsite)
        assert sa.energy[-1] == sb.energy[-1] and sa.entropy[-1] == sb.entropy[-1]
        for x, y in zip(a.psi.A, b.psi.A):
            assert np.array_equal(x, y)
        for x, y in zip(sa.lasteigs, sb.lasteigs):
            assert np.array_equal(x, y)
    a, sa = prepared()
    dims = [len(q) for q in a.psi.links]
    md = max(dims)
    left, _ = O.dynamic_sweep(a, sa, md, 1e-12, 0.0, tau)
    # the left half meets each link as the previous sweep left it
    assert left == [1 if dims[b + 1] >= md else 2 for b in range(N - 1)]
    assert 1 in left and 2 in left


def test_oracle_update_h_reuse_and_recalc():
    """updateH! (src/mps/state_envs.jl:181-212): with recalcEnv = false the first half sweep
    after the change reads right environments of the old MPO, so after a quench of the
    couplings the two choices differ (here by ~1.7e-7 in the energy); with the MPO unchanged
    the reused environments are exact and both choices agree to rounding."""
    N = 10
    H1, H2 = O.heisenberg_mpo(N), O.heisenberg_mpo(N, 0.5, Jz=2.0)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]

    def run(Hnew, recalc):
        psi = O.product_mps(start, O.SPIN_HALF_Q)
        psi.A = [a.astype(np.complex128) for a in psi.A]
        env, sw = O.StateEnvs(psi, H1), O.SweepData()
        for _ in range(4):
            O.tdvp_sweep(env, sw, -0.2j, 16, 1e-12)
        env.update_h(Hnew, recalc)
        O.tdvp_sweep(env, sw, -0.2j, 16, 1e-12)
        return sw.energy[-1]

    assert abs(run(H2, True) - run(H2, False)) > 1e-8
    assert abs(run(H1, True) - run(H1, False)) < 1e-12
