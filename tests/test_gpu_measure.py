"""Local expectation values on the GPU (tn_mps_expect_local) against the oracle.

Tolerance: 1e-12 absolute per site (values are O(1)); the sum of <S^z_i> over a state of
total S^z = 0 vanishes to 1e-12.
"""
import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import random_qn_mps, upload_mps

pytestmark = pytest.mark.gpu


def _oracle_state(psi, N):
    A = [psi.site(i) for i in range(N)]
    links = [psi.link_charges(i).astype(np.int64) for i in range(N + 1)]
    return O.MPS(A, links, O.SPIN_HALF_Q.copy(), center=psi.center)


def test_measure_ground_state_matches_oracle(tn, ctx):
    N = 12
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    env = tn.StateEnvs(tn.MPS.product(tn.models.neel_states(N), pq, ctx), H)
    sw = tn.SweepData()
    for md in (8, 16, 32, 32):
        tn.fullsweep_(env, tn.eig_solver, 2, sw, maxdim=md, cutoff=1e-12, outputlevel=0)
    psi = env.getpsi()
    sz = tn.measure(psi, "Sz")
    ref = O.expect_local(_oracle_state(psi, N), np.diag([0.5, -0.5]))
    assert np.allclose(sz, ref, atol=1e-12)
    assert abs(sum(sz)) < 1e-12
    assert tn.measure(psi, "Sz", pos=3) == pytest.approx(sz[3], abs=1e-15)
    assert np.allclose(tn.measure(psi, "Id"), 1.0, atol=1e-12)
    # mirror symmetry of the open chain ground state
    assert np.allclose(sz, -np.array(sz[::-1]), atol=1e-8)


def test_measure_mixed_canonical_random_state(tn, ctx):
    """A random charge-conserving MPS with the centre in the middle (left- and
    right-grouped site layouts both present), unnormalised."""
    rng = np.random.default_rng(7)
    N = 8
    mps = random_qn_mps(N, rng, maxsec_dim=3)
    psi = upload_mps(tn, ctx, mps, center=4)
    sz = np.diag([0.5, -0.5])
    # dense reference: contract the whole state
    v = mps.A[0]
    for a in mps.A[1:]:
        v = np.tensordot(v, a, axes=([-1], [0]))
    v = v.reshape(-1)
    nrm = v @ v
    ref = []
    for i in range(N):
        op = [np.eye(2)] * N
        op[i] = sz
        M = op[0]
        for o in op[1:]:
            M = np.kron(M, o)
        ref.append(v @ (M @ v) / nrm)
    got = psi.expect_local(sz)
    assert np.allclose(got, ref, atol=1e-12)
    nup = psi.expect_local(np.diag([1.0, 0.0]))
    assert np.allclose(nup, 0.5 + np.array(ref), atol=1e-12)


def _dense(mps):
    v = mps.A[0]
    for a in mps.A[1:]:
        v = np.tensordot(v, a, axes=([-1], [0]))
    return v.reshape(-1)


def _drop_sector(mps, i, rng):
    """The same kind of random state with the largest charge removed from link i."""
    links = [q.copy() for q in mps.links]
    links[i] = links[i][links[i] != links[i].max()]
    A = []
    for j in range(len(links) - 1):
        t = rng.standard_normal((len(links[j]), 2, len(links[j + 1])))
        A.append(t * O.qn_mask3(links[j], mps.phys_q, links[j + 1]))
    return O.MPS(A, links, mps.phys_q, center=0)


def test_overlap_random_states(tn, ctx):
    """<a|b> of two random charge-conserving states whose link sectors differ (a sector
    carried by one state only drops out), against the dense contraction and the oracle."""
    N = 10
    a = random_qn_mps(N, np.random.default_rng(11), maxsec_dim=3)
    b = _drop_sector(random_qn_mps(N, np.random.default_rng(12), maxsec_dim=4), 5,
                     np.random.default_rng(13))
    assert len(set(a.links[5]) - set(b.links[5])) == 1
    ga = upload_mps(tn, ctx, a, center=0)
    gb = upload_mps(tn, ctx, b, center=5)
    ref = _dense(a) @ _dense(b)
    assert O.inner(a, b) == pytest.approx(ref, rel=1e-12, abs=1e-12)
    scale = np.linalg.norm(_dense(a)) * np.linalg.norm(_dense(b))
    assert abs(ga.inner(gb) - ref) < 1e-12 * scale
    assert abs(gb.inner(ga) - ref) < 1e-12 * scale
    assert ga.inner(ga) == pytest.approx(_dense(a) @ _dense(a), rel=1e-12)


def test_overlap_split_vs_fp64_ground_state(tn):
    """The split-precision and FP64 sweeps reach the same ground state: |<psi_s|psi_d>| = 1
    to 1e-8 (fidelity of two normalised states, both from the same start)."""
    N = 16
    states = {}
    c = tn.Context()
    try:
        W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
        H = tn.MPO(W, delta, pq, c)
        for mode in ("fp64", "split"):
            c.set_precision(mode)
            env = tn.StateEnvs(tn.MPS.product(tn.models.neel_states(N), pq, c), H)
            sw = tn.SweepData()
            for md in (8, 16, 32, 64, 64, 64):
                tn.fullsweep_(env, tn.eig_solver, 2, sw, maxdim=md, cutoff=1e-12, outputlevel=0)
            states[mode] = env.getpsi()
        f = states["split"].inner(states["fp64"])
        assert abs(abs(f) - 1.0) < 1e-8
        assert states["fp64"].inner(states["fp64"]) == pytest.approx(1.0, abs=1e-12)
    finally:
        states.clear()
        c.close()


def test_operator_strings_match_dense(tn, ctx):
    """measure(psi, [("Sz", i), ("Sz", j), ...]) (src/mps/measure.jl:222-330): two- and
    three-site strings, charge-changing factors (S+ S-, Sx Sx: split into parts of definite
    charge change) and same-site products, on a DMRG ground state, against its dense state
    (1e-12)."""
    N = 10
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    env = tn.StateEnvs(tn.MPS.product(tn.models.neel_states(N), pq, ctx), tn.MPO(W, delta, pq, ctx))
    tn.dmrg_(env, tn.DMRGParams(nsweeps=[4, 4], maxdim=[16, 32], cutoff=1e-14), 2, outputlevel=0)
    psi = env.getpsi()
    v = psi.site(0)
    for i in range(1, N):
        v = np.tensordot(v, psi.site(i), axes=([-1], [0]))
    v = v.reshape(-1)
    v = v / np.linalg.norm(v)
    mats = {"Sz": np.diag([0.5, -0.5]), "Sx": np.array([[0.0, 0.5], [0.5, 0.0]]),
            "S+": np.array([[0.0, 1.0], [0.0, 0.0]]), "S-": np.array([[0.0, 0.0], [1.0, 0.0]])}

    def dense(pairs):
        ops = {}
        for name, site in pairs:
            ops[site] = ops[site] @ mats[name] if site in ops else mats[name]
        full = np.ones((1, 1))
        for i in range(N):
            full = np.kron(full, ops.get(i, np.eye(2)))
        return float(v @ full @ v)

    for pairs in ([("Sz", 1), ("Sz", 8)], [("Sx", 0), ("Sx", 5)], [("S+", 2), ("S-", 7)],
                  [("Sz", 3), ("Sz", 3)], [("Sz", 0), ("Sz", 4), ("Sz", 9)],
                  [("S+", 1), ("S-", 1), ("Sx", 6), ("Sx", 8)]):
        assert abs(tn.measure(psi, pairs) - dense(pairs)) < 1e-12, pairs
