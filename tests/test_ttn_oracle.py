"""The TTN oracle pinned against exact results, and the package's tree bookkeeping against
the oracle (CPU only)."""
import numpy as np
import pytest

from oracle import ttn_oracle as T


@pytest.mark.parametrize("N", [5, 6, 7, 8, 12, 16, 24, 64])
def test_package_tree_matches_oracle(tn, N):
    g1, s1 = tn.ttn.default_graph_sitenodes(N)
    g2, s2 = T.default_graph_sitenodes(N)
    assert g1 == g2
    assert s1 == s2
    assert tn.ttn.default_sweeppath(N) == T.default_sweeppath(N, g2.keys())
    assert tn.ttn.eccentric_central_node(g1, set(s1)) == T.eccentric_center(g2, set(s2))


def test_default_tree_64_sites():
    g, s = T.default_graph_sitenodes(64)
    assert len(g) == 62
    assert s[0] == s[1] == (1, 1) and s[63] == (1, 32)
    assert g[(5, 1)] == [(4, 1), (4, 2), (5, 2)]
    path = T.default_sweeppath(64, g.keys())
    assert len(path) == 62 and set(path) == set(g)
    assert path[:6] == [(5, 1), (5, 2), (4, 4), (4, 3), (4, 2), (4, 1)]


def test_random_ttn_state_matches_package_draws(tn):
    """The package draws the same Gaussian tensors as the oracle (same stream, same order);
    isometrisation keeps the state, so the normalised state vectors agree."""
    N, chi, seed = 8, 4, 11
    graph, sitenodes, tensors, center = tn.ttn.random_ttn_tensors(N, chi, seed)
    raw = T.TTN(graph, sitenodes, 2, tensors, center)
    v1 = T.ttn_to_dense(raw)
    v1 /= np.linalg.norm(v1)
    psi = T.random_ttn(N, chi, seed)
    assert psi.center == center
    v2 = T.ttn_to_dense(psi)
    assert np.allclose(v1, v2, atol=1e-13)


def test_isometries_and_norm():
    psi = T.random_ttn(16, 8, 3)
    c = psi.center
    for v in psi.nodes:
        if v == c:
            continue
        nxt = T.shortest_path(psi.adj, v, c)[1]
        A, _ = T._matricize(psi.tensors[v], psi.leg_index(v, nxt))
        assert np.allclose(A.T @ A, np.eye(A.shape[1]), atol=1e-13)
    assert np.isclose(np.linalg.norm(psi.tensors[c]), 1.0)


def test_tfim_free_fermion_matches_ed():
    for seed in (1, 2):
        J, h = T.tfim_instance(8, seed)
        H = T.dense_hamiltonian(8, T.tfim_terms(J, h))
        assert abs(np.linalg.eigvalsh(H)[0] - T.tfim_exact_energy(J, h)) < 1e-12


def test_oracle_product_is_the_projected_hamiltonian():
    N = 8
    J, h = T.tfim_instance(N, 4)
    terms = T.tfim_terms(J, h)
    psi = T.random_ttn(N, 16, 5)
    se = T.StateEnvsTTN(psi, terms)
    Hd = T.dense_hamiltonian(N, terms)
    v = T.ttn_to_dense(se.psi)
    x = se.psi.tensors[se.psi.center]
    assert np.isclose(np.vdot(x, se.product(x)), v @ Hd @ v, atol=1e-12)
    se.position((1, 3))
    x = se.psi.tensors[(1, 3)]
    v = T.ttn_to_dense(se.psi)
    assert np.isclose(np.vdot(x, se.product(x)), v @ Hd @ v, atol=1e-12)


def test_oracle_sweeps_reach_exact_energies():
    N = 16
    J, h = T.tfim_instance(N, 5)
    se = T.StateEnvsTTN(T.random_ttn(N, 32, 2), T.tfim_terms(J, h))
    g, _ = T.default_graph_sitenodes(N)
    sw = T.optimize(se, [32], [4], T.default_sweeppath(N, g.keys()))
    assert abs(sw.energy[-1] - T.tfim_exact_energy(J, h)) < 1e-10
    assert sw.maxchi[-1] == 32
    N = 8
    se = T.StateEnvsTTN(T.random_ttn(N, 16, 4), T.heisenberg_terms(N))
    g, _ = T.default_graph_sitenodes(N)
    sw = T.optimize(se, [16], [4], T.default_sweeppath(N, g.keys()))
    e0 = np.linalg.eigvalsh(T.dense_hamiltonian(N, T.heisenberg_terms(N)))[0]
    assert abs(sw.energy[-1] - e0) < 1e-10


def test_ttn_oracle_excited_state_projector():
    """EnvCouplingModelProjTTN / LinkProjTTN (src/ttn/environment.jl:44-110,
    src/ttn/linkproj.jl): with the ground state projected out (weight 10, as in the
    reference's test/test_TTN.jl:36-48) the sweep reaches the second eigenvalue of the dense
    Hamiltonian and a state orthogonal to the ground state."""
    N = 8
    J, h = T.tfim_instance(N, 3)
    terms = T.tfim_terms(J, h)
    ev = np.linalg.eigvalsh(T.dense_hamiltonian(N, terms))
    path = T.default_sweeppath(N, T.default_graph_sitenodes(N)[0].keys())
    se = T.StateEnvsTTN(T.random_ttn(N, 16, 1), terms)
    sw = T.optimize(se, [16], [6], path)
    assert abs(sw.energy[-1] - ev[0]) < 1e-10
    gs = se.psi
    with pytest.raises(ValueError):
        T.StateEnvsTTN(T.random_ttn(N, 16, 2), terms, [gs], weight=0.0)
    ex = T.StateEnvsTTN(T.random_ttn(N, 16, 2), terms, [gs], weight=10.0)
    sx = T.optimize(ex, [16], [8], path)
    assert abs(sx.energy[-1] - ev[1]) < 1e-8
    ov = float(np.vdot(T.ttn_to_dense(ex.psi), T.ttn_to_dense(gs)))
    assert abs(ov) < 1e-6


def test_ttn_oracle_subspace_expansion_grows_bonds_to_exact():
    """fullsweep! with noise > 0 (subspace_expand!, src/ttn/update_site_ttn.jl:75-109, and the
    noisy branch of src/ttn/sweep_ttn.jl:180-243), as in the reference's own TTN test
    (test/test_TTN.jl:26-48: a chi = 12 random TTN, maxdim 128, cutoff 1e-14, noise 1e-2,
    noisedecay 5, noise off after 2 sweeps): the bonds grow beyond the initial 12 and the
    Heisenberg N = 12 ground energy and, with the ground state projected out (weight 10),
    the second eigenvalue of the dense Hamiltonian are reached.  The padding stream is
    deterministic: the same seed gives the same sweep."""
    N = 12
    terms = T.heisenberg_terms(N)
    ev = np.linalg.eigvalsh(T.dense_hamiltonian(N, terms))
    path = T.default_sweeppath(N, T.default_graph_sitenodes(N)[0].keys())
    kw = dict(cutoff=1e-14, noise=1e-2, noisedecay=5, disable_noise_after=2, seed=7)
    se = T.StateEnvsTTN(T.random_ttn(N, 12, 1), terms)
    sw = T.optimize(se, [128], [5], path, **kw)
    assert sw.maxchi[0] > 12
    assert abs(sw.energy[-1] - ev[0]) < 1e-10
    se2 = T.StateEnvsTTN(T.random_ttn(N, 12, 1), terms)
    sw2 = T.optimize(se2, [128], [5], path, **kw)
    assert sw2.energy == sw.energy and sw2.maxchi == sw.maxchi
    ex = T.StateEnvsTTN(T.random_ttn(N, 12, 2), terms, [se.psi], weight=10.0)
    sx = T.optimize(ex, [128], [10], path, cutoff=1e-14, noise=1e-2, noisedecay=5,
                    disable_noise_after=6, seed=8)
    assert abs(sx.energy[-1] - ev[1]) < 1e-8
    vals = T.padding_values(7, 3, 1, 0, 5)
    assert vals.min() >= -1.0 and vals.max() < 1.0 and len(set(vals.tolist())) == 5
