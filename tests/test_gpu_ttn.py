"""TTN sweep engine (tn_ttn_* C ABI) against the TTN oracle and exact energies.

Tolerances: products at the initial centre 1e-12 relative (same gauge on both sides);
gauge-invariant quantities after isometry moves (<x|H x>, |H x|, the dense state) 1e-11;
per-sweep energies |dE/E| <= 1e-10 (FP64 and split precision); ground energies against
the free-fermion solution 1e-9 relative.
"""
import numpy as np
import pytest

from oracle import ttn_oracle as T

pytestmark = pytest.mark.gpu


def upload(tn, ctx, psi):
    return tn.ttn.TTN(psi.adj, psi.site_nodes, psi.d, psi.tensors, psi.center, ctx)


def model(tn, N, terms):
    return tn.ttn.CouplingModel(terms, N)


def tfim(N, seed):
    J, h = T.tfim_instance(N, seed)
    return T.tfim_terms(J, h), T.tfim_exact_energy(J, h)


def test_product_at_centre_matches_oracle(tn, ctx):
    N = 16
    terms, _ = tfim(N, 1)
    psi = T.random_ttn(N, 8, 3)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), model(tn, N, terms))
    x = np.random.default_rng(0).standard_normal(psi.tensors[psi.center].shape)
    yo = eo.product(x)
    yg = eg.product(x)
    assert np.linalg.norm(yg - yo) <= 1e-12 * np.linalg.norm(yo)
    assert eg.product_flops() > 0


@pytest.mark.parametrize("terms_of", ["tfim", "heisenberg"])
def test_positions_keep_state_and_effective_hamiltonian(tn, ctx, terms_of):
    N = 8
    terms = tfim(N, 2)[0] if terms_of == "tfim" else T.heisenberg_terms(N)
    psi = T.random_ttn(N, 16, 7)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), model(tn, N, terms))
    Hd = T.dense_hamiltonian(N, terms)
    for node in [(1, 3), (1, 1), (2, 2), (1, 4), (2, 1)]:
        eo.position(node)
        eg.position_(node)
        assert eg.orthocenter == node
        pg = eg.getpsi()
        tg = {v: pg[v] for v in pg.labels}
        dense_g = T.ttn_to_dense(T.TTN(psi.adj, psi.site_nodes, 2, tg, node))
        dense_o = T.ttn_to_dense(eo.psi)
        assert np.allclose(dense_g, dense_o, atol=1e-11)
        xg, xo = tg[node], eo.psi.tensors[node]
        hg, ho = eg.product(xg), eo.product(xo)
        assert abs(np.vdot(xg, hg) - np.vdot(xo, ho)) < 1e-11
        assert abs(np.vdot(xo, ho) - dense_o @ Hd @ dense_o) < 1e-11
        assert abs(np.linalg.norm(hg) - np.linalg.norm(ho)) < 1e-11


def _isometric(psi_g, center):
    for v in psi_g.labels:
        if v == center:
            continue
        t = psi_g[v]
        nxt = T.shortest_path({k: list(x) for k, x in psi_g.graph.items()}, v, center)[1]
        leg = psi_g.legs(v).index(("n", nxt))
        A = np.moveaxis(t, leg, -1).reshape(-1, t.shape[leg])
        if np.abs(A.T @ A - np.eye(A.shape[1])).max() > 1e-12:
            return False
    return True


def test_gpu_isometrize_blocked_qr(tn, ctx):
    """N = 32, chi = 64: the top nodes (64, 64, 64) take the blocked Householder path."""
    N, chi, seed = 32, 64, 5
    graph, sitenodes, tensors, center = tn.ttn.random_ttn_tensors(N, chi, seed)
    pg = tn.ttn.TTN(graph, sitenodes, 2, tensors, None, ctx).isometrize_(center)
    assert pg.orthocenter == center
    assert _isometric(pg, center)
    assert np.isclose(np.linalg.norm(pg[center]), 1.0, atol=1e-13)
    # same physical state as the oracle's host QR: compare <H> (gauge invariant)
    terms, _ = tfim(N, 3)
    po = T.random_ttn(N, chi, seed)
    eo = T.StateEnvsTTN(po, terms)
    eg = tn.ttn.StateEnvsTTN(pg, model(tn, N, terms))
    xo, xg = po.tensors[center], pg[center]
    assert abs(np.vdot(xg, eg.product(xg)) - np.vdot(xo, eo.product(xo))) < 1e-10
    # move the centre across the tree and back (QR moves through the big nodes)
    for node in [(3, 4), (1, 1), center]:
        eg.position_(node)
        eo.position(node)
        x_g = eg.getpsi()[node]
        x_o = eo.psi.tensors[node]
        assert abs(np.vdot(x_g, eg.product(x_g)) - np.vdot(x_o, eo.product(x_o))) < 1e-10
    assert _isometric(eg.getpsi(), center)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_sweeps_match_oracle(tn, precision):
    ctx = tn.Context(0, precision=precision, slices=5)
    N, chi = 16, 16
    terms, exact = tfim(N, 4)
    psi = T.random_ttn(N, chi, 9)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), model(tn, N, terms))
    path = tn.ttn.default_sweeppath(N)
    so, sg = T.SweepDataTTN(), tn.ttn.SweepDataTTN()
    for _ in range(3):
        T.fullsweep(eo, path, so, maxdim=chi)
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, maxdim=chi, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1] == chi
    assert abs(sg.energy[-1] - exact) < 1e-8 * abs(exact)
    st = sg.stats[-1]
    assert st["matvecs"] > 0 and st["heff_flops"] > 0 and st["sweep_ms"] > 0


def test_update_position_matches_oracle(tn, ctx):
    N = 8
    terms = T.heisenberg_terms(N)
    psi = T.random_ttn(N, 8, 1)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), model(tn, N, terms))
    for node in [(2, 1), (1, 2), (1, 3)]:
        e_o, _ = T.update_position(eo, node, maxdim=8)
        e_g = tn.ttn.update_position_(eg, tn.eig_solver, node, maxdim=8)
        assert abs(e_g - e_o) <= 1e-10 * abs(e_o)


def test_batched_sweeps_equal_single_sweeps_and_reach_exact(tn, ctx):
    """Three instances (different couplings and bond dimensions) swept in lockstep give
    the energies of three separate sweeps, and converge to the free-fermion energies."""
    N = 16
    chis = [4, 8, 16]
    insts = [tfim(N, 10 + i) for i in range(3)]
    path = tn.ttn.default_sweeppath(N)
    psis = [tn.ttn.default_randomTTN(N, c, 20 + i, ctx=ctx) for i, c in enumerate(chis)]
    models = [model(tn, N, t) for t, _ in insts]
    batch = tn.ttn.StateEnvsTTN.batch(psis, models)
    singles = [tn.ttn.StateEnvsTTN(p, m) for p, m in zip(psis, models)]
    swb = [tn.ttn.SweepDataTTN() for _ in range(3)]
    sws = [tn.ttn.SweepDataTTN() for _ in range(3)]
    for _ in range(4):
        tn.ttn.fullsweep_batch_(batch, path, tn.eig_solver, swb, maxdim=64, outputlevel=0)
        for e, s in zip(singles, sws):
            tn.ttn.fullsweep_(e, path, tn.eig_solver, s, maxdim=64, outputlevel=0)
    for i in range(3):
        assert np.allclose(swb[i].energy, sws[i].energy, rtol=1e-12, atol=0)
        assert swb[i].maxchi[-1] == chis[i]
    assert abs(swb[2].energy[-1] - insts[2][1]) < 1e-9 * abs(insts[2][1])
    # a member of a group cannot be swept alone
    with pytest.raises(tn.TenNetError):
        tn.ttn.fullsweep_(batch[0], path, tn.eig_solver, tn.ttn.SweepDataTTN(), outputlevel=0)


def test_optimize_api_and_argument_errors(tn, ctx):
    N = 8
    terms, exact = tfim(N, 6)
    psi = tn.ttn.default_randomTTN(N, 16, 2, ctx=ctx)
    H = model(tn, N, terms)
    params = tn.ttn.OptimizeParamsTTN(maxdim=[16], nsweeps=[5])
    e, psi2 = tn.ttn.optimize(psi, H, params, tn.ttn.default_sweeppath(N), outputlevel=0)
    assert abs(e - exact) < 1e-10 * abs(exact)
    assert psi2.maxlinkdim() == 16
    se = tn.ttn.StateEnvsTTN(psi, H)
    # the reference's check of the expansion settings (sweep_ttn.jl:146-149)
    with pytest.raises(tn.TenNetError, match="expand_numiter"):
        tn.ttn.fullsweep_(se, tn.ttn.default_sweeppath(N), tn.eig_solver, tn.ttn.SweepDataTTN(),
                          noise=1e-3, expand_numiter=1, outputlevel=0)
    with pytest.raises(tn.TenNetError):
        tn.ttn.fullsweep_(se, tn.ttn.default_sweeppath(N)[:-1], tn.eig_solver,
                          tn.ttn.SweepDataTTN(), outputlevel=0)


def test_batched_blocked_qr_matches_single(tn, ctx):
    """Tall QR moves of several instances share one cooperative panel launch; results equal
    those of each instance alone (N = 32: the (48|64)^3 top nodes take the blocked path)."""
    N = 32
    chis = [64, 48, 64]
    path = tn.ttn.default_sweeppath(N)
    insts = [tfim(N, 30 + i) for i in range(3)]
    psis = [tn.ttn.default_randomTTN(N, c, 40 + i, ctx=ctx) for i, c in enumerate(chis)]
    models = [model(tn, N, t) for t, _ in insts]
    batch = tn.ttn.StateEnvsTTN.batch(psis, models)
    swb = [tn.ttn.SweepDataTTN() for _ in range(3)]
    for _ in range(2):
        tn.ttn.fullsweep_batch_(batch, path, tn.eig_solver, swb, maxdim=64, outputlevel=0)
    for i in range(3):
        se = tn.ttn.StateEnvsTTN(psis[i], models[i])
        sw = tn.ttn.SweepDataTTN()
        for _ in range(2):
            tn.ttn.fullsweep_(se, path, tn.eig_solver, sw, maxdim=64, outputlevel=0)
        assert np.allclose(swb[i].energy, sw.energy, rtol=1e-10, atol=0), (i, swb[i].energy, sw.energy)
    assert _isometric(batch[0].getpsi(), batch[0].orthocenter)


def test_sweeps_with_blocked_qr_match_oracle(tn, ctx):
    """N = 32, chi = 64: the isometry moves through the (64, 64, 64) top nodes take the
    blocked (cooperative, double-float panel) Householder path; per-sweep energies agree
    with the oracle's host QR to 1e-10."""
    N, chi = 32, 64
    terms, _ = tfim(N, 8)
    psi = T.random_ttn(N, chi, 12)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), model(tn, N, terms))
    path = tn.ttn.default_sweeppath(N)
    so, sg = T.SweepDataTTN(), tn.ttn.SweepDataTTN()
    for _ in range(2):
        T.fullsweep(eo, path, so, maxdim=chi)
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, maxdim=chi, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
    assert _isometric(eg.getpsi(), eg.orthocenter)


def test_truncating_isometry_moves_match_oracle(tn, ctx):
    """Sweeping a chi = 16 TTN with maxdim = 8: every move through a 16-dimensional link
    takes the truncating SVD path of moveisometry_to_next! (src/ttn/ttn.jl:292-300)."""
    N = 16
    terms, _ = tfim(N, 21)
    psi = T.random_ttn(N, 16, 22)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), model(tn, N, terms))
    path = tn.ttn.default_sweeppath(N)
    so, sg = T.SweepDataTTN(), tn.ttn.SweepDataTTN()
    for _ in range(2):
        T.fullsweep(eo, path, so, maxdim=8)
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, maxdim=8, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1] == 8
    assert _isometric(eg.getpsi(), eg.orthocenter)


@pytest.mark.parametrize("N", [6, 12])
def test_ragged_trees_match_oracle(tn, ctx, N):
    """Site counts that are not powers of two: sites attach to layer-2 nodes
    (default_graph_sitenodes, src/ttn/ttn_generators.jl:69-96)."""
    terms, exact = tfim(N, 2)
    psi = T.random_ttn(N, 8, 3)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), model(tn, N, terms))
    path = tn.ttn.default_sweeppath(N)
    so, sg = T.SweepDataTTN(), tn.ttn.SweepDataTTN()
    for _ in range(3):
        T.fullsweep(eo, path, so, maxdim=8)
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, maxdim=8, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
    assert abs(sg.energy[-1] - exact) < 1e-7 * abs(exact)
