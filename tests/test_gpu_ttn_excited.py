"""Excited-state TTN sweeps on the GPU: LinkProjTTN / EnvCouplingModelProjTTN (TenNetLib
src/ttn/linkproj.jl, src/ttn/environment.jl:44-110, StateEnvsTTN(psi, H, Ms; weight) of
src/ttn/state_envs_ttn.jl:36-52) against the oracle's restatement, as in the reference's own
excited-state test (test/test_TTN.jl:36-48: the ground state as M, weight 10).

Tolerances: the product H_eff x + w sum_k m_k (m_k . x) at the initial centre 1e-12
relative (same gauge); after isometry moves the gauge-invariant <x|H_P x> and |H_P x| 1e-11;
per sweep |dE/E| <= 1e-10 (FP64 and split precision); at the end the second eigenvalue of
the dense Hamiltonian to 1e-8 and an overlap with the ground state below 1e-6."""
import numpy as np
import pytest

from oracle import ttn_oracle as T

pytestmark = pytest.mark.gpu
N = 8


def upload(tn, ctx, psi):
    return tn.ttn.TTN(psi.adj, psi.site_nodes, psi.d, psi.tensors, psi.center, ctx)


def dense_of(psi_g, psi_o):
    tg = {v: psi_g[v] for v in psi_g.labels}
    return T.ttn_to_dense(T.TTN(psi_o.adj, psi_o.site_nodes, 2, tg, psi_g.orthocenter))


def _instance():
    J, h = T.tfim_instance(N, 3)
    terms = T.tfim_terms(J, h)
    ev = np.linalg.eigvalsh(T.dense_hamiltonian(N, terms))
    return terms, ev


def test_projected_product_matches_oracle(tn, ctx):
    terms, _ = _instance()
    psi = T.random_ttn(N, 8, 3)
    Ms = [T.random_ttn(N, 16, 1), T.random_ttn(N, 6, 2)]  # overlaps 8 x 16 and 8 x 6
    eo = T.StateEnvsTTN(psi, terms, Ms, weight=3.5)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), tn.ttn.CouplingModel(terms, N),
                             [upload(tn, ctx, m) for m in Ms], weight=3.5)
    x = np.random.default_rng(0).standard_normal(psi.tensors[psi.center].shape)
    yo, yg = eo.product(x), eg.product(x)
    assert np.linalg.norm(yg - yo) <= 1e-12 * np.linalg.norm(yo)
    for node in [(1, 3), (1, 1), (2, 2), (1, 4), (2, 1)]:
        eo.position(node)
        eg.position_(node)
        xg, xo = eg.getpsi()[node], eo.psi.tensors[node]
        hg, ho = eg.product(xg), eo.product(xo)
        assert abs(np.vdot(xg, hg) - np.vdot(xo, ho)) < 1e-11, node
        assert abs(np.linalg.norm(hg) - np.linalg.norm(ho)) < 1e-11, node
    # removing the projectors gives the plain product (same gauge: psi read back from the GPU)
    eg.set_projectors([], 0.0)
    pg = eg.getpsi()
    plain = T.StateEnvsTTN(T.TTN(psi.adj, psi.site_nodes, 2, {v: pg[v] for v in pg.labels},
                                 pg.orthocenter), terms)
    xg = pg[pg.orthocenter]
    yp = plain.product(xg)
    assert np.linalg.norm(eg.product(xg) - yp) <= 1e-12 * np.linalg.norm(yp)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_excited_sweeps_match_oracle(tn, precision):
    ctx = tn.Context(0, precision=precision, slices=5)
    terms, ev = _instance()
    path = tn.ttn.default_sweeppath(N)
    se = T.StateEnvsTTN(T.random_ttn(N, 16, 1), terms)
    T.optimize(se, [16], [6], path)
    gs = se.psi
    start = T.random_ttn(N, 16, 2)
    eo = T.StateEnvsTTN(start, terms, [gs], weight=10.0)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, start), tn.ttn.CouplingModel(terms, N),
                             [upload(tn, ctx, gs)], weight=10.0)
    so, sg = T.SweepDataTTN(), tn.ttn.SweepDataTTN()
    for _ in range(8):
        T.fullsweep(eo, path, so, maxdim=16)
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, maxdim=16, outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1]
    assert abs(sg.energy[-1] - ev[1]) < 1e-8
    ov = float(np.vdot(dense_of(eg.getpsi(), start), T.ttn_to_dense(gs)))
    assert abs(ov) < 1e-6


def test_optimize_api_with_projectors(tn, ctx):
    terms, ev = _instance()
    H = tn.ttn.CouplingModel(terms, N)
    path = tn.ttn.default_sweeppath(N)
    params = tn.ttn.OptimizeParamsTTN(maxdim=[16], nsweeps=[6])
    e0, gs = tn.ttn.optimize(tn.ttn.default_randomTTN(N, 16, 1, ctx=ctx), H, params, path,
                             outputlevel=0)
    assert abs(e0 - ev[0]) < 1e-10
    params = tn.ttn.OptimizeParamsTTN(maxdim=[16], nsweeps=[8])
    e1, ex = tn.ttn.optimize(tn.ttn.default_randomTTN(N, 16, 2, ctx=ctx), H, [gs], params, path,
                             weight=10.0, outputlevel=0)
    assert abs(e1 - ev[1]) < 1e-8
    ref = T.random_ttn(N, 16, 1)
    ov = float(np.vdot(dense_of(ex, ref), dense_of(gs, ref)))
    assert abs(ov) < 1e-6
    for w in (0.0, -1.0):
        with pytest.raises(tn.TenNetError, match="weight"):
            tn.ttn.StateEnvsTTN(tn.ttn.default_randomTTN(N, 16, 2, ctx=ctx), H, [gs], weight=w)
    with pytest.raises(tn.TenNetError, match="weight"):
        tn.ttn.optimize(tn.ttn.default_randomTTN(N, 16, 2, ctx=ctx), H, [gs], params, path,
                        outputlevel=0)
