"""TTN at the benchmark's scale: binary trees of 64 sites, transverse-field Ising instances
with random couplings (the benchmark's instances), maxdim 64, 128 and 256.

 * The maxdim-64 instance against the TTN oracle from the same random start: two sweeps,
   per-sweep energies |dE/E| <= 1e-10 and the same bond dimension.
 * The three instances swept in lockstep to convergence (energy change below 1e-12
   relative, at most 16 sweeps): each within 1e-9 relative of its free-fermion ground
   energy and variational (E >= E_exact - 1e-12 |E_exact|).
"""
import pytest

from oracle import ttn_oracle as T

pytestmark = pytest.mark.gpu

N = 64
CHIS = [64, 128, 256]


def _instance(i):
    J, h = T.tfim_instance(N, 1000 + i)
    return T.tfim_terms(J, h), T.tfim_exact_energy(J, h)


def test_maxdim64_sweeps_match_oracle(tn):
    ctx = tn.Context(0, precision="split", slices=5)
    terms, _ = _instance(0)
    psi = T.random_ttn(N, CHIS[0], 2000)
    eo = T.StateEnvsTTN(psi, terms)
    eg = tn.ttn.StateEnvsTTN(tn.ttn.TTN(psi.adj, psi.site_nodes, psi.d, psi.tensors, psi.center,
                                        ctx), tn.ttn.CouplingModel(terms, N))
    path = tn.ttn.default_sweeppath(N)
    so, sg = T.SweepDataTTN(), tn.ttn.SweepDataTTN()
    for _ in range(2):
        T.fullsweep(eo, path, so, maxdim=CHIS[0])
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, maxdim=CHIS[0], outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1] == CHIS[0]


def test_three_instances_converge_to_free_fermions(tn):
    ctx = tn.Context(0, precision="split", slices=5)
    insts = [_instance(i) for i in range(3)]
    psis = [T.random_ttn(N, c, 2000 + i) for i, c in enumerate(CHIS)]
    gp = [tn.ttn.TTN(p.adj, p.site_nodes, p.d, p.tensors, p.center, ctx) for p in psis]
    models = [tn.ttn.CouplingModel(t, N) for t, _ in insts]
    batch = tn.ttn.StateEnvsTTN.batch(gp, models)
    path = tn.ttn.default_sweeppath(N)
    sws = [tn.ttn.SweepDataTTN() for _ in range(3)]
    for _ in range(16):
        tn.ttn.fullsweep_batch_(batch, path, tn.eig_solver, sws, maxdim=max(CHIS), outputlevel=0)
        if len(sws[0].energy) >= 2 and all(
                abs(s.energy[-1] - s.energy[-2]) <= 1e-12 * abs(s.energy[-1]) for s in sws):
            break
    for i, (s, (_, exact)) in enumerate(zip(sws, insts)):
        assert s.maxchi[-1] == CHIS[i]
        assert s.energy[-1] >= exact - 1e-12 * abs(exact), i
        assert s.energy[-1] - exact <= 1e-9 * abs(exact), i
