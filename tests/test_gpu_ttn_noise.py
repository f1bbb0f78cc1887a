"""TTN sweeps with noise > 0 on the GPU: subspace expansion (subspace_expand!,
src/ttn/update_site_ttn.jl:75-109, the noisy branch of src/ttn/sweep_ttn.jl:180-243) and
the optimize! noise schedule (src/ttn/optimize_ttn.jl:148-226), as in the reference's own TTN
test (test/test_TTN.jl:26-48: a chi = 12 random TTN, maxdim 128, cutoff 1e-14, noise 1e-2,
noisedecay 5), against the oracle with the same padding stream.

Tolerances: per sweep energies 1e-10 relative; largest bond dimensions within one (the
expansion puts singular values at the cutoff: a relative perturbation of 1e-12 of the
initial state flips one truncation of the oracle's own first sweep, 37 <-> 38, and the
noise-free sweeps that follow keep the dimensions of the last noisy one, QR moves); the
Heisenberg N = 12 ground energy (dense
diagonalisation) 1e-10 and, with the ground state projected out (weight 10), the second
eigenvalue 1e-8; batched instances equal to the oracle's separate runs (instance i draws
padding stream i)."""
import numpy as np
import pytest

from oracle import ttn_oracle as T

pytestmark = pytest.mark.gpu
N = 12


def upload(tn, ctx, psi):
    return tn.ttn.TTN(psi.adj, psi.site_nodes, psi.d, psi.tensors, psi.center, ctx)


def _setup():
    terms = T.heisenberg_terms(N)
    ev = np.linalg.eigvalsh(T.dense_hamiltonian(N, terms))
    return terms, ev


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_noisy_optimize_matches_oracle_and_exact(tn, precision):
    ctx = tn.Context(0, precision=precision, slices=5)
    terms, ev = _setup()
    path = tn.ttn.default_sweeppath(N)
    psi = T.random_ttn(N, 12, 1)
    kw = dict(cutoff=1e-14, noise=1e-2, noisedecay=5, disable_noise_after=2)
    so = T.optimize(T.StateEnvsTTN(psi, terms), [128], [5], path, seed=7, **kw)
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), tn.ttn.CouplingModel(terms, N))
    params = tn.ttn.OptimizeParamsTTN(maxdim=[128], nsweeps=[5], **kw)
    sg = tn.ttn.optimize_(eg, params, path, seed=7, outputlevel=0)
    assert so.maxchi[0] > 12
    assert all(abs(a - b) <= 1 for a, b in zip(sg.maxchi, so.maxchi))
    for a, b in zip(sg.energy, so.energy):
        assert abs(a - b) <= 1e-10 * abs(b)
    assert abs(sg.energy[-1] - ev[0]) < 1e-10
    # excited state with noise, the reference's second test
    gs = eg.getpsi()
    px = T.random_ttn(N, 12, 2)
    params = tn.ttn.OptimizeParamsTTN(maxdim=[128], nsweeps=[10], cutoff=1e-14, noise=1e-2,
                                      noisedecay=5, disable_noise_after=6)
    e1, _ = tn.ttn.optimize(upload(tn, ctx, px), tn.ttn.CouplingModel(terms, N), [gs], params,
                            path, weight=10.0, seed=8, outputlevel=0)
    assert abs(e1 - ev[1]) < 1e-8


def test_noisy_batched_sweeps_match_oracle(tn, ctx):
    """Two instances (different couplings and initial bond dimensions) swept in lockstep
    with noise; the arena grows once for the widened tensors of both."""
    path = tn.ttn.default_sweeppath(N)
    insts = [T.tfim_terms(*T.tfim_instance(N, 20 + i)) for i in range(2)]
    psis = [T.random_ttn(N, 6 + 4 * i, 3 + i) for i in range(2)]
    kw = dict(maxdim=24, cutoff=1e-12, noise=1e-3)
    refs = []
    for i in range(2):
        se = T.StateEnvsTTN(psis[i], insts[i])
        sw = T.SweepDataTTN()
        for _ in range(3):
            T.fullsweep(se, path, sw, seed=11, instance=i, **kw)
        refs.append(sw)
    batch = tn.ttn.StateEnvsTTN.batch([upload(tn, ctx, p) for p in psis],
                                      [tn.ttn.CouplingModel(t, N) for t in insts])
    sws = [tn.ttn.SweepDataTTN() for _ in range(2)]
    for _ in range(3):
        tn.ttn.fullsweep_batch_(batch, path, tn.eig_solver, sws, seed=11, outputlevel=0, **kw)
    for i in range(2):
        assert all(abs(a - b) <= 1 for a, b in zip(sws[i].maxchi, refs[i].maxchi))
        for a, b in zip(sws[i].energy, refs[i].energy):
            assert abs(a - b) <= 1e-10 * abs(b), i


def test_noisy_sweeps_within_the_creation_slots(tn, ctx):
    """A chi = 32 TTN truncated to maxdim 12 by a noise-free sweep, then noisy sweeps at the
    same maxdim (expand_dim 4): the widened tensors fit the slots laid out at creation, so
    the arena is not re-laid."""
    terms, ev = _setup()
    path = tn.ttn.default_sweeppath(N)
    psi = T.random_ttn(N, 32, 4)
    se = T.StateEnvsTTN(psi, terms)
    so = T.SweepDataTTN()
    eg = tn.ttn.StateEnvsTTN(upload(tn, ctx, psi), tn.ttn.CouplingModel(terms, N))
    sg = tn.ttn.SweepDataTTN()
    kw = dict(maxdim=12, cutoff=1e-12, expand_dim=4)
    for noise in (0.0, 1e-3, 1e-4):
        T.fullsweep(se, path, so, noise=noise, seed=3, **kw)
        tn.ttn.fullsweep_(eg, path, tn.eig_solver, sg, noise=noise, seed=3, outputlevel=0, **kw)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), noise
        assert abs(sg.maxchi[-1] - so.maxchi[-1]) <= 1
    assert sg.maxchi[-1] <= 12
