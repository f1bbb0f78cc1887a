"""Two-site TDVP (tdvpsweep!, real time step = imaginary-time evolution) against the oracle.

Tolerances: energies per sweep |dE/E| <= 1e-10, bond dimensions and charge sectors
bit-exact, imaginary-time ground energy against exact diagonalisation.
"""
import json
import os

import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import upload_mpo

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))


def _run_both(tn, ctx, N, tau, maxdims, cutoff, krylovdim=30):
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    eng = tn.TDVPEngine(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), ctx),
                        upload_mpo(tn, ctx, H))
    for md in maxdims:
        O.tdvp_sweep(eo, so, tau, md, cutoff, 1, krylovdim, 100, 1e-12)
        tn.tdvpsweep_(eng, tau, maxdim=md, cutoff=cutoff, solver_krylovdim=krylovdim)
        yield so, eng, eo


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_tdvp_sweeps_match_oracle(tn, precision):
    ctx = tn.Context(0, precision=precision, slices=5)
    for so, eng, eo in _run_both(tn, ctx, 12, -0.1, [8, 16, 16, 32, 32], 1e-12):
        e_o, e_g = so.energy[-1], eng.getenergy()
        assert abs(e_g - e_o) <= 1e-10 * abs(e_o)
        assert eng.maxchi() == so.maxchi[-1]
        assert abs(eng.getentropy() - so.entropy[-1]) < 1e-9
    psi = eng.getpsi()
    for i in range(len(eo.psi.links)):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert eng.abstime == pytest.approx(0.5)
    assert eng.sweepcount() == 5


def test_tdvp_imaginary_time_reaches_ground_state(tn):
    ctx = tn.Context(0)
    N = 10
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    eng = tn.TDVPEngine(tn.MPS.product(tn.models.neel_states(N), pq, ctx),
                        tn.MPO(W, delta, pq, ctx))
    for _ in range(40):
        tn.tdvpsweep_(eng, -1.0, maxdim=32, cutoff=1e-14)
    assert abs(eng.getenergy() - GOLD["heisenberg_chain"]["10"]) < 1e-8
    assert eng.totalerror() >= 0.0


def test_tdvp_mode_errors(tn):
    """nsite outside {1, 2, "dynamic"} and extendat with a fixed nsite are errors, as in
    tdvp.jl:262-274; a first dynamic sweep of a single MPO would open with global subspace
    expansion, which is not built, and raises NotImplementedError without touching the state."""
    ctx = tn.Context(0)
    N = 6
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    eng = tn.TDVPEngine(tn.MPS.product(tn.models.neel_states(N), pq, ctx),
                        tn.MPO(W, delta, pq, ctx))
    with pytest.raises(NotImplementedError, match="krylov_extend"):
        tn.tdvpsweep_(eng, -0.05, nsite="dynamic", maxdim=8)
    with pytest.raises(ValueError, match="nsite"):
        tn.tdvpsweep_(eng, -0.05, nsite=3, maxdim=8)
    with pytest.raises(ValueError, match="extendat"):
        tn.tdvpsweep_(eng, -0.05, nsite=2, maxdim=8, extendat=2)
    assert eng.sweepcount() == 0
    tn.tdvpsweep_(eng, -0.05, maxdim=8)
    with pytest.raises(NotImplementedError, match="krylov_extend"):  # (1 + 1) % 2 == 0
        tn.tdvpsweep_(eng, -0.05, nsite="dynamic", maxdim=8, extendat=2)
    tn.tdvpsweep_(eng, -0.05, nsite="dynamic", maxdim=8)
    assert eng.sweepcount() == 2
