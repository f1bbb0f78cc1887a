"""GPU against the CPU oracle at the benchmark's scale: the open S=1/2 Heisenberg chain with
N = 100, U(1) S^z = 0, cutoff 1e-12 (the bond dimension settles near 180 in the bulk).

The engine prepares the state (Neel start, maxdim 64, 128, 256, 256: one sweep each); the
state is copied to the oracle, and both then run the same bond updates from bond 1 to the
middle of the chain (left-to-right, eig_solver defaults krylovdim 5 / maxiter 2).  Per
update: energies |dE/E| <= 1e-10, kept bond dimensions and the kept S^2 spectra (1e-9 FP64,
1e-8 split precision, whose products carry 5e-11 relative errors); at the end
the charge sectors of every link bit-exact.  Charge blocks of up to ~110 columns occur: the
FP64 case fixes the SVD threshold at 96 columns, so both the one-CTA and the multi-SM block
SVD take part; the split case runs the tuned schedule (every candidate is timed on the first
bonds, so both paths take part there too)."""
import numpy as np
import pytest

from oracle import tn_oracle as O

pytestmark = pytest.mark.gpu

N = 100
CUTOFF = 1e-12


@pytest.mark.parametrize("prec,svd_split", [("fp64", 96), ("split", -1)])
def test_heisenberg_chain_N100_bond_updates_match_oracle(tn, prec, svd_split):
    ctx = tn.Context(0, precision=prec, slices=5, svd_split=svd_split)
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    env = tn.StateEnvs(tn.MPS.product(tn.models.neel_states(N), pq, ctx), H)
    sw = tn.SweepData()
    for md in (64, 128, 256, 256):
        tn.fullsweep_(env, tn.eig_solver, 2, sw, maxdim=md, cutoff=CUTOFF, outputlevel=0)
    assert sw.maxchi[-1] > 150
    psi = env.getpsi()
    tensors = [psi.site(i) for i in range(N)]
    links = [psi.link_charges(i) for i in range(N + 1)]
    oe = O.StateEnvs(O.MPS([np.asarray(t) for t in tensors],
                           [np.asarray(q, dtype=np.int64) for q in links],
                           O.SPIN_HALF_Q.copy(), center=0), O.heisenberg_mpo(N))
    ge = tn.StateEnvs(tn.MPS(tensors, links, pq, 0, ctx), H)
    big = 0
    for b in range(N // 2 + 2):
        e_g, err_g, eigs_g = tn.update_position_(ge, tn.eig_solver, b, 2, "left", maxdim=1024,
                                                 cutoff=CUTOFF)
        e_o, spec, _ = O.update_two_site(oe, b, "left", 1024, 1, CUTOFF, 5, 2, 1e-14)
        assert abs(e_g - e_o) <= 1e-10 * abs(e_o), b
        assert len(eigs_g) == len(spec.eigs), b
        # S^2 of the normalised state to 1e-9: the solve stops after two restarts of a
        # 5-vector Krylov space, so its Ritz vector (unlike its Ritz value, checked above at
        # 1e-10) carries the rounding differences of the two implementations amplified by the
        # small spectral gap of the long chain
        assert np.allclose(eigs_g, spec.eigs, rtol=0, atol=1e-9 if prec == "fp64" else 1e-8), b
        assert abs(err_g - spec.truncerr) <= 1e-14 + 1e-8 * spec.truncerr, b
        big = max(big, len(eigs_g))
    assert big > 150
    gp = ge.getpsi()
    for i in range(N + 1):
        assert np.array_equal(gp.link_charges(i), oe.psi.links[i]), i
