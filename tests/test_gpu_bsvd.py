"""Multi-SM block SVD (blocked Householder QR, cooperative one-sided Jacobi on R^T) against
LAPACK and the CPU oracle, through the C ABI.

Tolerances: singular values within 1e-13 of the block's largest one (LAPACK's own accuracy
is ~1e-16 of the largest value; 2e-13 in split precision, whose Newton-Schulz and R^T V
GEMMs leave V orthogonal to ~1e-13, and 5e-13 for its 2100 x 2048 block, see the tests);
kept dimensions bit-exact against the oracle's ITensors truncation; DMRG energies per sweep
|dE/E| <= 1e-10 with identical bond dimensions and charge sectors when every block above
8 columns takes the multi-SM pipeline.
"""
import json
import os

import numpy as np
import pytest

from oracle import tn_oracle as O

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))


def _graded(rng, r, c, decades=14.0):
    """r x c block with singular values spread over `decades` (DMRG-like grading)."""
    k = min(r, c)
    U, _ = np.linalg.qr(rng.standard_normal((r, k)))
    V, _ = np.linalg.qr(rng.standard_normal((c, k)))
    s = 10.0 ** (-decades * (np.arange(k) / k) ** 0.7) * rng.uniform(0.8, 1.2, size=k)
    return (U * s) @ V.T


def _two_sided(rng, r, c, decades=12.0):
    """Rows and columns scaled by graded weights, as the two-site tensor between Schmidt bases."""
    dl = 10.0 ** (-decades * (np.arange(r) / r) ** 0.8) * rng.uniform(0.7, 1.3, r)
    dr = 10.0 ** (-decades * (np.arange(c) / c) ** 0.8) * rng.uniform(0.7, 1.3, c)
    return dl[:, None] * rng.standard_normal((r, c)) * dr[None, :]


def _check(tn, ctx, blocks, cases, tol=1e-13):
    refs = [np.linalg.svd(b, compute_uv=False) for b in blocks]
    P = np.sort(np.concatenate([r * r for r in refs]))[::-1]
    for maxdim, cutoff in cases:
        kept, sv, err = tn.svd_truncate(blocks, maxdim=maxdim, cutoff=cutoff, ctx=ctx)
        # the oracle's truncation (ITensors truncate! restated) on the LAPACK values
        _, truncerr, docut = O.truncation_rule(P, maxdim, 1, cutoff)
        kept_ref = [int(np.sum(r * r > docut)) for r in refs]
        assert list(kept) == kept_ref, (maxdim, cutoff)
        assert abs(err - truncerr) <= 1e-14 + 1e-10 * truncerr
        for b, s, ref in zip(blocks, sv, refs):
            assert np.all(np.diff(s) <= 0)
            assert np.allclose(s, ref, rtol=0, atol=tol * ref[0]), b.shape


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_big_blocks_match_lapack_and_oracle(tn, prec):
    ctx = tn.Context(0, precision=prec, slices=5)
    rng = np.random.default_rng(31)
    blocks = [_graded(rng, 256, 256), _two_sided(rng, 600, 400), _graded(rng, 420, 610),
              _two_sided(rng, 130, 97), _graded(rng, 40, 30), _graded(rng, 97, 300)]
    # split precision: the Jacobi rotations are refined in double-float, but V is made
    # orthogonal by two Newton-Schulz steps and Y = R^T V is formed by 7-slice tensor-core
    # GEMMs, whose ~1e-13 relative error reaches the column norms (FP64 path: 1e-13)
    _check(tn, ctx, blocks, [(10**6, 1e-12), (500, 1e-10), (60, 1e-15)],
           tol=1e-13 if prec == "fp64" else 2e-13)


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_big_block_2048_columns(tn, prec):
    ctx = tn.Context(0, precision=prec, slices=5)
    rng = np.random.default_rng(32)
    blocks = [_two_sided(rng, 2100, 2048, decades=10.0), _graded(rng, 600, 600)]
    # split precision: the 2100-row block takes 8-column panels, i.e. 256 successive
    # trailing updates, and GEMMs with k ~ 2100 whose tensor-core products are summed in
    # double-float (about 48 bits): 5e-13 of the largest value (FP64 path: 1e-13)
    _check(tn, ctx, blocks, [(10**6, 1e-12), (1024, 1e-10)], tol=1e-13 if prec == "fp64" else 5e-13)


def test_every_block_on_the_multi_sm_path(tn):
    # threshold 0: even 1 x 1 and 2 x 1 blocks take the blocked QR + cooperative Jacobi path
    ctx = tn.Context(0, svd_split=0)
    rng = np.random.default_rng(33)
    blocks = [_graded(rng, 1, 1), _graded(rng, 2, 1), _graded(rng, 3, 7), _graded(rng, 33, 17),
              _two_sided(rng, 65, 64), np.zeros((5, 4))]
    _check(tn, ctx, blocks, [(10**6, 1e-12), (20, 1e-15)])


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_dmrg_sweeps_on_multi_sm_svd_match_oracle(tn, prec):
    # blocks above 8 columns take the multi-SM pipeline: its factors (not only its singular
    # values) enter the state, the environments and the next bond's solve
    N = 14
    ctx = tn.Context(0, precision=prec, slices=5, svd_split=8)
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    eg = tn.StateEnvs(tn.MPS.product(start, pq, ctx), tn.MPO(W, delta, pq, ctx))
    sg = tn.SweepData()
    for md in [8, 16, 32, 48, 64, 64]:
        O.fullsweep(eo, so, md, 1e-12, 1, 4, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-12, solver_krylovdim=4,
                      outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1]), md
        assert sg.maxchi[-1] == so.maxchi[-1], md
    psi = eg.getpsi()
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert abs(sg.energy[-1] - GOLD["heisenberg_chain"][str(N)]) < 1e-8
