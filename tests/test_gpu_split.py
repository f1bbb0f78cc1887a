"""Split-precision path (bf16 slices on tcgen05 tensor cores) against the CPU oracle.

Tolerances: products and environments relative 5e-11 (Frobenius) at 5 slices (41 bits
per operand element, two chained contractions); DMRG energies |dE/E| <= 1e-10 (the
accuracy bound of the sweep); bond dimensions and charge sectors bit-exact.
"""
import json
import os

import numpy as np
import pytest

from oracle import ed
from oracle import tn_oracle as O
from tests.helpers import oracle_envs, random_qn_mps, upload_mpo, upload_mps

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ed_energies.json")))


@pytest.fixture(scope="module")
def sctx(tn):
    return tn.Context(0, precision="split", slices=5)


def _mask2(ql, pq, qr):
    return (ql[:, None, None, None] + pq[None, :, None, None] + pq[None, None, :, None]) == \
        qr[None, None, None, :]


def _product_case(tn, ctx, mps, H, p, rng):
    env = tn.StateEnvs(upload_mps(tn, ctx, mps, center=p), upload_mpo(tn, ctx, H))
    env.position_(p, 2)
    Lp, Rp = oracle_envs(mps, H, p)
    v = rng.standard_normal((len(mps.links[p]), 2, 2, len(mps.links[p + 2])))
    v *= _mask2(mps.links[p], mps.phys_q, mps.links[p + 2])
    ref = O.heff2_apply(Lp, H.W[p], H.W[p + 1], Rp, v)
    return env.product(v), ref


@pytest.mark.parametrize("qn", [True, False])
def test_split_product_small_blocks(tn, sctx, qn):
    rng = np.random.default_rng(7 + qn)
    N = 8
    mps = random_qn_mps(N, rng, maxsec_dim=3, qn=qn)
    H = O.heisenberg_mpo(N, qn=qn)
    for p in (0, 3, 6):
        got, ref = _product_case(tn, sctx, mps, H, p, rng)
        assert np.linalg.norm(got - ref) <= 5e-11 * np.linalg.norm(ref), p


def test_split_product_large_blocks(tn, sctx):
    # sector dimensions up to 60: several row tiles (128), column tiles (64), k tiles (64)
    # and accumulation chunks (128) per task
    rng = np.random.default_rng(11)
    N = 6
    mps = random_qn_mps(N, rng, maxsec_dim=60)
    H = O.mpo_from_terms(N, ed.heisenberg_chain_terms(N))
    got, ref = _product_case(tn, sctx, mps, H, 2, rng)
    assert np.linalg.norm(got - ref) <= 5e-11 * np.linalg.norm(ref)
    # elementwise: error bounded by the row/column scales, not only in norm
    assert np.max(np.abs(got - ref)) <= 5e-11 * np.max(np.abs(ref))


def test_split_product_no_qn_wide(tn, sctx):
    rng = np.random.default_rng(12)
    N = 6
    mps = random_qn_mps(N, rng, maxsec_dim=70, qn=False)
    H = O.heisenberg_mpo(N, qn=False)
    got, ref = _product_case(tn, sctx, mps, H, 2, rng)
    assert np.linalg.norm(got - ref) <= 5e-11 * np.linalg.norm(ref)


def test_split_accuracy_improves_with_slices(tn):
    rng = np.random.default_rng(13)
    N = 6
    mps = random_qn_mps(N, rng, maxsec_dim=20)
    H = O.heisenberg_mpo(N)
    errs = []
    for s in (4, 5, 6):
        ctx = tn.Context(0, precision="split", slices=s)
        got, ref = _product_case(tn, ctx, mps, H, 2, np.random.default_rng(99))
        errs.append(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    assert errs[0] < 1e-8 and errs[1] < 5e-11 and errs[2] < 5e-13, errs
    assert errs[2] < errs[1] < errs[0]


def test_split_environments(tn, sctx):
    rng = np.random.default_rng(21)
    N, p = 10, 5
    mps = random_qn_mps(N, rng, maxsec_dim=8)
    H = O.mpo_from_terms(N, ed.heisenberg_chain_terms(N))
    env = tn.StateEnvs(upload_mps(tn, sctx, mps, center=p), upload_mpo(tn, sctx, H))
    env.position_(p, 2)
    eo = O.StateEnvs(mps, H)
    eo.position(p, 2)
    for i in range(1, p + 1):
        ref = eo.L[i]
        assert np.linalg.norm(env.environment("left", i) - ref) <= 5e-11 * np.linalg.norm(ref), i
    for i in range(p + 1, N - 1):
        ref = eo.R[i]
        assert np.linalg.norm(env.environment("right", i) - ref) <= 5e-11 * np.linalg.norm(ref), i


def test_split_dmrg_matches_oracle(tn, sctx):
    N = 16
    H = O.heisenberg_mpo(N)
    start = [0 if i % 2 == 0 else 1 for i in range(N)]
    eo = O.StateEnvs(O.product_mps(start, O.SPIN_HALF_Q), H)
    so = O.SweepData()
    eg = tn.StateEnvs(tn.MPS.product(start, np.array([1, -1], dtype=np.int32), sctx),
                      upload_mpo(tn, sctx, H))
    sg = tn.SweepData()
    for md in [8, 16, 32, 48, 64, 64]:
        O.fullsweep(eo, so, md, 1e-12, 1, 4, 2, 1e-14)
        tn.fullsweep_(eg, tn.eig_solver, 2, sg, maxdim=md, cutoff=1e-12, solver_krylovdim=4,
                      outputlevel=0)
        assert abs(sg.energy[-1] - so.energy[-1]) <= 1e-10 * abs(so.energy[-1])
        assert sg.maxchi[-1] == so.maxchi[-1]
    psi = eg.getpsi()
    for i in range(N + 1):
        assert np.array_equal(psi.link_charges(i), eo.psi.links[i]), i
    assert abs(sg.energy[-1] - GOLD["heisenberg_chain"]["16"]) < 1e-8
