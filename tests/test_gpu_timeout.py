"""Failure path of the bounded device waits, made to run out from the host.

tn_ctx_inject_wait_timeout arms a test hook read by the next launch of one kernel: the
split-precision GEMM withholds one stage's bulk copies (its MMA warp's wait runs out and
every role drains before TMEM is released), the cooperative SVD Jacobi and the cooperative
TTN Householder panel lose one CTA before their first barrier (the other CTAs' barrier waits
run out).  Each call must return TN_E_TIMEOUT after about a second, and the next calls on
the same context and on a fresh one must give correct results.  Nothing faults or hangs.
"""
import numpy as np
import pytest

from oracle import tn_oracle as O
from tests.helpers import oracle_envs, random_qn_mps, upload_mpo, upload_mps

pytestmark = pytest.mark.gpu


def _product_setup(tn, ctx, rng):
    N, p = 6, 2
    mps = random_qn_mps(N, rng, maxsec_dim=12)
    H = O.heisenberg_mpo(N)
    env = tn.StateEnvs(upload_mps(tn, ctx, mps, center=p), upload_mpo(tn, ctx, H))
    env.position_(p, 2)
    Lp, Rp = oracle_envs(mps, H, p)
    v = rng.standard_normal((len(mps.links[p]), 2, 2, len(mps.links[p + 2])))
    v *= ((mps.links[p][:, None, None, None] + mps.phys_q[None, :, None, None]
           + mps.phys_q[None, None, :, None]) == mps.links[p + 2][None, None, None, :])
    return env, v, O.heff2_apply(Lp, H.W[p], H.W[p + 1], Rp, v)


def _expect_timeout(tn, fn):
    with pytest.raises(tn._lib.TenNetError) as ei:
        fn()
    assert ei.value.code == tn._lib.TN_E_TIMEOUT


def test_split_gemm_wait_runs_out(tn):
    ctx = tn.Context(0, precision="split", slices=5)
    env, v, ref = _product_setup(tn, ctx, np.random.default_rng(41))
    tn._lib.check(ctx.lib.tn_ctx_inject_wait_timeout(ctx.h, 1))
    _expect_timeout(tn, lambda: env.product(v))
    got = env.product(v)  # same context, next call
    assert np.linalg.norm(got - ref) <= 5e-11 * np.linalg.norm(ref)
    ctx2 = tn.Context(0, precision="split", slices=5)
    env2, v2, ref2 = _product_setup(tn, ctx2, np.random.default_rng(42))
    assert np.linalg.norm(env2.product(v2) - ref2) <= 5e-11 * np.linalg.norm(ref2)


def test_svd_jacobi_barrier_wait_runs_out(tn):
    ctx = tn.Context(0, svd_split=0)
    rng = np.random.default_rng(43)
    blocks = [rng.standard_normal((300, 200)), rng.standard_normal((150, 150))]
    refs = [np.linalg.svd(b, compute_uv=False) for b in blocks]
    tn._lib.check(ctx.lib.tn_ctx_inject_wait_timeout(ctx.h, 2))
    _expect_timeout(tn, lambda: tn.svd_truncate(blocks, cutoff=0.0, ctx=ctx))
    for c in (ctx, tn.Context(0, svd_split=0)):
        _, sv, _ = tn.svd_truncate(blocks, cutoff=0.0, ctx=c)
        for s, r in zip(sv, refs):
            assert np.allclose(s, r, rtol=0, atol=1e-13 * r[0])


def test_ttn_qr_panel_barrier_wait_runs_out(tn):
    ctx = tn.Context(0)
    N, chi, seed = 32, 64, 5   # the top nodes (64, 64, 64) take the cooperative panel path
    graph, sitenodes, tensors, center = tn.ttn.random_ttn_tensors(N, chi, seed)
    psi = tn.ttn.TTN(graph, sitenodes, 2, tensors, None, ctx)
    tn._lib.check(ctx.lib.tn_ctx_inject_wait_timeout(ctx.h, 3))
    _expect_timeout(tn, lambda: psi.isometrize_(center))
    for c in (ctx, tn.Context(0)):
        pg = tn.ttn.TTN(graph, sitenodes, 2, tensors, None, c).isometrize_(center)
        assert np.isclose(np.linalg.norm(pg[center]), 1.0, atol=1e-13)
