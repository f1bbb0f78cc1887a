"""Tuned block-SVD schedule (the split of a bond's charge blocks between the one-CTA kernel
and the multi-SM pipeline, keyed on the bond's block-size histogram).

Every candidate threshold of a key is timed once on the first bonds with that key, then the
fastest is kept; whatever the schedule, the singular values stay within 1e-13 of the
largest (LAPACK) and the kept dimensions equal those of a fixed schedule."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _blocks(rng, shapes):
    out = []
    for r, c in shapes:
        k = min(r, c)
        U, _ = np.linalg.qr(rng.standard_normal((r, k)))
        V, _ = np.linalg.qr(rng.standard_normal((c, k)))
        s = 10.0 ** (-10 * (np.arange(k) / k) ** 0.7)
        out.append((U * s) @ V.T)
    return out


def test_schedule_times_each_candidate_then_keeps_the_fastest(tn):
    ctx = tn.Context(0)  # default: tuned
    fixed = tn.Context(0, svd_split=96)
    rng = np.random.default_rng(3)
    # largest block 120 columns: bucket 4 (97..128), candidates one-CTA / 64 / 96
    blocks = _blocks(rng, [(150, 120), (100, 90), (60, 50), (20, 12)])
    refs = [np.linalg.svd(b, compute_uv=False) for b in blocks]
    kept_fixed, _, _ = tn.svd_truncate(blocks, cutoff=1e-12, ctx=fixed)
    for call in range(5):
        kept, sv, _ = tn.svd_truncate(blocks, cutoff=1e-12, ctx=ctx)
        assert list(kept) == list(kept_fixed), call
        for s, ref in zip(sv, refs):
            assert np.allclose(s, ref, rtol=0, atol=1e-13 * ref[0]), call
    sched = {e["bucket"]: e for e in ctx.svd_schedule()}
    e = sched[4]
    assert e["candidates"] == [None, 64, 96]
    assert e["settled"] and e["timed"] == 3
    assert all(m > 0 for m in e["ms"])
    best = int(np.argmin(e["ms"]))
    assert e["chosen"] == e["candidates"][best]
    # a bond whose largest block is below 64 columns has a single candidate
    tn.svd_truncate(_blocks(rng, [(40, 30), (30, 20)]), cutoff=1e-12, ctx=ctx)
    sched = {e["bucket"]: e for e in ctx.svd_schedule()}
    assert sched[1]["candidates"] == [None] and sched[1]["settled"]
    # a fixed threshold leaves the table alone
    assert fixed.svd_schedule() == []


def test_large_bond_candidates_exclude_one_cta(tn):
    ctx = tn.Context(0)
    rng = np.random.default_rng(4)
    blocks = _blocks(rng, [(320, 300), (140, 130), (70, 66)])
    refs = [np.linalg.svd(b, compute_uv=False) for b in blocks]
    for _ in range(4):
        kept, sv, _ = tn.svd_truncate(blocks, cutoff=1e-12, ctx=ctx)
        for s, ref in zip(sv, refs):
            assert np.allclose(s, ref, rtol=0, atol=1e-13 * ref[0])
    e = {x["bucket"]: x for x in ctx.svd_schedule()}[10]
    assert e["candidates"] == [64, 96, 128, 176]
    assert e["settled"]
