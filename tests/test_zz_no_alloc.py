"""The allocation-free entry point tn_block_svals_noalloc (runs last on purpose).

It is meant for callers that cannot let the library allocate device memory: their
inputs and outputs already live on the device, and the library works in a fixed
file-scope device array.  The test calls it through the C ABI on device buffers and
compares with tn_svd_truncate (which copies host data and allocates its own work space)
and with LAPACK, on two consecutive calls with different blocks, so that a stale work
array would show.  The second list holds a 300 x 200 block behind a small one: its
Jacobi matrices do not fit shared memory and live at a nonzero offset of the array.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _blocks(rng, shapes):
    out = []
    for (r, c) in shapes:
        U, _ = np.linalg.qr(rng.standard_normal((r, r)))
        V, _ = np.linalg.qr(rng.standard_normal((c, c)))
        k = min(r, c)
        s = np.exp(-np.linspace(0, 20, k)) * rng.uniform(0.5, 1.5, size=k)
        out.append((U[:, :k] * s) @ V[:k, :])
    return out


def _noalloc(tn, torch, blocks):
    lib = tn._lib.load()
    rows = np.array([b.shape[0] for b in blocks], dtype=np.int32)
    cols = np.array([b.shape[1] for b in blocks], dtype=np.int32)
    flat = np.concatenate([b.ravel(order="F") for b in blocks])
    d_in = torch.from_numpy(flat).to("cuda:0")
    nsv = int(np.minimum(rows, cols).sum())
    d_out = torch.full((nsv,), float("nan"), dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream(0)
    dev_before = torch.cuda.current_device()
    rc = lib.tn_block_svals_noalloc(0, C.c_void_p(d_in.data_ptr()), len(blocks),
                                    rows.ctypes.data_as(tn._lib.i32p),
                                    cols.ctypes.data_as(tn._lib.i32p),
                                    C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.tn_last_error()
    assert torch.cuda.current_device() == dev_before
    stream.synchronize()
    sv = d_out.cpu().numpy()
    out, o = [], 0
    for r, c in zip(rows, cols):
        k = min(r, c)
        out.append(sv[o:o + k])
        o += k
    return out


def test_noalloc_matches_allocating_entry_point(tn):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = tn.Context(0)
    rng = np.random.default_rng(2024)
    for shapes in ([(40, 40), (12, 70), (90, 30), (1, 1), (7, 3)],
                   [(64, 64), (33, 50), (300, 200), (5, 9)]):
        blocks = _blocks(rng, shapes)
        got = _noalloc(tn, torch, blocks)
        _, ref, _ = tn.svd_truncate(blocks, maxdim=10**6, cutoff=0.0, ctx=ctx)
        for b, g, r in zip(blocks, got, ref):
            # same tolerance as the block SVD parity tests: 1e-13 of the largest value
            assert np.allclose(g, r, rtol=0, atol=1e-13 * r[0])
            lap = np.linalg.svd(b, compute_uv=False)
            assert np.allclose(g, lap, rtol=0, atol=1e-13 * lap[0])


def test_noalloc_rejects_oversize(tn):
    lib = tn._lib.load()
    rows = np.array([1000, 1000], dtype=np.int32)
    cols = np.array([600, 600], dtype=np.int32)   # 1.2e6 elements > 524288
    rc = lib.tn_block_svals_noalloc(0, C.c_void_p(1), 2, rows.ctypes.data_as(tn._lib.i32p),
                                    cols.ctypes.data_as(tn._lib.i32p), C.c_void_p(1), None)
    assert rc == tn._lib.TN_E_INVALID
    assert b"524288" in lib.tn_last_error()
