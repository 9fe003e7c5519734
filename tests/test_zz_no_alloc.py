"""fvg_spmv_no_alloc — the CRS product for callers that cannot allocate
device memory (plug-ins inside a framework that owns every device
allocation, latency-critical loops that must avoid cudaMalloc's implicit
synchronisation).  Its scratch is a fixed array inside the library, so this
test checks it against the allocating fvg_spmv on a matrix whose long rows
use that scratch, over two calls in a row (the array keeps the previous
call's contents).  Collected last so a failure here leaves the other GPU
tests' results intact; it also passes on its own in a fresh process.

Tolerance: as the other parity tests — FP64 rel 1e-12, FP32/BF16 storage
2e-5 of the row's absolute sum.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _matrix(rng, m=600, n=50000):
    lens = rng.integers(0, 60, m)
    for r, L in ((5, 45000), (77, 20000), (300, 1500)):  # long rows: pieces whose sums go to the scratch
        if r < m:
            lens[r] = min(L, n)
    rows = [np.sort(rng.choice(n, L, replace=False)) for L in lens]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate(rows).astype(np.int32)
    val = rng.standard_normal(int(off[-1]))
    return m, n, off, idx, val


def test_no_alloc_spmv_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    import frovedis_gb300 as fv

    rng = np.random.default_rng(42)
    m, n, off, idx, val = _matrix(rng)
    ctx = fv.Context(0)
    A = ctx.matrix(m, n, off, idx, val)
    A.prepare("CRS", transpose=False)
    A.add_storage("f32")
    A.add_storage("bf16")
    absval = np.abs(val)
    for storage, vec, tol in (("f64", "f64", 1e-12), ("f32", "f32", 2e-5), ("bf16", "f32", 2e-5)):
        tdt = torch.float64 if vec == "f64" else torch.float32
        x = torch.randn(n, dtype=tdt, device="cuda")
        y = torch.empty(m, dtype=tdt, device="cuda")
        xh = x.cpu().numpy()
        ref = A.spmv(xh, storage=storage, vec=vec).astype(np.float64)
        scale = np.zeros(m)
        for r in range(m):
            s, e = off[r], off[r + 1]
            scale[r] = np.sum(absval[s:e] * np.abs(xh[idx[s:e]].astype(np.float64)))
        for call in range(2):
            y.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = ctx.L.fvg_spmv_no_alloc(ctx.h, A.h, fv.DTYPES[storage], fv.DTYPES[vec],
                                         ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()))
            assert rc == 0, ctx.L.fvg_ctx_last_error(ctx.h)
            ctx.synchronize()
            got = y.cpu().numpy().astype(np.float64)
            assert np.all(np.abs(got - ref) <= tol * (scale + 1e-30)), (storage, call)
    A.close()
    ctx.close()


def test_no_alloc_spmv_rejects_unprepared_matrix():
    torch = pytest.importorskip("torch")
    import frovedis_gb300 as fv

    rng = np.random.default_rng(7)
    m, n, off, idx, val = _matrix(rng, m=50, n=1000)
    ctx = fv.Context(0)
    A = ctx.matrix(m, n, off, idx, val)  # no fvg_matrix_prepare: no work schedule yet
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    y = torch.zeros(m, dtype=torch.float64, device="cuda")
    rc = ctx.L.fvg_spmv_no_alloc(ctx.h, A.h, fv.F64, fv.F64, ctypes.c_void_p(x.data_ptr()),
                                 ctypes.c_void_p(y.data_ptr()))
    assert rc == 1 and b"prepare" in ctx.L.fvg_ctx_last_error(ctx.h)
    rc = ctx.L.fvg_spmv_no_alloc(ctx.h, A.h, fv.F64, fv.F32, ctypes.c_void_p(x.data_ptr()),
                                 ctypes.c_void_p(y.data_ptr()))
    assert rc == 1
    A.close()
    ctx.close()
