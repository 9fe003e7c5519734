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

# CUmemPool_attribute values (cuda.h): the default pool's usage counters
_USED_MEM_CURRENT, _USED_MEM_HIGH = 7, 8


class _PoolWatch:
    """The device's default memory pool (where the library's stream-ordered
    allocations come from), read through the CUDA driver API: resetting the
    used-memory high-water mark and reading it back shows whether anything
    was allocated from the pool in between, even if it was freed again."""

    def __init__(self, device=0):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), device) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def _get(self, attr):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = ctypes.c_uint64(0)  # resets the high-water mark to the current usage
        assert self.cu.cuMemPoolSetAttribute(self.pool, _USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def used(self):
        return self._get(_USED_MEM_CURRENT), self._get(_USED_MEM_HIGH)


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
    # the property the entry point exists for: two calls in a row take no
    # memory from the device's pool (not even briefly) and no other device
    # memory (free memory unchanged)
    watch = _PoolWatch(0)
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    y = torch.empty(m, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.synchronize()
    watch.reset_high()
    cur0, _ = watch.used()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        rc = ctx.L.fvg_spmv_no_alloc(ctx.h, A.h, fv.F64, fv.F64, ctypes.c_void_p(x.data_ptr()),
                                     ctypes.c_void_p(y.data_ptr()))
        assert rc == 0, ctx.L.fvg_ctx_last_error(ctx.h)
    ctx.synchronize()
    cur1, high1 = watch.used()
    free1, _ = torch.cuda.mem_get_info()
    assert (cur1, high1) == (cur0, cur0), "the allocation-free entry point allocated from the pool"
    assert free1 == free0, "device memory changed across the allocation-free calls"
    # the allocating entry point does use the pool (the check can see it)
    watch.reset_high()
    A.spmv(x.cpu().numpy())
    ctx.synchronize()
    assert watch.used()[1] > cur0
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
