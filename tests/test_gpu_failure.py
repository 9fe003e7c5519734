"""Failure detection without faulting the GPU.

The reference reports failures through exceptions on the host
(core/exceptions.hpp:22-43) and MPI error handlers (core/mpi_rpc.cc:471-491).
Here the device side never traps: every wait inside a kernel (the L-BFGS
direction's grid barriers, the row-panel kernels' bulk-copy waits) has a poll
budget, after which the kernel records the failure in the context's error
word and finishes; the call then returns FVG_ERR_INTERNAL and the context
stays usable.  These tests make the waits run out (a budget of 0 polls gives
up on any wait that is not already complete), inject allocation failures on
the host, and feed NaN inputs — then check the status and that the next
call on the same context gives the right answer.
"""
import ctypes

import numpy as np
import pytest

import oracle

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu

FVG_ERR_OUT_OF_MEMORY, FVG_ERR_INTERNAL = 5, 6


def _lr_data(seed=0, m=3000, n=2000, lam=15.0):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed))
    return oracle.CRS(m, n, off, idx, val), label


def test_grid_barrier_budget_runs_out_and_context_recovers():
    a, label = _lr_data(1)
    ctx = fv.Context(0)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=5, reg_type="L2", reg_param=1e-3)
    good = fv.logreg_lbfgs(A, label, **kw)
    # n + 1 = 2001 model entries: the direction kernel runs on several CTAs,
    # so with no polls allowed every CTA but the last to arrive gives up
    ctx.set_wait_limit(0)
    with pytest.raises(fv.FvgError) as e:
        fv.logreg_lbfgs(A, label, **kw)
    assert e.value.code == FVG_ERR_INTERNAL and "grid barrier" in str(e.value)
    ctx.set_wait_limit(-1)
    again = fv.logreg_lbfgs(A, label, **kw)
    assert again["loss"] == good["loss"] and np.array_equal(again["w"], good["w"])
    ro = oracle.logreg_lbfgs(a, label, **kw)
    assert abs(again["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    A.close()
    ctx.close()


def test_bulk_copy_budget_runs_out_and_context_recovers():
    a, label = _lr_data(2, m=6000, n=400)
    ctx = fv.Context(0)
    v32 = a.val.astype(np.float32).astype(np.float64)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, v32)
    A.set_panels(256, 1.0)  # row panels and the forward head forced on: their kernels stage by bulk copies
    A.set_head(64)
    w = np.random.default_rng(3).standard_normal(a.n) * 0.2
    g0, l0 = fv.logreg_eval(A, label, w, b=0.3, intercept=True, storage="f32")
    assert A.panel_info()[2] > 0 and A.head_info()[0] == 64
    ctx.set_wait_limit(0)
    with pytest.raises(fv.FvgError) as e:
        fv.logreg_eval(A, label, w, b=0.3, intercept=True, storage="f32")
    assert e.value.code == FVG_ERR_INTERNAL and "bulk copy" in str(e.value)
    ctx.set_wait_limit(-1)
    g1, l1 = fv.logreg_eval(A, label, w, b=0.3, intercept=True, storage="f32")
    assert l1 == l0 and np.array_equal(g1, g0)
    A.close()
    ctx.close()


def _pool_used():
    cu = ctypes.CDLL("libcuda.so.1")
    dev = ctypes.c_int()
    assert cu.cuDeviceGet(ctypes.byref(dev), 0) == 0
    pool = ctypes.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    v = ctypes.c_uint64()
    assert cu.cuMemPoolGetAttribute(pool, 7, ctypes.byref(v)) == 0  # CU_MEMPOOL_ATTR_USED_MEM_CURRENT
    return v.value


@pytest.mark.parametrize("after", [0, 3, 12])
def test_injected_allocation_failure(after):
    a, label = _lr_data(4, m=2000, n=300)
    ctx = fv.Context(0)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.prepare("CRS", transpose=True)
    kw = dict(num_iter=6, reg_type="L2", reg_param=1e-3)
    good = fv.logreg_lbfgs(A, label, **kw)
    ctx.synchronize()
    used0 = _pool_used()
    fv.load().fvg_debug_inject_alloc_failure(after)
    try:
        with pytest.raises(fv.FvgError) as e:
            fv.logreg_lbfgs(A, label, **kw)
    finally:
        fv.load().fvg_debug_inject_alloc_failure(-1)
    assert e.value.code == FVG_ERR_OUT_OF_MEMORY
    ctx.synchronize()
    assert _pool_used() == used0, "the failed call left device memory allocated"
    again = fv.logreg_lbfgs(A, label, **kw)
    assert again["loss"] == good["loss"] and np.array_equal(again["w"], good["w"])
    A.close()
    ctx.close()


def test_nan_inputs_propagate_like_the_reference():
    # the reference checks neither values nor labels for NaN: the loss and
    # gradient become NaN and training runs on; here the same, without a
    # hang or a fault, and the context serves the next call
    a, label = _lr_data(5, m=1500, n=200)
    ctx = fv.Context(0)
    val = a.val.copy()
    val[7] = np.nan
    B = ctx.matrix(a.m, a.n, a.off, a.idx, val)
    w = np.full(a.n, 0.1)
    g, loss = fv.logreg_eval(B, label, w)
    go, losso = oracle.logreg_eval(oracle.CRS(a.m, a.n, a.off, a.idx, val), label, w)
    assert np.isnan(loss) and np.isnan(losso)
    assert np.array_equal(np.isnan(g), np.isnan(go))
    lab = label.copy()
    lab[3] = np.nan
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    r = fv.logreg_lbfgs(A, lab, num_iter=3, reg_type="L2", reg_param=1e-3)
    assert np.isnan(r["loss"])
    ok = fv.logreg_lbfgs(A, label, num_iter=3, reg_type="L2", reg_param=1e-3)
    ro = oracle.logreg_lbfgs(a, label, num_iter=3, reg_type="L2", reg_param=1e-3)
    assert abs(ok["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    A.close()
    B.close()
    ctx.close()
