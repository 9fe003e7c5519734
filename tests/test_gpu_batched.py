"""GPU parity of the multi-vector products and of batched L-BFGS training.

SpMM (operator*(crs_matrix_local, rowmajor_matrix_local), crs_matrix.hpp:
2053-2064) against the oracle: FP64 rel 1e-12, FP32/BF16 values rel 2e-5 of
the row's absolute sum.  Batched L-BFGS: every model against its own oracle
logistic_regression_with_lbfgs::train run (FP64): identical iteration count,
final loss rel 1e-6, weights rel 1e-5.
"""
import numpy as np
import pytest

import oracle
from test_gpu_parity import close, rand_crs

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fv.Context(0)
    yield c
    c.close()


def _lr(seed, m=3000, n=200, lam=12.0):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed))
    return oracle.CRS(m, n, off, idx, val), label


def test_spmm_long_rows_many_columns(ctx):
    rng = np.random.default_rng(21)
    a = rand_crs(rng, 300, 40000, maxlen=70, long_rows=[(3, 39000), (150, 20000), (151, 16385)])
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.add_storage("f32")
    A.add_storage("bf16")
    for k in (1, 3, 33, 64, 130):
        X = rng.standard_normal((a.n, k))
        ref = oracle.spmm(a, X)
        assert close(A.spmm(X), ref, 1e-12), k
        absref = oracle.spmm(oracle.CRS(a.m, a.n, a.off, a.idx, np.abs(a.val)), np.abs(X))
        y32 = A.spmm(X.astype(np.float32), storage="f32", vec="f32")
        assert np.max(np.abs(y32 - ref) / (absref + 1e-30)) <= 2e-5, k
        vb = fv.bf16_bits(a.val).astype(np.uint32) << 16
        ab = oracle.CRS(a.m, a.n, a.off, a.idx, vb.view(np.float32).astype(np.float64))
        yb = A.spmm(X.astype(np.float32), storage="bf16", vec="f32")
        assert np.max(np.abs(yb - oracle.spmm(ab, X.astype(np.float32))) / (absref + 1e-30)) <= 2e-5, k


def test_spmm_empty_rows_and_matrix(ctx):
    rng = np.random.default_rng(22)
    z = oracle.CRS(40, 10, np.zeros(41, np.int32), np.zeros(0, np.int32), np.zeros(0))
    Z = ctx.matrix(z.m, z.n, z.off, z.idx, z.val)
    assert np.array_equal(Z.spmm(rng.standard_normal((10, 7))), np.zeros((40, 7)))
    a = rand_crs(rng, 500, 60, empty_every=3)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    X = rng.standard_normal((a.n, 64))
    assert close(A.spmm(X), oracle.spmm(a, X), 1e-12)


def _check_models(r, a, label, lams, **kw):
    for j, lam in enumerate(lams):
        ro = oracle.logreg_lbfgs(a, label, reg_param=lam, **kw)
        assert r["n_iter"][j] == ro["n_iter"], (j, lam)
        assert abs(r["loss"][j] - ro["loss"]) <= 1e-6 * abs(ro["loss"]), (j, lam)
        assert np.max(np.abs(r["w"][j] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"]))), (j, lam)
        assert abs(r["b"][j] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"])), (j, lam)


@pytest.mark.parametrize("reg", ["L2", "L1", "ZERO"])
def test_batched_lbfgs_matches_separate_runs(ctx, reg):
    a, label = _lr(31)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    lams = [0.0, 1e-4, 1e-3, 1e-2, 0.1, 0.5]
    kw = dict(num_iter=20, reg_type=reg, intercept=True)
    r = fv.logreg_lbfgs_batched(A, label, lams, **kw)
    _check_models(r, a, label, lams, **kw)


def test_batched_lbfgs_models_stop_on_their_own(ctx):
    # a loose tolerance: models converge at different iterations
    a, label = _lr(32, m=2000, n=80)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    lams = list(np.logspace(-4, 0, 9))
    kw = dict(num_iter=60, reg_type="L2", intercept=True, tol=0.05)
    r = fv.logreg_lbfgs_batched(A, label, lams, **kw)
    assert len(set(r["n_iter"].tolist())) > 1, r["n_iter"]
    _check_models(r, a, label, lams, **kw)


def test_batched_lbfgs_sample_weight_and_initial_models(ctx):
    a, label = _lr(33, m=1500, n=120)
    rng = np.random.default_rng(4)
    sw = rng.uniform(0.5, 2.0, a.m)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    lams = [1e-3, 1e-2, 3e-2]
    w0 = rng.standard_normal((3, a.n)) * 0.1
    b0 = np.array([0.0, 0.5, -0.5])
    r = fv.logreg_lbfgs_batched(A, label, lams, sample_weight=sw, w0=w0, b0=b0, num_iter=15, reg_type="L2",
                                intercept=True)
    for j, lam in enumerate(lams):
        ro = oracle.logreg_lbfgs(a, label, num_iter=15, reg_type="L2", reg_param=lam, intercept=True, sw=sw,
                                 w0=w0[j], b0=b0[j])
        assert r["n_iter"][j] == ro["n_iter"]
        assert abs(r["loss"][j] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
        assert np.max(np.abs(r["w"][j] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))


def test_batched_lbfgs_64_models(ctx):
    a, label = _lr(34, m=2500, n=150)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    lams = np.logspace(-6, 0, 64)
    r = fv.logreg_lbfgs_batched(A, label, lams, num_iter=10, reg_type="L2", intercept=True, w0=np.zeros(a.n))
    for j in (0, 17, 40, 63):
        ro = oracle.logreg_lbfgs(a, label, num_iter=10, reg_type="L2", reg_param=lams[j], intercept=True,
                                 w0=np.zeros(a.n))
        assert r["n_iter"][j] == ro["n_iter"]
        assert abs(r["loss"][j] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
        assert np.max(np.abs(r["w"][j] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))


def test_batched_lbfgs_one_model_equals_single_driver(ctx):
    a, label = _lr(35)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=20, reg_type="L2", intercept=True)
    rb = fv.logreg_lbfgs_batched(A, label, [1e-3], **kw)
    rs = fv.logreg_lbfgs(A, label, reg_param=1e-3, **kw)
    assert rb["n_iter"][0] == rs["n_iter"]
    assert abs(rb["loss"][0] - rs["loss"]) <= 1e-9 * abs(rs["loss"])
    assert np.max(np.abs(rb["w"][0] - rs["w"])) <= 1e-7 * max(1.0, np.max(np.abs(rs["w"])))


def test_batched_lbfgs_reduced_precision(ctx):
    a, label = _lr(36)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    lams = [1e-4, 1e-2]
    kw = dict(num_iter=20, reg_type="L2", intercept=True, w0=np.zeros(a.n))
    for storage in ("f32", "bf16"):
        r = fv.logreg_lbfgs_batched(A, label, lams, storage=storage, **kw)
        for j, lam in enumerate(lams):
            rs = fv.logreg_lbfgs(A, label, reg_param=lam, storage=storage, **kw)
            ro = oracle.logreg_lbfgs(a, label, reg_param=lam, **kw)
            assert abs(r["loss"][j] - ro["loss"]) <= 1e-3 * abs(ro["loss"]), (storage, j)
            if storage == "f32":  # the batch and the single driver share the FP32 arithmetic
                assert abs(r["loss"][j] - rs["loss"]) <= 1e-4 * abs(rs["loss"]), j


def test_batched_lbfgs_errors(ctx):
    a, label = _lr(37, m=200, n=30)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_batched(A, label, [1e-3, 1e-2], mat_type="HYBRID")
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_batched(A, label, [])
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_batched(A, label, [1e-3, -1.0])
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_batched(A, label, np.full(257, 1e-3))
