"""Split storage (FP32 values + BF16 residuals, double-FP32 arithmetic)
against the FP64 oracle on the original FP64 values.

The stored value hi + lo is within 2^-33 (1.2e-10) of the FP64 value and the
arithmetic carries about 48 bits, so a single product or evaluation agrees
with the FP64 oracle to ~1e-10 of the sum of magnitudes, and trained models
meet the path's FP64 bar: relative error <= 1e-6 on the final loss and
<= 1e-5 on the weights, with the same line-search decisions.
"""
import numpy as np
import pytest

import oracle

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu

# products / evaluations: relative to the sum of |a_ij x_j| of the row
SPLIT_RTOL = 1e-9


@pytest.fixture(scope="module")
def ctx():
    c = fv.Context(0)
    yield c
    c.close()


def _lr_data(seed=0, m=4000, n=300, lam=15.0, val_kind="absnormal"):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed, val_kind=val_kind))
    return oracle.CRS(m, n, off, idx, val), label


def _rand_crs(rng, m, n, maxlen=40, long_rows=(), empty_every=13):
    lens = np.minimum(rng.integers(0, maxlen + 1, m), n)
    lens[::empty_every] = 0
    for r, L in long_rows:
        lens[r] = min(L, n)
    rows = [np.sort(rng.choice(n, lens[r], replace=False)) for r in range(m)]
    off = np.concatenate([[0], np.cumsum([len(x) for x in rows])]).astype(np.int32)
    idx = np.concatenate(rows).astype(np.int32) if off[-1] else np.zeros(0, np.int32)
    val = rng.standard_normal(int(off[-1])) * np.exp(rng.uniform(-3, 3, int(off[-1])))
    return oracle.CRS(m, n, off, idx, val)


def _abs_rowsum(a, x):
    return oracle.spmv(oracle.CRS(a.m, a.n, a.off, a.idx, np.abs(a.val)), np.abs(x))


@pytest.mark.parametrize("shape", [(500, 300), (3000, 2000), (64, 20000)])
def test_split_spmv_and_trans_mv(ctx, shape):
    m, n = shape
    rng = np.random.default_rng(m + n)
    # long rows (pieces summed by the finalize kernel) and empty rows
    a = _rand_crs(rng, m, n, long_rows=[(1, 5000), (m // 2, 1200)])
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    x = rng.standard_normal(n) * np.exp(rng.uniform(-2, 2, n))
    y = A.spmv(x, storage="split")
    yo = oracle.spmv(a, x)
    assert np.all(np.abs(y - yo) <= SPLIT_RTOL * _abs_rowsum(a, x) + 1e-300)
    r = rng.standard_normal(m)
    z = A.trans_mv(r, storage="split")
    at = oracle.transpose(a)
    zo = oracle.spmv(at, r)
    assert np.all(np.abs(z - zo) <= SPLIT_RTOL * _abs_rowsum(at, r) + 1e-300)
    # run-to-run identical
    assert np.array_equal(A.spmv(x, storage="split"), y)
    assert np.array_equal(A.trans_mv(r, storage="split"), z)


def test_split_tutorial_golden(ctx):
    from _golden import crs, golden
    g = golden()["tut_spmv"]
    a = crs(g)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    assert np.array_equal(A.spmv(np.ones(a.n), storage="split"), np.array(g["expected_y_ones"]))


def test_split_is_closer_than_fp32(ctx):
    # values with full 53-bit mantissas: FP32 storage is off by ~1e-7 of the
    # row sum, split storage by at most its representation error (2^-33 per
    # value, 1.2e-10) plus the df64 arithmetic's ~1e-14
    rng = np.random.default_rng(5)
    a = _rand_crs(rng, 2000, 1500)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    x = rng.standard_normal(a.n)
    yo = oracle.spmv(a, x)
    scale = _abs_rowsum(a, x) + 1e-300
    e_split = np.max(np.abs(A.spmv(x, storage="split") - yo) / scale)
    e_f32 = np.max(np.abs(A.spmv(x.astype(np.float32), storage="f32", vec="f32") - yo) / scale)
    assert e_split <= 2.0 ** -33 + 1e-13 and e_split * 100 < e_f32, (e_split, e_f32)


@pytest.mark.parametrize("loss", [None, "linear", "hinge", "eps", "sqeps"])
def test_split_eval_matches_fp64_oracle(ctx, loss):
    a, label = _lr_data(1, val_kind="lognormal")
    rng = np.random.default_rng(2)
    sw = rng.uniform(0.5, 2.0, a.m)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    colscale = oracle.spmv(oracle.transpose(oracle.CRS(a.m, a.n, a.off, a.idx, np.abs(a.val))), sw)
    for icpt in (False, True):
        w = rng.standard_normal(a.n) * 0.3
        kw = dict(b=0.7, intercept=icpt, sample_weight=sw)
        ko = dict(b=0.7, intercept=icpt, sw=sw)
        if loss is not None:
            kw.update(loss=loss, epsilon=0.25)
            ko.update(loss=loss, eps=0.25)
        g, lv = fv.logreg_eval(A, label, w, storage="split", **kw)
        go, lo = oracle.logreg_eval(a, label, w, **ko)
        assert abs(lv - lo) <= 1e-10 * abs(lo) + 1e-12, (loss, icpt, lv, lo)
        dmax = 1.0 if loss in (None, "hinge", "eps") else 2.0 * (np.max(np.abs(a.to_dense() @ w)) + 3.0)
        assert np.all(np.abs(g[:-1] - go[:-1]) <= 1e-9 * colscale * dmax + 1e-12), (loss, icpt)
        assert abs(g[-1] - go[-1]) <= 1e-9 * np.sum(sw) * dmax, (loss, icpt)


def test_split_eval_extreme_margins(ctx):
    # the z > 18 / z < -18 branches and everything between (gradient.hpp:29-48)
    a, label = _lr_data(3, m=2000, n=50)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for scale in (0.0, 0.05, 3.0, 40.0):
        w = np.full(a.n, scale)
        g, loss = fv.logreg_eval(A, label, w, b=-scale, intercept=True, storage="split")
        go, losso = oracle.logreg_eval(a, label, w, b=-scale, intercept=True)
        assert abs(loss - losso) <= 1e-10 * abs(losso) + 1e-300, scale
        assert np.max(np.abs(g - go) / (np.abs(go) + 1.0)) <= 1e-9, scale


@pytest.mark.parametrize("reg", ["L2", "ZERO", "L1"])
def test_split_lbfgs_matches_fp64_oracle(ctx, reg):
    a, label = _lr_data(4, val_kind="lognormal")
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=20, reg_type=reg, reg_param=1e-3, intercept=True)
    r = fv.logreg_lbfgs(A, label, trace=True, storage="split", **kw)
    ro = oracle.logreg_lbfgs(a, label, **kw)
    assert r["n_iter"] == ro["n_iter"]
    assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1]), "line-search trial counts differ"
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    assert abs(r["b"] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"]))


def test_split_lbfgs_100k_20k_configuration(ctx):
    # 100,000 x 20,000, nnz/row 1+Poisson(39), Zipf(1.1), |N(0,1)|, L2 1e-3,
    # 20 iterations from zero weights: the FP64 bar against the FP64 oracle
    from frovedis_gb300 import datagen
    spec = datagen.logreg_100k_20k()
    off, idx, val, label = datagen.generate(spec)
    a = oracle.CRS(spec.m, spec.n, off, idx, val)
    A = ctx.matrix(spec.m, spec.n, off, idx, val)
    kz = dict(num_iter=20, reg_type="L2", reg_param=1e-3, w0=np.zeros(spec.n))
    r = fv.logreg_lbfgs(A, label, trace=True, storage="split", **kz)
    ro = oracle.logreg_lbfgs(a, label, nthreads=8, **kz)
    assert r["n_iter"] == ro["n_iter"] == 20
    assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1])
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))


def test_split_glm_lbfgs(ctx):
    # ridge regression (squared loss, L2) and linear SVM (hinge) on split values
    a, label = _lr_data(9, m=3000, n=200, val_kind="lognormal")
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for loss in ("linear", "hinge"):
        kw = dict(num_iter=15, reg_type="L2", reg_param=1e-3, w0=np.zeros(a.n))
        r = fv.glm_lbfgs(A, label, loss=loss, storage="split", trace=True, **kw)
        ro = oracle.logreg_lbfgs(a, label, loss=loss, **kw)
        assert r["n_iter"] == ro["n_iter"], loss
        assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1]), loss
        assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"]), loss
        assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"]))), loss


def test_split_deterministic_and_errors(ctx):
    a, label = _lr_data(11, m=3000, n=500)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=8, reg_type="L2", reg_param=1e-3, storage="split")
    r1 = fv.logreg_lbfgs(A, label, **kw)
    r2 = fv.logreg_lbfgs(A, label, **kw)
    assert r1["loss"] == r2["loss"] and np.array_equal(r1["w"], r2["w"])
    with pytest.raises(fv.FvgError):  # CRS only
        fv.logreg_lbfgs(A, label, mat_type="ELL", **kw)
    with pytest.raises(fv.FvgError):  # the SGD trainers keep FP64/FP32/BF16
        fv.logreg_sgd(A, label, num_iter=2, storage="split")
    with pytest.raises(fv.FvgError):  # FP64 vectors only
        A.spmv(np.ones(a.n, np.float32), storage="split", vec="f32")
    with pytest.raises(fv.FvgError):
        A.spmv(np.ones(a.n), fmt="JDS", storage="split")


def test_split_rejects_values_beyond_fp32(ctx):
    off = np.array([0, 2, 3], np.int32)
    idx = np.array([0, 1, 1], np.int32)
    A = ctx.matrix(2, 2, off, idx, np.array([1.0, 1e300, 2.0]))
    with pytest.raises(fv.FvgError):
        A.spmv(np.ones(2), storage="split")


def _zipf(m, n, lam=30.0, seed=3, val_kind="lognormal"):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed, val_kind=val_kind))
    return oracle.CRS(m, n, off, idx, val), label


@pytest.mark.parametrize("rows,mpp", [(512, 1.0), (1000, 2.0), (4, 0.5), (8192, 1.0)])
def test_split_panel_trans_mv(ctx, rows, mpp):
    # the row-panel layout on split values: hot columns from the panels,
    # the rest from the cold transposed CRS; FP64 oracle on the FP64 values
    a, _ = _zipf(12000, 900, seed=rows)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.set_panels(rows, mpp)
    rng = np.random.default_rng(rows)
    r = rng.standard_normal(a.m)
    z = A.trans_mv(r, storage="split")
    assert A.panel_info()[2] > 0
    at = oracle.transpose(a)
    zo = oracle.spmv(at, r)
    assert np.all(np.abs(z - zo) <= SPLIT_RTOL * _abs_rowsum(at, r) + 1e-300)
    assert np.array_equal(A.trans_mv(r, storage="split"), z)


def test_split_panel_long_segments(ctx):
    # a column with more entries in one panel than a work item holds (its
    # pieces are added after the CTA barrier) and rows of one entry
    rng = np.random.default_rng(17)
    m, n = 20000, 300
    rows = [np.sort(rng.choice(n, rng.integers(0, 6), replace=False)) for _ in range(m)]
    for i in range(0, m, 3):  # column 7 in every third row: ~6,700 entries
        if 7 not in rows[i]:
            rows[i] = np.sort(np.append(rows[i], 7))
    off = np.concatenate([[0], np.cumsum([len(x) for x in rows])]).astype(np.int32)
    idx = np.concatenate(rows).astype(np.int32)
    val = rng.standard_normal(int(off[-1])) * np.exp(rng.uniform(-2, 2, int(off[-1])))
    a = oracle.CRS(m, n, off, idx, val)
    A = ctx.matrix(m, n, off, idx, val)
    A.set_panels(8000, 1.0)  # within the tallest panel a CTA can stage
    r = rng.standard_normal(m)
    z = A.trans_mv(r, storage="split")
    at = oracle.transpose(a)
    assert np.all(np.abs(z - oracle.spmv(at, r)) <= SPLIT_RTOL * _abs_rowsum(at, r) + 1e-300)


@pytest.mark.parametrize("head,panels", [(64, 0), (700, 512), (1500, 0), (0, 256)])
def test_split_head_and_panels_eval(ctx, head, panels):
    # evaluation with the forward head and/or the row panels forced on
    a, label = _zipf(9000, 1600, seed=head + panels)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.set_head(head)
    A.set_panels(panels, 1.0)
    rng = np.random.default_rng(4)
    w = rng.standard_normal(a.n) * 0.2
    sw = rng.uniform(0.5, 2.0, a.m)
    g, loss = fv.logreg_eval(A, label, w, b=0.4, intercept=True, sample_weight=sw, storage="split")
    assert A.head_info()[0] == head and (A.panel_info()[2] > 0) == (panels > 0)
    go, lo = oracle.logreg_eval(a, label, w, b=0.4, intercept=True, sw=sw)
    colscale = oracle.spmv(oracle.transpose(oracle.CRS(a.m, a.n, a.off, a.idx, np.abs(a.val))), sw)
    assert abs(loss - lo) <= 1e-10 * abs(lo)
    assert np.all(np.abs(g[:-1] - go[:-1]) <= 1e-9 * colscale + 1e-12)
    assert abs(g[-1] - go[-1]) <= 1e-9 * np.sum(sw)
    g2, loss2 = fv.logreg_eval(A, label, w, b=0.4, intercept=True, sample_weight=sw, storage="split")
    assert loss2 == loss and np.array_equal(g2, g)


def test_split_head_and_panels_lbfgs(ctx):
    # training with both layouts on: the FP64 bar and the same decisions
    a, label = _zipf(20000, 3000, seed=31)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.set_head(1024)
    A.set_panels(2048, 1.0)
    kw = dict(num_iter=20, reg_type="L2", reg_param=1e-3, w0=np.zeros(a.n))
    r = fv.logreg_lbfgs(A, label, trace=True, storage="split", **kw)
    ro = oracle.logreg_lbfgs(a, label, **kw)
    assert r["n_iter"] == ro["n_iter"]
    assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1])
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
