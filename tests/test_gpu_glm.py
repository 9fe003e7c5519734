"""GPU parity of the GLM family on the shared device path: linear / ridge /
lasso regression (linear_gradient), linear SVM (hinge_gradient) and SVM
regression (epsilon_insensitive, squared_epsilon_insensitive) against the
oracle restatement (ml/glm/gradient.hpp, lbfgs_parallelizer.hpp,
sgd_parallelizer.hpp) and the reference's test/ml fixtures.

Tolerances as for logistic regression: one FP64 evaluation rel 1e-12 on
the loss and 1e-11 on the gradient; trained models rel 1e-6 on the final
loss and 1e-5 on the weights, identical iteration and line-search trial
counts.  FP32/BF16 storage: loss rel 1e-5 of the FP64 evaluation on the same
(representable) values."""
import numpy as np
import pytest

import oracle
from _golden import crs, golden
from test_gpu_parity import FMTS, close

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu

LOSSES = ["linear", "hinge", "eps", "sqeps"]
EPS = {"linear": 0.0, "hinge": 0.0, "eps": 0.1, "sqeps": 0.05}


@pytest.fixture(scope="module")
def ctx():
    c = fv.Context(0)
    yield c
    c.close()


def _data(seed, m=4000, n=300, lam=15.0):
    """A sparse problem with +-1 labels (SVM) and real targets y = 0.25 A x
    + 0.5 label (regression)."""
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed))
    a = oracle.CRS(m, n, off, idx, val)
    x = np.random.default_rng(seed + 100).standard_normal(n)
    y = 0.25 * oracle.spmv(a, x) + 0.5 * label
    return a, label, y


def _target(loss, label, y):
    return label if loss == "hinge" else y


@pytest.mark.parametrize("loss", LOSSES)
@pytest.mark.parametrize("fmt", FMTS)
def test_glm_eval_matches_oracle(ctx, loss, fmt):
    a, label, y = _data(1)
    t = _target(loss, label, y)
    rng = np.random.default_rng(2)
    sw = rng.uniform(0.5, 2.0, a.m)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for icpt in (False, True):
        w = rng.standard_normal(a.n) * 0.3
        g, lo = fv.glm_eval(A, t, w, b=0.7, intercept=icpt, sample_weight=sw, fmt=fmt, loss=loss, epsilon=EPS[loss])
        go, loo = oracle.logreg_eval(a, t, w, b=0.7, intercept=icpt, sw=sw, fmt=fmt, loss=loss, eps=EPS[loss])
        assert abs(lo - loo) <= 1e-12 * abs(loo), (loss, fmt, icpt)
        assert close(g, go, 1e-11), (loss, fmt, icpt)


def test_glm_eval_clip_and_thresholds(ctx):
    # MAX_LOSS clip of the squared losses (gradient.hpp:81-83, 195-197) and
    # rows sitting exactly on the hinge / epsilon thresholds
    m, n = 6, 1
    off = np.arange(m + 1, dtype=np.int32)
    idx = np.zeros(m, np.int32)
    val = np.ones(m)
    a = oracle.CRS(m, n, off, idx, val)
    A = ctx.matrix(m, n, off, idx, val)
    lab = np.array([1.0, -1.0, 0.5, -2e12, 3e12, 1.1])
    for loss, w in (("linear", 1.0), ("hinge", 1.0), ("eps", 0.6), ("sqeps", 0.4), ("sqeps", 1e12)):
        g, lo = fv.glm_eval(A, lab, np.array([w]), loss=loss, epsilon=0.5)
        go, loo = oracle.logreg_eval(a, lab, np.array([w]), loss=loss, eps=0.5)
        # the gradient sums +-1e12 terms that cancel: bound by the terms' size
        d, _ = oracle.glm_dloss(lab, np.full(m, w), loss, 0.5)
        assert np.max(np.abs(g - go)) <= 1e-15 * (np.sum(np.abs(d)) + 1.0), loss
        assert abs(lo - loo) <= 1e-13 * abs(loo), loss


@pytest.mark.parametrize("loss", LOSSES)
def test_glm_eval_reduced_precision(ctx, loss):
    from frovedis_gb300 import datagen
    n = 2000
    off, idx, val, label = datagen.generate(datagen.Spec(m=6000, n=n, lam=30.0, seed=8))
    val = (fv.bf16_bits(val).astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    a = oracle.CRS(6000, n, off, idx, val)
    y = 0.25 * oracle.spmv(a, np.random.default_rng(3).standard_normal(n)) + 0.5 * label
    t = _target(loss, label, y)
    A = ctx.matrix(6000, n, off, idx, val)
    w = np.random.default_rng(9).standard_normal(n) * 0.2
    g64, l64 = fv.glm_eval(A, t, w, b=0.3, intercept=True, loss=loss, epsilon=EPS[loss])
    plain = {}
    for storage in ("f32", "bf16"):
        g, lo = fv.glm_eval(A, t, w, b=0.3, intercept=True, storage=storage, loss=loss, epsilon=EPS[loss])
        assert abs(lo - l64) <= 1e-5 * abs(l64), (loss, storage)
        plain[storage] = g
    # the same through the forward head and the row-panel backward product
    # (forced on this small matrix): the loss kind rides in the tail pass's
    # epilogue
    A.set_panels(512, 1.0)
    A.set_head(300)
    for storage in ("f32", "bf16"):
        g, lo = fv.glm_eval(A, t, w, b=0.3, intercept=True, storage=storage, loss=loss, epsilon=EPS[loss])
        assert abs(lo - l64) <= 1e-5 * abs(l64), (loss, storage, "head/panels")
        gp = plain[storage]
        assert np.max(np.abs(g - gp)) <= 1e-4 * max(1.0, np.max(np.abs(gp))), (loss, storage, "head/panels")
    assert A.head_info()[0] == 300 and A.panel_info()[2] > 0


@pytest.mark.parametrize("loss,reg,fmt", [("linear", "ZERO", "CRS"), ("linear", "L1", "CRS"), ("linear", "L2", "CRS"),
                                          ("linear", "L2", "ELL"), ("linear", "ZERO", "HYBRID"),
                                          ("hinge", "L2", "CRS"), ("hinge", "L1", "HYBRID"), ("hinge", "L2", "ELL")])
def test_glm_lbfgs_matches_oracle(ctx, loss, reg, fmt):
    a, label, y = _data(4)
    t = _target(loss, label, y)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    r = fv.glm_lbfgs(A, t, loss=loss, num_iter=20, reg_type=reg, reg_param=1e-3, intercept=True, mat_type=fmt,
                     trace=True)
    ro = oracle.logreg_lbfgs(a, t, loss=loss, num_iter=20, reg_type=reg, reg_param=1e-3, intercept=True, fmt=fmt)
    assert r["n_iter"] == ro["n_iter"]
    assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1]), "line-search trial counts differ"
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    assert abs(r["b"] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"]))


SGD_ALPHA = {"linear": 1e-4, "hinge": 0.05, "eps": 0.01, "sqeps": 1e-4}


@pytest.mark.parametrize("loss", LOSSES)
@pytest.mark.parametrize("fmt", FMTS)
def test_glm_sgd_matches_oracle(ctx, loss, fmt):
    # minibatch fraction 0.3: two minibatches of 1024-row multiples, so the
    # squared loss's running halving (gradient.hpp:70-73) is exercised
    a, label, y = _data(5, m=5000, n=200)
    t = _target(loss, label, y)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=15, alpha=SGD_ALPHA[loss], mini_batch_fraction=0.3, reg_type="L2", reg_param=1e-2,
              intercept=True)
    r = fv.glm_sgd(A, t, loss=loss, epsilon=EPS[loss], mat_type=fmt, **kw)
    ro = oracle.logreg_sgd(a, t, loss=loss, eps=EPS[loss], fmt=fmt, **kw)
    assert r["n_iter"] == ro["n_iter"]
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    assert abs(r["b"] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"]))


def test_glm_sgd_ranks_with_empty_rank(ctx):
    # per-rank running loss summed in rank order; rank 2 holds no rows
    a, label, y = _data(6, m=3000, n=100)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    splits = [0, 700, 1500, 1500, 3000]
    kw = dict(num_iter=10, alpha=1e-4, mini_batch_fraction=0.5, reg_type="ZERO", intercept=True)
    r = fv.glm_sgd(A, y, loss="linear", row_splits=splits, **kw)
    ro = oracle.logreg_sgd(a, y, loss="linear", splits=splits, **kw)
    assert abs(r["loss"] - ro["loss"]) <= 1e-9 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))


@pytest.mark.parametrize("loss", ["linear", "hinge"])
def test_glm_batched_matches_single_runs(ctx, loss):
    a, label, y = _data(7, m=3000, n=200)
    t = _target(loss, label, y)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    lams = np.array([1e-4, 1e-3, 1e-2])
    rb = fv.glm_lbfgs_batched(A, t, lams, loss=loss, num_iter=15, reg_type="L2", intercept=True)
    for j, lam in enumerate(lams):
        ro = oracle.logreg_lbfgs(a, t, loss=loss, num_iter=15, reg_type="L2", reg_param=lam, intercept=True)
        assert rb["n_iter"][j] == ro["n_iter"], j
        assert abs(rb["loss"][j] - ro["loss"]) <= 1e-6 * abs(ro["loss"]), j
        assert np.max(np.abs(rb["w"][j] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"]))), j


@pytest.mark.parametrize("storage", ["f32", "bf16"])
def test_glm_lbfgs_reduced_precision(ctx, storage):
    a, label, y = _data(8, m=6000, n=400)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    ro = oracle.logreg_lbfgs(a, y, loss="linear", num_iter=30, reg_type="L2", reg_param=1e-3)
    r = fv.glm_lbfgs(A, y, loss="linear", num_iter=30, reg_type="L2", reg_param=1e-3, storage=storage)
    assert abs(r["loss"] - ro["loss"]) <= 1e-3 * abs(ro["loss"]), storage


def _fixture(name):
    e = golden()[name]
    return e, crs(e), np.array(e["label"])


@pytest.mark.parametrize("name", ["test1.1-1", "test1.2-1", "test1.3-1"])
def test_regression_sgd_golden(ctx, name):
    # test/ml/test1.{1,2,3}-1: stored predictions reproduced to their six
    # digits with the earlier initial model (weights 0, intercept 1) and L2
    # without USE_ETA, as the oracle pins them
    e, a, label = _fixture(name)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    r = fv.glm_sgd(A, label, loss="linear", num_iter=int(e["num_iteration"]), alpha=e["alpha"],
                   mini_batch_fraction=e["minibatch_fraction"], reg_param=e.get("regParam", 0.0),
                   reg_type=e["reg_type"], intercept=e["intercept"], w0=np.zeros(a.n), b0=1.0, l2_no_eta=1)
    assert r["n_iter"] == 3
    pred = A.spmv(r["w"]) + r["b"]
    assert np.max(np.abs(pred - e["expected_out"])) <= 5e-6


@pytest.mark.parametrize("name", ["test2.2-1", "test2.2-2"])
def test_svm_golden_predictions(ctx, name):
    e, a, label = _fixture(name)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(loss="hinge", num_iter=int(e["num_iteration"]), alpha=e["alpha"], reg_param=e["regParam"],
              reg_type=e["reg_type"], intercept=e["intercept"])
    if e["solver"] == "sgd":
        r = fv.glm_sgd(A, label, mini_batch_fraction=e["minibatch_fraction"], **kw)
    else:
        r = fv.glm_lbfgs(A, label, hist_size=int(e["hist_size"]), **kw)
    pred = np.where(A.spmv(r["w"]) + r["b"] > 0, 1.0, -1.0)
    assert np.array_equal(pred, e["expected_out_p"])


def test_glm_errors_and_logistic_entry_points(ctx):
    a, label, y = _data(9, m=500, n=40)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    with pytest.raises(fv.FvgError, match="Unsupported loss kind"):
        fv.glm_lbfgs(A, y, loss=7, num_iter=3)
    with pytest.raises(fv.FvgError, match="Unsupported input matrix type"):
        fv.glm_lbfgs(A, label, loss="hinge", num_iter=3, mat_type="JDS")
    # the fvg_logreg_* entry points train logistic regression whatever loss says
    r1 = fv.logreg_lbfgs(A, label, num_iter=5)
    r2 = fv.logreg_lbfgs(A, label, num_iter=5, loss="hinge")
    assert np.array_equal(r1["w"], r2["w"])
    r3 = fv.glm_lbfgs(A, label, loss="logistic", num_iter=5)
    assert np.array_equal(r1["w"], r3["w"])


# ------------------------------------------------------------- shrink SGD
def _shrunk_problem():
    """Columns 260.. unused by every rank; column 255 used only by the last
    rank's rows (splits 0 / 1000 / 2500 / 4000)."""
    a, label, _ = _data(10, m=4000, n=300)
    rows = np.repeat(np.arange(a.m), np.diff(a.off))
    keep = (a.idx < 260) & ~((a.idx == 255) & (rows < 2500))
    off = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=a.m))]).astype(np.int32)
    return oracle.CRS(a.m, a.n, off, a.idx[keep], a.val[keep]), label


@pytest.mark.parametrize("fmt", FMTS)
@pytest.mark.parametrize("reg", ["L1", "L2"])
def test_shrink_sgd_matches_oracle(ctx, fmt, reg):
    a, label = _shrunk_problem()
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    splits = [0, 1000, 2500, 4000]
    kw = dict(num_iter=20, alpha=0.05, mini_batch_fraction=0.4, reg_type=reg, reg_param=1e-2, intercept=True)
    r = fv.logreg_shrink_sgd(A, label, mat_type=fmt, row_splits=splits, **kw)
    ro = oracle.logreg_sgd(a, label, shrink=True, fmt=fmt, splits=splits, **kw)
    # ELL: the no-trans driver reports numIteration + 1 (shrink_sgd_parallelizer.hpp:315)
    assert r["n_iter"] == ro["n_iter"] == (21 if fmt == "ELL" else 20)
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    assert abs(r["b"] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"]))
    assert np.all(r["w"][260:] == 0.0) and r["w"][255] != 0.0


def test_shrink_sgd_stop_test(ctx):
    # RMS of the summed change before regularisation + rank 0's intercept
    # change over rank 0's column count + 1: stops earlier than plain SGD here
    a, label, _ = _data(10, m=4000, n=300)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    splits = [0, 1000, 2500, 4000]
    kw = dict(num_iter=50, alpha=3e-5, reg_type="L2", reg_param=1e-2, intercept=True, tol=1e-3)
    r = fv.logreg_shrink_sgd(A, label, row_splits=splits, **kw)
    ro = oracle.logreg_sgd(a, label, shrink=True, splits=splits, **kw)
    assert r["n_iter"] == ro["n_iter"] < 50
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
