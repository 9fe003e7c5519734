"""GPU parity of multinomial logistic regression
(multinomial_logistic_regression::train, softmax_parallelizer::do_train)
against the oracle restatement.

FP64: weights and intercepts rel 1e-9 of the largest magnitude (gradient
descent has no line search, so summation-order differences stay at rounding
level), identical iteration counts under the RMS stop test.  FP32/BF16
storage: rel 1e-3 (BF16: 3e-2) of the largest weight.  Probabilities: 1e-12.
"""
import numpy as np
import pytest

import oracle
from test_gpu_parity import rand_crs

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fv.Context(0)
    yield c
    c.close()


def _problem(seed, m=2000, n=300, K=7, lam=12.0):
    from frovedis_gb300 import datagen
    off, idx, val, _ = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed, labels=False))
    a = oracle.CRS(m, n, off, idx, val)
    rng = np.random.default_rng(seed)
    Wt = rng.standard_normal((n, K)) * 0.5
    Z = a.to_dense() @ Wt + 0.5 * rng.standard_normal((m, K))
    return a, np.argmax(Z, 1).astype(np.float64)


def _close(x, ref, rtol):
    x = np.asarray(x)
    ref = np.asarray(ref)
    return np.max(np.abs(x - ref)) <= rtol * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("reg", ["ZERO", "L1", "L2"])
def test_multinomial_matches_oracle(ctx, reg):
    a, label = _problem(51)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=40, alpha=0.2, reg_param=1e-3, reg_type=reg, tol=0.0)
    r = fv.multinomial_train(A, label, 7, **kw)
    ro = oracle.softmax_train(a, label, 7, **kw)
    assert r["n_iter"] == ro["n_iter"] == 40
    assert _close(r["W"], ro["W"], 1e-9)


def test_multinomial_intercept_and_sample_weight(ctx):
    # the reference's intercept step uses the column sums of the gradient
    # matrix (softmax_parallelizer.hpp:165-170); reproduced as is
    a, label = _problem(52, K=5)
    sw = np.random.default_rng(3).uniform(0.5, 2.0, a.m)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=15, alpha=0.05, reg_type="L2", reg_param=1e-2, intercept=True, tol=0.0)
    r = fv.multinomial_train(A, label, 5, sample_weight=sw, **kw)
    ro = oracle.softmax_train(a, label, 5, sw=sw, **kw)
    assert _close(r["W"], ro["W"], 1e-9)
    assert _close(r["b"], ro["b"], 1e-9)


def test_multinomial_stops_on_rms(ctx):
    a, label = _problem(53, K=4)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=500, alpha=0.1, tol=2e-3)
    r = fv.multinomial_train(A, label, 4, **kw)
    ro = oracle.softmax_train(a, label, 4, **kw)
    assert 1 < ro["n_iter"] < 500
    assert r["n_iter"] == ro["n_iter"]
    assert _close(r["W"], ro["W"], 1e-9)


@pytest.mark.parametrize("K", [1, 33, 128, 150])
def test_multinomial_class_counts(ctx, K):
    a, label = _problem(54, m=800, n=120, K=K)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=8, alpha=0.3, tol=0.0, intercept=(K == 150))
    r = fv.multinomial_train(A, label, K, **kw)
    ro = oracle.softmax_train(a, label, K, **kw)
    assert _close(r["W"], ro["W"], 1e-9), K
    assert _close(r["b"], ro["b"], 1e-9), K


def test_multinomial_long_rows(ctx):
    rng = np.random.default_rng(55)
    a = rand_crs(rng, 300, 3000, maxlen=40, long_rows=[(5, 2900), (100, 1500), (101, 700)])
    label = rng.integers(0, 9, a.m).astype(np.float64)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=6, alpha=0.05, tol=0.0)
    r = fv.multinomial_train(A, label, 9, **kw)
    ro = oracle.softmax_train(a, label, 9, **kw)
    assert _close(r["W"], ro["W"], 1e-9)


def test_multinomial_probability(ctx):
    a, label = _problem(56, K=6)
    rng = np.random.default_rng(5)
    W = rng.standard_normal((a.n, 6))
    b = rng.standard_normal(6)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for icpt in (False, True):
        P = fv.multinomial_probability(A, W, b, intercept=icpt)
        Po = oracle.softmax_probability(a, W, b, intercept=icpt)
        assert np.max(np.abs(P - Po)) <= 1e-12
    W2 = rng.standard_normal((a.n, 140))
    P = fv.multinomial_probability(A, W2, np.zeros(140))
    assert np.max(np.abs(P - oracle.softmax_probability(a, W2, np.zeros(140)))) <= 1e-12


@pytest.mark.parametrize("storage,rtol", [("f32", 1e-3), ("bf16", 3e-2)])
def test_multinomial_reduced_precision(ctx, storage, rtol):
    a, label = _problem(57)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=30, alpha=0.2, reg_type="L2", reg_param=1e-3, tol=0.0)
    r = fv.multinomial_train(A, label, 7, storage=storage, **kw)
    ro = oracle.softmax_train(a, label, 7, **kw)
    assert _close(r["W"], ro["W"], rtol)
    acc = np.mean(np.argmax(oracle.softmax_probability(a, r["W"], r["b"]), 1) == label)
    acc_o = np.mean(np.argmax(oracle.softmax_probability(a, ro["W"], ro["b"]), 1) == label)
    assert abs(acc - acc_o) <= 0.01


def test_multinomial_errors(ctx):
    a, label = _problem(58, m=200, n=30, K=3)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for fmt in ("JDS", "ELL"):  # softmax_parallelizer.hpp:340
        with pytest.raises(fv.FvgError, match="Unsupported input matrix type"):
            fv.multinomial_train(A, label, 3, mat_type=fmt)
    r = fv.multinomial_train(A, label, 3, mat_type="HYBRID", num_iter=3, tol=0.0)
    ro = oracle.softmax_train(a, label, 3, num_iter=3, tol=0.0)
    assert _close(r["W"], ro["W"], 1e-9)
    with pytest.raises(fv.FvgError):
        fv.multinomial_train(A, label, 0)
    with pytest.raises(fv.FvgError):
        fv.multinomial_train(A, label, 3, alpha=0.0)


# ------------------------------------------------ multinomial by L-BFGS
def _mlr_data(m=3000, n=200, K=5, seed=3):
    from frovedis_gb300 import datagen
    off, idx, val, _ = datagen.generate(datagen.Spec(m=m, n=n, lam=15.0, seed=seed, labels=False))
    a = oracle.CRS(m, n, off, idx, val)
    rng = np.random.default_rng(seed)
    Z = oracle.spmm(a, rng.standard_normal((n, K)) * 0.3)
    label = np.argmax(Z + rng.gumbel(size=Z.shape), axis=1).astype(np.float64)
    return a, label


@pytest.mark.parametrize("K,reg", [(5, "L2"), (5, "ZERO"), (37, "L1"), (128, "L2")])
def test_multinomial_lbfgs_matches_oracle(ctx, K, reg):
    # the reference's softmax gradient with the L-BFGS driver, FP64: the same
    # line-search decisions, loss within 1e-6, weights within 1e-5
    a, label = _mlr_data(m=2500, n=150, K=K, seed=K)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=25, reg_type=reg, reg_param=1e-4)
    r = fv.multinomial_lbfgs(A, label, K, trace=True, **kw)
    ro = oracle.softmax_lbfgs(a, label, K, **kw)
    assert r["n_iter"] == ro["n_iter"]
    assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1]), "line-search trial counts differ"
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["W"] - ro["W"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["W"])))


def test_multinomial_lbfgs_sample_weights_and_start(ctx):
    a, label = _mlr_data(m=2000, n=120, K=7, seed=11)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    rng = np.random.default_rng(2)
    sw = rng.uniform(0.5, 2.0, a.m)
    W0 = rng.standard_normal((a.n, 7)) * 0.05
    kw = dict(num_iter=15, reg_type="L2", reg_param=1e-3)
    r = fv.multinomial_lbfgs(A, label, 7, sample_weight=sw, W0=W0, **kw)
    ro = oracle.softmax_lbfgs(a, label, 7, sw=sw, W0=W0, **kw)
    assert r["n_iter"] == ro["n_iter"]
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["W"] - ro["W"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["W"])))


def test_multinomial_lbfgs_reduced_precision_and_errors(ctx):
    # FP32 / BF16 values (FP32 accumulation): the loss within 1e-3 of the
    # FP64 oracle on the same rounded values; unsupported settings rejected
    a, label = _mlr_data(m=3000, n=200, K=10, seed=5)
    vb = (fv.bf16_bits(a.val).astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    ab = oracle.CRS(a.m, a.n, a.off, a.idx, vb)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, vb)
    kw = dict(num_iter=15, reg_type="L2", reg_param=1e-4)
    ro = oracle.softmax_lbfgs(ab, label, 10, **kw)
    for storage in ("f32", "bf16"):
        r = fv.multinomial_lbfgs(A, label, 10, storage=storage, **kw)
        assert abs(r["loss"] - ro["loss"]) <= 1e-3 * abs(ro["loss"]), storage
    with pytest.raises(fv.FvgError):
        fv.multinomial_lbfgs(A, label, 10, intercept=True, **kw)
    with pytest.raises(fv.FvgError):
        fv.multinomial_lbfgs(A, label, 200, **kw)
