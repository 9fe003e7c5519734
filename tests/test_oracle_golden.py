"""Pins the CPU oracle to the reference's own fixtures and stored outputs
(tests/golden/golden.json, extracted by tests/golden/make_golden.py)."""
import numpy as np
import pytest

import oracle
from _golden import crs, crs_text, golden


def test_tutorial_spmv_all_formats():
    # doc/tutorial/tutorial.md:1348-1355 (tut3.2.1-1); tut3.2.2 runs the same
    # product through ELL / JDS / hybrid.
    g = golden()["tut_spmv"]
    a = crs(g)
    x = np.ones(a.n)
    exp = np.array(g["expected_y_ones"])
    assert np.array_equal(oracle.spmv(a, x), exp)
    assert np.array_equal(oracle.ell_spmv(a, x), exp)
    assert np.array_equal(oracle.jds_spmv(a, x), exp)
    for thr in (0, 1, 2, 3, 256):
        assert np.array_equal(oracle.hyb_spmv(a, x, thr), exp), thr


def test_tutorial_transpose():
    # doc/tutorial/tutorial.md:1413-1420 (tut3.2.1-2, binary CRS fixture)
    g = golden()["tut_binary"]
    t = oracle.transpose(crs(g))
    assert crs_text(t) == g["expected_transpose_text"]


def _glm(name):
    e = golden()[name]
    a = crs(e)
    label = np.array(e["label"])
    splits = oracle.text_rank_splits(bytes.fromhex(e["data_bytes_hex"]), golden()["glm_test_ranks"])
    return e, a, label, splits


def test_text_loader_rank_split():
    # 4 ranks over the 48-byte fixture: rows {0}, {1,2}, {3}, {} (core/dvector.cc:198-300)
    _, _, _, splits = _glm("test2.1-2")
    assert splits == [0, 1, 3, 4, 4]


@pytest.mark.parametrize("ranks", [1, 4])
def test_lbfgs_golden(ranks):
    # test/ml/test2.1-2/test.cc: predictions {1,-1,1,1}, probabilities {1,0,1,1}, RMS < 0.01
    e, a, label, splits = _glm("test2.1-2")
    r = oracle.logreg_lbfgs(a, label, num_iter=int(e["num_iteration"]), alpha=e["alpha"],
                            hist_size=int(e["hist_size"]), reg_param=e["regParam"], reg_type=e["reg_type"],
                            intercept=e["intercept"], splits=splits if ranks == 4 else None)
    pb = oracle.predict_probability(a, r["w"], r["b"])
    pred = np.where(pb >= 0.5, 1.0, -1.0)
    assert np.sqrt(np.mean((pred - e["expected_out_p"]) ** 2)) < e["rms_tol"]
    assert np.sqrt(np.mean((pb - e["expected_out_pb"]) ** 2)) < e["rms_tol"]


@pytest.mark.parametrize("ranks", [1, 4])
def test_sgd_golden(ranks):
    # test/ml/test2.1-1/test.cc stores probabilities {0.952718, 0.437991,
    # 0.958198, 0.955715}.  They are reproduced to all six printed digits with
    # an earlier source's initial model (weights 0, intercept 1) and the L2
    # branch built without USE_ETA (regularizer.hpp:50-54); the current
    # source's defaults (weights 1, intercept 0, eta = alpha/sqrt(i)) give
    # other values, checked against labels only.
    e, a, label, splits = _glm("test2.1-1")
    kw = dict(num_iter=int(e["num_iteration"]), alpha=e["alpha"], mini_batch_fraction=e["minibatch_fraction"],
              reg_param=e["regParam"], reg_type=e["reg_type"], intercept=e["intercept"],
              splits=splits if ranks == 4 else None)
    r = oracle.logreg_sgd(a, label, w0=np.zeros(a.n), b0=1.0, l2_no_eta=True, **kw)
    pb = oracle.predict_probability(a, r["w"], r["b"])
    assert np.max(np.abs(pb - e["expected_out_pb"])) < 5e-7
    assert r["n_iter"] == 129
    cur = oracle.logreg_sgd(a, label, **kw)
    pred = np.where(oracle.predict_probability(a, cur["w"], cur["b"]) >= 0.5, 1.0, -1.0)
    assert np.array_equal(pred, e["expected_out_p"])


def test_formats_agree_on_random_matrix():
    rng = np.random.default_rng(1)
    m, n = 700, 90
    lens = rng.integers(0, 40, m)
    lens[::97] = 0
    lens[5] = 600 if n >= 600 else n
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate([np.sort(rng.choice(n, l, replace=False)) for l in lens]).astype(np.int32)
    val = rng.standard_normal(off[-1])
    a = oracle.CRS(m, n, off, idx, val)
    x = rng.standard_normal(n)
    ref = a.to_dense() @ x
    for fn in (oracle.spmv, oracle.ell_spmv, oracle.jds_spmv, oracle.hyb_spmv):
        np.testing.assert_allclose(fn(a, x), ref, rtol=1e-12, atol=1e-12)
    r = rng.standard_normal(m)
    reft = a.to_dense().T @ r
    np.testing.assert_allclose(oracle.ell_trans_mv(a, r), reft, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle.spmv(oracle.transpose(a), r), reft, rtol=1e-12, atol=1e-12)
    for fmt in ("CRS", "JDS", "ELL", "HYBRID"):
        np.testing.assert_allclose(oracle.fmt_mv(a, fmt, r, trans=True), reft, rtol=1e-12, atol=1e-12)
    X = rng.standard_normal((n, 5))
    np.testing.assert_allclose(oracle.spmm(a, X), a.to_dense() @ X, rtol=1e-12, atol=1e-12)


def test_jds_order_ties_by_descending_row():
    # (len,row) sorted with std::greater: equal lengths → larger row first
    off = np.array([0, 2, 4, 5, 7], dtype=np.int32)
    idx = np.array([0, 1, 0, 1, 1, 0, 1], dtype=np.int32)
    a = oracle.CRS(4, 2, off, idx, np.arange(1.0, 8.0))
    perm, joff, jidx, jval = oracle.jds_build(a)
    assert list(perm) == [3, 1, 0, 2]
    assert list(joff) == [0, 4, 7]


def test_oracle_loaders_on_tutorial_files(tmp_path):
    # make_crs_matrix_local_load on doc/tutorial/src/tut3.2.1-1/data and
    # make_crs_matrix_local_loadbinary on tut3.2.1-2/data_binary
    g = golden()
    p = tmp_path / "data"
    p.write_text(g["tut_spmv"]["raw_text"])
    off, idx, val, m, n = oracle.load_text(str(p))
    assert (m, n) == (g["tut_spmv"]["m"], g["tut_spmv"]["n"])
    assert off.tolist() == g["tut_spmv"]["off"] and idx.tolist() == g["tut_spmv"]["idx"]
    assert val.tolist() == g["tut_spmv"]["val"]
    d = tmp_path / "data_binary"
    d.mkdir()
    rf = g["tut_binary"]["raw_files"]
    for k in ("nums", "type"):
        (d / k).write_text(rf[k])
    for k in ("val", "idx", "off"):
        (d / k).write_bytes(bytes.fromhex(rf[k]))
    off, idx, val, m, n = oracle.load_binary(str(d))
    assert (m, n) == (g["tut_binary"]["m"], g["tut_binary"]["n"])
    assert off.tolist() == g["tut_binary"]["off"] and idx.tolist() == g["tut_binary"]["idx"]
    assert val.tolist() == g["tut_binary"]["val"]


@pytest.mark.parametrize("name", ["test1.1-1", "test1.2-1", "test1.3-1"])
@pytest.mark.parametrize("ranks", [1, 4])
def test_regression_sgd_golden(name, ranks):
    # test/ml/test1.{1,2,3}-1/test.cc: linear_regression_with_sgd,
    # lasso_with_sgd, ridge_regression_with_sgd, predictions stored with six
    # significant digits.  Reproduced to those digits (|err| <= 5e-6) by the
    # same earlier initial model as test2.1-1 (weights 0, intercept 1; L2
    # without USE_ETA); all three stop at iteration 3 on the RMS test.
    e, a, label, splits = _glm(name)
    r = oracle.logreg_sgd(a, label, loss=e["loss"], num_iter=int(e["num_iteration"]), alpha=e["alpha"],
                          mini_batch_fraction=e["minibatch_fraction"], reg_param=e.get("regParam", 0.0),
                          reg_type=e["reg_type"], intercept=e["intercept"], w0=np.zeros(a.n), b0=1.0,
                          l2_no_eta=True, splits=splits if ranks == 4 else None)
    pred = a.to_dense() @ r["w"] + r["b"]
    assert np.max(np.abs(pred - e["expected_out"])) <= 5e-6
    assert r["n_iter"] == 3


@pytest.mark.parametrize("name", ["test1.1-2", "test1.2-2", "test1.3-2"])
def test_regression_lbfgs_golden(name):
    # test/ml/test1.{1,2,3}-2/test.cc store predictions of an earlier L-BFGS
    # (they sit next to the SGD ones, a model barely moved from its start);
    # the current lbfgs_parallelizer (unit first step, line search on the
    # loss) fits the six points far better.  Not reproducible from the
    # current source: the check is that the current trainer's squared loss
    # is below the stored model's.
    e, a, label, splits = _glm(name)
    r = oracle.logreg_lbfgs(a, label, loss="linear", num_iter=int(e["num_iteration"]), alpha=e["alpha"],
                            hist_size=int(e["hist_size"]), reg_param=e.get("regParam", 0.0), reg_type=e["reg_type"],
                            intercept=e["intercept"], splits=splits)
    stored = 0.5 * np.sum((np.array(e["expected_out"]) - label) ** 2)
    assert r["loss"] < stored


@pytest.mark.parametrize("name", ["test2.2-1", "test2.2-2"])
def test_svm_golden_predictions(name):
    # test/ml/test2.2-{1,2}/test.cc: svm_with_sgd / svm_with_lbfgs, predicted
    # classes {1,-1,1,1}.  The stored raw scores (predict_probability) come
    # from an earlier source and are not reproducible; the classes are.
    e, a, label, splits = _glm(name)
    kw = dict(loss="hinge", num_iter=int(e["num_iteration"]), alpha=e["alpha"], reg_param=e["regParam"],
              reg_type=e["reg_type"], intercept=e["intercept"], splits=splits)
    if e["solver"] == "sgd":
        r = oracle.logreg_sgd(a, label, mini_batch_fraction=e["minibatch_fraction"], **kw)
    else:
        r = oracle.logreg_lbfgs(a, label, hist_size=int(e["hist_size"]), **kw)
    pred = np.where(a.to_dense() @ r["w"] + r["b"] > 0, 1.0, -1.0)
    assert np.array_equal(pred, e["expected_out_p"])


def test_glm_dloss_kinds():
    # gradient.hpp:55-202 on hand-checked values
    lab = np.array([1.0, -1.0, 1.0])
    wtx = np.array([0.5, 2.0, 3.0])
    d, s = oracle.glm_dloss(lab, wtx, "hinge")
    assert d.tolist() == [-1.0, 1.0, 0.0] and s == 3.5
    d, s = oracle.glm_dloss(lab, wtx, "linear")
    assert d.tolist() == [-0.5, 3.0, 2.0] and s == 0.5 * (0.25 + 9.0 + 4.0)
    d, s = oracle.glm_dloss(lab, wtx, "eps", 0.6)
    assert d.tolist() == [0.0, 1.0, 1.0] and abs(s - 3.8) < 1e-15
    d, s = oracle.glm_dloss(lab, wtx, "sqeps", 0.6)
    assert np.allclose(d, [0.0, 4.8, 2.8], rtol=0, atol=1e-15) and abs(s - (2.4 ** 2 + 1.4 ** 2)) < 1e-12
    d, _ = oracle.glm_dloss(np.zeros(2), np.array([2e12, -3e12]), "linear")
    assert d.tolist() == [1e12, -1e12]  # MAX_LOSS / MIN_LOSS clip


def test_shrink_sgd_equals_sgd_without_regulariser():
    # with no regulariser and no stop test the shrink driver only differs in
    # the columns no rank uses (returned as 0); the update is the same
    rng = np.random.default_rng(12)
    m, n = 600, 80
    lens = rng.integers(0, 8, m)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate([np.sort(rng.choice(60, k, replace=False)) for k in lens]).astype(np.int32)
    a = oracle.CRS(m, n, off, idx, rng.standard_normal(off[-1]))
    label = np.where(rng.random(m) < 0.5, 1.0, -1.0)
    kw = dict(num_iter=10, alpha=0.05, reg_type="ZERO", intercept=True, tol=0.0, splits=[0, 200, 600])
    r1 = oracle.logreg_sgd(a, label, shrink=True, **kw)
    r2 = oracle.logreg_sgd(a, label, **kw)
    used = np.zeros(n, bool)
    used[idx] = True
    assert np.array_equal(r1["w"][used], r2["w"][used]) and r1["b"] == r2["b"]
    assert np.all(r1["w"][~used] == 0.0) and np.all(r2["w"][~used] == 1.0)


def test_oracle_problem_matches_one_shot_trainer():
    # the prebuilt problem (per-rank matrices built once) runs the same
    # trainer: identical results to the one-shot call, run after run
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=3000, n=400, lam=12.0, seed=21))
    a = oracle.CRS(3000, 400, off, idx, val)
    splits = [0, 900, 2000, 3000]
    kw = dict(num_iter=12, reg_type="L2", reg_param=1e-3, intercept=True)
    ro = oracle.logreg_lbfgs(a, label, splits=splits, nthreads=3, **kw)
    pr = oracle.Problem(a, label, splits=splits, nthreads=3)
    for _ in range(2):
        rp = pr.lbfgs(**kw)
        assert rp["n_iter"] == ro["n_iter"] and rp["loss"] == ro["loss"]
        assert np.array_equal(rp["w"], ro["w"]) and rp["b"] == ro["b"]
        assert np.array_equal(rp["trace"], ro["trace"])
    pr.close()
