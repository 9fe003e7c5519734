"""GPU parity of the multi-dataset batched L-BFGS trainer (fvg_logreg_lbfgs_multi).

Datasets of uneven size (rows, columns, nonzeros, long rows, empty rows) are
stacked and trained together with k regularisation values each.  Every
model (d, j) is checked against its own oracle run of
logistic_regression_with_lbfgs::train on dataset d
(logistic_regression_with_lbfgs.hpp:395-437, FP64): identical iteration
count, final loss rel 1e-6, weights and intercept rel 1e-5.
"""
import numpy as np
import pytest

import oracle

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fv.Context(0)
    yield c
    c.close()


def _ds(seed, m, n, lam=12.0, long_rows=0, empty_every=0):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed))
    a = oracle.CRS(m, n, off, idx, val)
    if long_rows or empty_every:
        # rows over the product's 512-nonzero work item (split into pieces),
        # and empty rows
        rng = np.random.default_rng(seed + 1000)
        rows = [np.sort(rng.choice(n, size=min(n, 900 + 37 * i), replace=False)) for i in range(long_rows)]
        lens = np.diff(a.off).astype(np.int64)
        segs = [a.idx[a.off[r]:a.off[r + 1]] for r in range(m)]
        vals = [a.val[a.off[r]:a.off[r + 1]] for r in range(m)]
        for i, cols in enumerate(rows):
            r = (7 + 131 * i) % m
            segs[r] = cols.astype(np.int32)
            vals[r] = np.abs(rng.standard_normal(len(cols))) * 0.05
            lens[r] = len(cols)
        if empty_every:
            for r in range(3, m, empty_every):
                if lens[r] < 512:
                    segs[r] = segs[r][:0]
                    vals[r] = vals[r][:0]
                    lens[r] = 0
        off = np.zeros(m + 1, np.int64)
        off[1:] = np.cumsum(lens)
        a = oracle.CRS(m, n, off.astype(np.int32), np.concatenate(segs).astype(np.int32), np.concatenate(vals))
    return a, label


def _check(r, d, j, a, label, lam, **kw):
    ro = oracle.logreg_lbfgs(a, label, reg_param=lam, **kw)
    assert r["n_iter"][d, j] == ro["n_iter"], (d, j)
    assert abs(r["loss"][d, j] - ro["loss"]) <= 1e-6 * abs(ro["loss"]), (d, j)
    assert np.max(np.abs(r["w"][d][j] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"]))), (d, j)
    assert abs(r["b"][d, j] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"])), (d, j)


def test_multi_uneven_datasets_match_oracle(ctx):
    shapes = [(3000, 200, 0), (700, 90, 0), (5200, 1500, 3), (150, 40, 0), (2100, 800, 1)]
    data = [_ds(50 + i, m, n, long_rows=lr, empty_every=11 if i == 2 else 0) for i, (m, n, lr) in enumerate(shapes)]
    mats = [ctx.matrix(a.m, a.n, a.off, a.idx, a.val) for a, _ in data]
    lams = [0.0, 1e-4, 1e-3, 1e-2, 0.1, 0.5]
    kw = dict(num_iter=20, reg_type="L2", intercept=True)
    w0 = [np.zeros(a.n) for a, _ in data]
    r = fv.logreg_lbfgs_multi(mats, [l for _, l in data], lams, w0=w0, **kw)
    assert r["loss"].shape == (len(shapes), len(lams))
    for d, (a, label) in enumerate(data):
        for j, lam in enumerate(lams):
            _check(r, d, j, a, label, lam, w0=np.zeros(a.n), **kw)


@pytest.mark.parametrize("reg", ["L1", "ZERO"])
def test_multi_other_regularisers(ctx, reg):
    data = [_ds(60 + i, m, n) for i, (m, n) in enumerate([(1800, 120), (600, 70), (2500, 160)])]
    mats = [ctx.matrix(a.m, a.n, a.off, a.idx, a.val) for a, _ in data]
    lams = [1e-3, 3e-2, 0.2]
    kw = dict(num_iter=15, reg_type=reg, intercept=False)
    r = fv.logreg_lbfgs_multi(mats, [l for _, l in data], lams, **kw)
    for d, (a, label) in enumerate(data):
        for j, lam in enumerate(lams):
            _check(r, d, j, a, label, lam, **kw)


def test_multi_sample_weights_initial_models_and_early_stop(ctx):
    rng = np.random.default_rng(7)
    data = [_ds(70 + i, m, n) for i, (m, n) in enumerate([(1500, 100), (900, 60)])]
    mats = [ctx.matrix(a.m, a.n, a.off, a.idx, a.val) for a, _ in data]
    sws = [rng.uniform(0.5, 2.0, data[0][0].m), None]
    lams = list(np.logspace(-4, 0, 5))
    w0 = [rng.standard_normal((len(lams), a.n)) * 0.01 for a, _ in data]
    b0 = rng.standard_normal((2, len(lams))) * 0.1
    kw = dict(num_iter=40, reg_type="L2", intercept=True, tol=3e-2)
    r = fv.logreg_lbfgs_multi(mats, [l for _, l in data], lams, sample_weights=sws, w0=w0, b0=b0, **kw)
    stopped = 0
    for d, (a, label) in enumerate(data):
        for j, lam in enumerate(lams):
            ro = oracle.logreg_lbfgs(a, label, reg_param=lam, sw=sws[d], w0=w0[d][j], b0=b0[d, j], **kw)
            assert r["n_iter"][d, j] == ro["n_iter"], (d, j)
            stopped += ro["n_iter"] < kw["num_iter"]
            assert abs(r["loss"][d, j] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
            assert np.max(np.abs(r["w"][d][j] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    assert stopped > 0  # some models stop on their own while the others go on


def test_multi_equals_separate_batched_runs(ctx):
    # stacking changes nothing but summation order: each dataset's models
    # equal the one-dataset batched trainer's
    data = [_ds(80 + i, m, n) for i, (m, n) in enumerate([(2000, 150), (400, 150), (3100, 150)])]
    mats = [ctx.matrix(a.m, a.n, a.off, a.idx, a.val) for a, _ in data]
    lams = np.logspace(-6, 0, 64)
    kw = dict(num_iter=10, reg_type="L2", intercept=True)
    w0 = [np.zeros(a.n) for a, _ in data]
    e0 = ctx.profile("batch_evals")
    r = fv.logreg_lbfgs_multi(mats, [l for _, l in data], lams, w0=w0, **kw)
    e1 = ctx.profile("batch_evals")
    evals, model_evals = e1[1] - e0[1], e1[0] - e0[0]
    # the initial evaluation and at least one trial per iteration; the later
    # trials evaluate only the models still searching
    assert evals >= kw["num_iter"] + 1
    assert 3 * 64 * (kw["num_iter"] + 1) <= model_evals < evals * 3 * 64
    for d, (A, (a, label)) in enumerate(zip(mats, data)):
        rb = fv.logreg_lbfgs_batched(A, label, lams, w0=np.zeros(a.n), **kw)
        assert np.array_equal(r["n_iter"][d], rb["n_iter"])
        assert np.max(np.abs(r["loss"][d] - rb["loss"]) / np.abs(rb["loss"])) <= 1e-9
        assert np.max(np.abs(r["w"][d] - rb["w"])) <= 1e-7 * max(1.0, np.max(np.abs(rb["w"])))
    for j in (0, 31, 63):
        _check(r, 1, j, data[1][0], data[1][1], lams[j], w0=np.zeros(data[1][0].n), **kw)


def test_multi_reduced_precision(ctx):
    data = [_ds(90 + i, m, n) for i, (m, n) in enumerate([(2500, 180), (1200, 90)])]
    mats = [ctx.matrix(a.m, a.n, a.off, a.idx, a.val) for a, _ in data]
    lams = [1e-4, 1e-2, 0.1]
    kw = dict(num_iter=20, reg_type="L2", intercept=True)
    for storage in ("f32", "bf16"):
        r = fv.logreg_lbfgs_multi(mats, [l for _, l in data], lams, storage=storage,
                                  w0=[np.zeros(a.n) for a, _ in data], **kw)
        for d, (a, label) in enumerate(data):
            for j, lam in enumerate(lams):
                ro = oracle.logreg_lbfgs(a, label, reg_param=lam, w0=np.zeros(a.n), **kw)
                assert abs(r["loss"][d, j] - ro["loss"]) <= 1e-3 * abs(ro["loss"]), (storage, d, j)


def test_multi_errors(ctx):
    a, label = _ds(99, 300, 40)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    B = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_multi([A, B], [label, label], np.full(257, 1e-3))
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_multi([A, B], [label, label], [1e-3], storage="split")
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_multi([A, B], [label, label], [1e-3], mat_type="ELL")
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs_multi([A, B], [label, label], [-1.0])
    c2 = fv.Context(0)
    try:
        C2 = c2.matrix(a.m, a.n, a.off, a.idx, a.val)
        with pytest.raises(fv.FvgError):
            fv.logreg_lbfgs_multi([A, C2], [label, label], [1e-3])
    finally:
        c2.close()
    # the context still works after the refusals
    r = fv.logreg_lbfgs_multi([A, B], [label, label], [1e-3], num_iter=3)
    assert np.allclose(r["loss"][0], r["loss"][1], rtol=1e-12)
