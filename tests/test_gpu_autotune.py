"""The training-layout autotuner (fvg_matrix_autotune).

Every candidate layout computes the same sums up to summation order, so the
tuner may pick any of them: each one the tuner timed must train, with split
storage, to the FP64 oracle's model within the path's bar (relative error
<= 1e-6 on the loss, <= 1e-5 on the weights, the same line-search
decisions), and the chosen one must be the fastest it measured and be left
set on the matrix.
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


def _data(m=400_000, n=30_000, seed=12):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=20.0, seed=seed, val_kind="lognormal"))
    return oracle.CRS(m, n, off, idx, val), label


def test_autotune_split_choices_train_to_the_bar(ctx):
    a, label = _data()
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    best, tried = A.autotune("split", label, reps=2)
    assert tried and all(t["eval_ms"] > 0 for t in tried)
    assert best["eval_ms"] == min(t["eval_ms"] for t in tried)
    assert best in tried
    # the best layout is left set
    assert (A.head_info()[0] > 0) == best["head"] and (A.panel_info()[2] > 0) == (best["panel_min"] > 0)
    kw = dict(num_iter=15, reg_type="L2", reg_param=1e-3, w0=np.zeros(a.n))
    ro = oracle.logreg_lbfgs(a, label, nthreads=8, **kw)
    for t in tried:
        A.set_head(-1 if t["head"] else 0)
        if t["panel_min"] > 0:
            A.set_panels(-1, t["panel_min"])
        else:
            A.set_panels(0)
        r = fv.logreg_lbfgs(A, label, storage="split", mat_type=t["format"], trace=True, **kw)
        assert r["n_iter"] == ro["n_iter"], t
        assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1]), t
        assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"]), t
        assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"]))), t
    A.close()


def test_autotune_lower_precision_candidates(ctx):
    # FP32 values: CRS with and without the layouts, the hybrid, and ELL when
    # its padding is small; every candidate timed and the fastest left set
    a, label = _data(m=120_000, n=20_000, seed=13)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.add_storage("f32")
    best, tried = A.autotune("f32", label, reps=2)
    fmts = {t["format"] for t in tried}
    assert "CRS" in fmts and "HYBRID" in fmts
    assert best["eval_ms"] == min(t["eval_ms"] for t in tried)
    with pytest.raises(fv.FvgError):
        A.autotune(7, label)  # unknown storage
    A.close()
