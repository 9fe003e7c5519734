"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle and
the reference's own fixtures.

Tolerances: integer/index layouts (transpose, ELL, JDS, hybrid, row
permutations) are compared bit for bit.  FP64 products differ from the
oracle only in summation order: rel 1e-12.  FP32/BF16 storage accumulates
in FP32: rel 2e-5 of the row's absolute sum.  Trained models: relative error
<= 1e-6 on the final loss and <= 1e-5 on the weights (the stated target).
"""
import numpy as np
import pytest

import oracle
from _golden import crs, crs_text, golden

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu

FMTS = ["CRS", "ELL", "JDS", "HYBRID"]


@pytest.fixture(scope="module")
def ctx():
    c = fv.Context(0)
    yield c
    c.close()


def rand_crs(rng, m, n, maxlen=40, long_rows=(), empty_every=13, dup_row=None):
    lens = np.minimum(rng.integers(0, maxlen + 1, m), n)
    lens[::empty_every] = 0
    for r, L in long_rows:
        lens[r] = min(L, n)
    rows = []
    for r in range(m):
        rows.append(np.sort(rng.choice(n, lens[r], replace=False)))
    if dup_row is not None and lens[dup_row] >= 2:
        rows[dup_row][1] = rows[dup_row][0]  # duplicate column id inside one row
    off = np.concatenate([[0], np.cumsum([len(x) for x in rows])]).astype(np.int32)
    idx = np.concatenate(rows).astype(np.int32) if off[-1] else np.zeros(0, np.int32)
    val = rng.standard_normal(int(off[-1]))
    return oracle.CRS(m, n, off, idx, val)


def close(a, b, rtol):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.max(np.abs(a - b) / (np.abs(b) + 1.0)) <= rtol if a.size else True


# ----------------------------------------------------------- reference fixtures
def test_tutorial_spmv_golden_all_formats(ctx):
    g = golden()["tut_spmv"]
    a = crs(g)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    exp = np.array(g["expected_y_ones"])
    for fmt in FMTS:
        assert np.array_equal(A.spmv(np.ones(a.n), fmt=fmt), exp), fmt
        assert np.array_equal(A.spmv(np.ones(a.n, np.float32), fmt=fmt, storage="f32", vec="f32"), exp), fmt
        assert np.array_equal(A.spmv(np.ones(a.n, np.float32), fmt=fmt, storage="bf16", vec="f32"), exp), fmt


def test_tutorial_transpose_golden(ctx):
    g = golden()["tut_binary"]
    a = crs(g)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    toff, tidx, tval = A.get_transpose()
    assert crs_text(oracle.CRS(a.n, a.m, toff, tidx, tval)) == g["expected_transpose_text"]


def _glm(name):
    e = golden()[name]
    return e, crs(e), np.array(e["label"])


def test_lbfgs_golden_test2_1_2(ctx):
    e, a, label = _glm("test2.1-2")
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    r = fv.logreg_lbfgs(A, label, num_iter=int(e["num_iteration"]), alpha=e["alpha"], hist_size=int(e["hist_size"]),
                        reg_param=e["regParam"], reg_type=e["reg_type"], intercept=e["intercept"])
    pb = fv.predict_probability(A, r["w"], r["b"])
    pred = np.where(pb >= 0.5, 1.0, -1.0)
    assert np.sqrt(np.mean((pred - e["expected_out_p"]) ** 2)) < e["rms_tol"]
    assert np.sqrt(np.mean((pb - e["expected_out_pb"]) ** 2)) < e["rms_tol"]
    ro = oracle.logreg_lbfgs(a, label, num_iter=int(e["num_iteration"]), alpha=e["alpha"],
                             hist_size=int(e["hist_size"]), reg_param=e["regParam"], reg_type=e["reg_type"],
                             intercept=e["intercept"])
    assert r["n_iter"] == ro["n_iter"]
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"]) + 1e-12


@pytest.mark.parametrize("ranks", [1, 4])
def test_sgd_golden_test2_1_1(ctx, ranks):
    e, a, label = _glm("test2.1-1")
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    splits = oracle.text_rank_splits(bytes.fromhex(e["data_bytes_hex"]), 4) if ranks == 4 else None
    r = fv.logreg_sgd(A, label, num_iter=int(e["num_iteration"]), alpha=e["alpha"],
                      mini_batch_fraction=e["minibatch_fraction"], reg_param=e["regParam"], reg_type=e["reg_type"],
                      intercept=e["intercept"], w0=np.zeros(a.n), b0=1.0, l2_no_eta=1, row_splits=splits)
    pb = fv.predict_probability(A, r["w"], r["b"])
    assert np.max(np.abs(pb - e["expected_out_pb"])) < 5e-7
    assert r["n_iter"] == 129


# ----------------------------------------------------------------- layouts
def _cases(rng):
    yield "random", rand_crs(rng, 700, 90, dup_row=7)
    yield "long_rows", rand_crs(rng, 300, 40000, maxlen=70, long_rows=[(3, 39000), (150, 20000), (151, 16385)])
    yield "all_empty", oracle.CRS(50, 20, np.zeros(51, np.int32), np.zeros(0, np.int32), np.zeros(0))
    yield "one_row", rand_crs(rng, 1, 64, maxlen=64, empty_every=1000)
    yield "tiny_hybrid", rand_crs(rng, 200, 30)  # rows <= 256: hybrid is all CRS


def test_transpose_bit_exact(ctx):
    rng = np.random.default_rng(5)
    for name, a in _cases(rng):
        A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
        toff, tidx, tval = A.get_transpose()
        t = oracle.transpose(a)
        assert np.array_equal(toff, t.off), name
        assert np.array_equal(tidx, t.idx), name
        assert np.array_equal(tval, t.val), name


def test_transpose_bit_exact_fp32_bf16_values(ctx):
    # the transposed copy's sort carries 4- and 2-byte values for matrices
    # uploaded with FP32 or BF16 values (odd tile tails included)
    rng = np.random.default_rng(15)
    for name, a in _cases(rng):
        for kind in ("f32", "bf16"):
            if kind == "f32":
                v = a.val.astype(np.float32)
                exact = v.astype(np.float64)
            else:
                v = fv.bf16_bits(a.val)
                exact = (v.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
            A = ctx.matrix(a.m, a.n, a.off, a.idx, v)
            toff, tidx, tval = A.get_transpose()
            t = oracle.transpose(oracle.CRS(a.m, a.n, a.off, a.idx, exact))
            assert np.array_equal(toff, t.off), (name, kind)
            assert np.array_equal(tidx, t.idx), (name, kind)
            assert np.array_equal(tval, t.val), (name, kind)


def test_ell_jds_hybrid_layouts_bit_exact(ctx):
    rng = np.random.default_rng(6)
    for name, a in _cases(rng):
        if name == "long_rows":
            continue  # ELL of a 39000-wide row is large; covered by the hybrid case below
        A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
        w, eidx, ev = A.get_ell()
        ow, oeidx, oev = oracle.ell_build(a)
        assert w == ow and np.array_equal(eidx, oeidx) and np.array_equal(ev, oev), name
        if a.nnz:
            perm, joff, jidx, jval = A.get_jds()
            operm, ojoff, ojidx, ojval = oracle.jds_build(a)
            assert np.array_equal(perm, operm) and np.array_equal(joff, ojoff), name
            assert np.array_equal(jidx, ojidx) and np.array_equal(jval, ojval), name
    for thr_case in ("random", "long_rows"):
        a = dict(_cases(np.random.default_rng(7)))[thr_case]
        A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
        h = A.get_hybrid()
        o = oracle.hyb_build(a)
        for k in ("perm", "joff", "jidx", "jval", "coff", "cidx", "cval"):
            assert np.array_equal(h[k], o[k]), (thr_case, k)
        assert h["crs_rows"] == o["crs_rows"]


# ---------------------------------------------------------------- products
def test_spmv_and_trans_mv_all_formats(ctx):
    rng = np.random.default_rng(8)
    for name, a in _cases(rng):
        A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
        x = rng.standard_normal(a.n)
        r = rng.standard_normal(a.m)
        ref_y = oracle.spmv(a, x)
        ref_t = oracle.spmv(oracle.transpose(a), r)
        for fmt in FMTS:
            if fmt == "ELL" and name == "long_rows":
                continue
            assert close(A.spmv(x, fmt=fmt), ref_y, 1e-12), (name, fmt)
            assert close(A.trans_mv(r, fmt=fmt), ref_t, 1e-12), (name, fmt)
            # oracle restatements of the same format agree too
        assert close(A.spmv(x, fmt="HYBRID"), oracle.hyb_spmv(a, x), 1e-12)
        if name != "long_rows":
            assert close(A.spmv(x, fmt="ELL"), oracle.ell_spmv(a, x), 1e-12)
            assert close(A.trans_mv(r, fmt="ELL"), oracle.ell_trans_mv(a, r), 1e-12)
        assert close(A.spmv(x, fmt="JDS"), oracle.jds_spmv(a, x), 1e-12)


def test_spmv_low_precision_storage(ctx):
    rng = np.random.default_rng(9)
    for name, a in _cases(rng):
        A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
        x = rng.standard_normal(a.n).astype(np.float32)
        absrow = oracle.spmv(oracle.CRS(a.m, a.n, a.off, a.idx, np.abs(a.val)), np.abs(x.astype(np.float64)))
        # FP32 storage: against FP32-rounded values in FP64
        v32 = a.val.astype(np.float32).astype(np.float64)
        ref32 = oracle.spmv(oracle.CRS(a.m, a.n, a.off, a.idx, v32), x.astype(np.float64))
        vb = (fv.bf16_bits(a.val).astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        refb = oracle.spmv(oracle.CRS(a.m, a.n, a.off, a.idx, vb), x.astype(np.float64))
        for fmt in FMTS:
            if fmt == "ELL" and name == "long_rows":
                continue
            y32 = A.spmv(x, fmt=fmt, storage="f32", vec="f32").astype(np.float64)
            assert np.all(np.abs(y32 - ref32) <= 2e-5 * (absrow + 1e-30)), (name, fmt)
            yb = A.spmv(x, fmt=fmt, storage="bf16", vec="f32").astype(np.float64)
            assert np.all(np.abs(yb - refb) <= 2e-5 * (absrow + 1e-30)), (name, fmt)


def test_spmv_deterministic(ctx):
    rng = np.random.default_rng(10)
    a = rand_crs(rng, 300, 40000, maxlen=70, long_rows=[(3, 39000), (150, 20000)])
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    x = rng.standard_normal(a.n)
    r = rng.standard_normal(a.m)
    y0, t0 = A.spmv(x), A.trans_mv(r)
    for _ in range(3):
        assert np.array_equal(A.spmv(x), y0)
        assert np.array_equal(A.trans_mv(r), t0)


def test_spmm(ctx):
    rng = np.random.default_rng(11)
    a = rand_crs(rng, 400, 120)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for k in (1, 5, 64, 70):
        X = rng.standard_normal((a.n, k))
        assert close(A.spmm(X), oracle.spmm(a, X), 1e-12), k


def test_size_and_argument_errors(ctx):
    rng = np.random.default_rng(12)
    a = rand_crs(rng, 20, 10)
    with pytest.raises(fv.FvgError):
        ctx.matrix(3, 2, np.array([0, 1, 2, 3]), np.array([0, 1, 5]), np.ones(3))  # column out of range
    with pytest.raises(fv.FvgError):
        ctx.matrix(2, 2, np.array([0, 2, 1]), np.array([0, 1]), np.ones(2))  # decreasing offsets
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs(A, np.ones(a.m), mat_type="JDS")  # lbfgs_parallelizer.hpp:596-597
    with pytest.raises(fv.FvgError):
        fv.logreg_lbfgs(A, np.ones(a.m), num_iter=0)
    with pytest.raises(fv.FvgError):
        A.spmv(np.ones(a.n), storage="f64", vec="f32")


# ------------------------------------------------------------ logistic path
def _lr_data(seed=0, m=4000, n=300, lam=15.0):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed))
    return oracle.CRS(m, n, off, idx, val), label


@pytest.mark.parametrize("fmt", FMTS)
def test_fused_eval_matches_oracle(ctx, fmt):
    a, label = _lr_data(1)
    rng = np.random.default_rng(2)
    sw = rng.uniform(0.5, 2.0, a.m)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for icpt in (False, True):
        w = rng.standard_normal(a.n) * 0.3
        g, loss = fv.logreg_eval(A, label, w, b=0.7, intercept=icpt, sample_weight=sw, fmt=fmt)
        go, losso = oracle.logreg_eval(a, label, w, b=0.7, intercept=icpt, sw=sw, fmt=fmt)
        assert abs(loss - losso) <= 1e-12 * abs(losso), (fmt, icpt)
        assert close(g, go, 1e-11), (fmt, icpt)
        if not icpt:
            assert g[-1] == 0.0


@pytest.mark.parametrize("n", [300, 20000])
def test_fp32_eval_matches_fp64_on_fp32_values(ctx, n):
    # Values are FP32- (BF16-) representable, so the FP64 evaluation is the
    # exact reference and the only difference is FP32 arithmetic; n = 300
    # gives dense Zipf-hot columns, n = 20000 a long tail.
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=6000, n=n, lam=30.0, seed=8))
    val = val.astype(np.float32).astype(np.float64)
    A = ctx.matrix(6000, n, off, idx, val)
    rng = np.random.default_rng(9)
    w = rng.standard_normal(n) * 0.2
    g64, l64 = fv.logreg_eval(A, label, w, b=0.3, intercept=True)
    aref = oracle.CRS(6000, n, off, idx, np.abs(val))
    scale = oracle.spmv(oracle.transpose(aref), np.ones(6000))  # sum |a_ij| per column
    for storage in ("f32", "bf16"):
        if storage == "bf16":
            vb = (fv.bf16_bits(val).astype(np.uint32) << 16).view(np.float32).astype(np.float64)
            B = ctx.matrix(6000, n, off, idx, vb)
            g64b, l64b = fv.logreg_eval(B, label, w, b=0.3, intercept=True)
            g, loss = fv.logreg_eval(B, label, w, b=0.3, intercept=True, storage="bf16")
        else:
            g64b, l64b = g64, l64
            g, loss = fv.logreg_eval(A, label, w, b=0.3, intercept=True, storage="f32")
        assert abs(loss - l64b) <= 1e-5 * abs(l64b), storage
        assert np.max(np.abs(g[:-1] - g64b[:-1]) / (scale + 1.0)) <= 1e-5, storage
        assert abs(g[-1] - g64b[-1]) <= 1e-5 * 6000, storage


def test_fused_eval_extreme_margins(ctx):
    # z > 18, z < -18 and the clip branches of compute_dloss (gradient.hpp:29-48)
    a, label = _lr_data(3, m=2000, n=50)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    for scale in (0.0, 3.0, 40.0):
        w = np.full(a.n, scale)
        g, loss = fv.logreg_eval(A, label, w, b=-scale, intercept=True)
        go, losso = oracle.logreg_eval(a, label, w, b=-scale, intercept=True)
        assert abs(loss - losso) <= 1e-12 * abs(losso) + 1e-300, scale
        assert close(g, go, 1e-11), scale


@pytest.mark.parametrize("fmt,reg", [("CRS", "L2"), ("CRS", "ZERO"), ("CRS", "L1"), ("HYBRID", "L2"),
                                     ("ELL", "L2")])
def test_lbfgs_matches_oracle(ctx, fmt, reg):
    a, label = _lr_data(4)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=20, reg_type=reg, reg_param=1e-3, intercept=True, fmt=fmt)
    r = fv.logreg_lbfgs(A, label, trace=True, **{("mat_type" if k == "fmt" else k): v for k, v in kw.items()})
    ro = oracle.logreg_lbfgs(a, label, **kw)
    assert r["n_iter"] == ro["n_iter"]
    assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1]), "line-search trial counts differ"
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    assert abs(r["b"] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"]))


@pytest.mark.parametrize("fmt", FMTS)
def test_sgd_matches_oracle(ctx, fmt):
    a, label = _lr_data(5, m=5000, n=200)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=15, alpha=0.05, mini_batch_fraction=0.3, reg_type="L2", reg_param=1e-2, intercept=True)
    r = fv.logreg_sgd(A, label, mat_type=fmt, **kw)
    ro = oracle.logreg_sgd(a, label, fmt=fmt, **kw)
    assert r["n_iter"] == ro["n_iter"]
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))


def test_sgd_multi_rank_emulation(ctx):
    a, label = _lr_data(6, m=3000, n=100)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    splits = [0, 700, 1500, 3000]
    kw = dict(num_iter=10, alpha=0.05, mini_batch_fraction=0.5, reg_type="L2", reg_param=1e-2, intercept=True)
    r = fv.logreg_sgd(A, label, row_splits=splits, **kw)
    ro = oracle.logreg_sgd(a, label, splits=splits, **kw)
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))


def test_mixed_precision_lbfgs_close_to_fp64(ctx):
    a, label = _lr_data(7, m=6000, n=400)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    ro = oracle.logreg_lbfgs(a, label, num_iter=30, reg_type="L2", reg_param=1e-3)
    for storage in ("f32", "bf16"):
        r = fv.logreg_lbfgs(A, label, num_iter=30, reg_type="L2", reg_param=1e-3, storage=storage)
        rel = abs(r["loss"] - ro["loss"]) / abs(ro["loss"])
        assert rel <= 1e-3, (storage, rel)


def test_predict_probability(ctx):
    a, label = _lr_data(8, m=500, n=40)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    w = np.random.default_rng(0).standard_normal(a.n) * 5
    for b in (0.0, 1.5):
        assert close(fv.predict_probability(A, w, b), oracle.predict_probability(a, w, b), 1e-13)


def test_lbfgs_logreg_100k_20k_configuration(ctx):
    # the reference's CPU-sized configuration at full size: 100,000 x 20,000,
    # nnz/row 1+Poisson(39), Zipf(1.1) columns, |N(0,1)| values, L2 1e-3,
    # 20 iterations, FP64 — every line-search decision as the oracle's.
    # From zero weights the run is well conditioned (the oracle with 1 and 4
    # emulated ranks agrees to 2e-14): loss 1e-6, weights 1e-5.  From the
    # reference's default all-ones start the first steps need 9, 7, 6, 5
    # trials and summation order alone moves the oracle's own result by up
    # to 4.8e-6 (loss) / 4.5e-5 (weights) between rank splits, so that run is
    # held to the same trial sequence and a loss within 2e-5.
    from frovedis_gb300 import datagen
    spec = datagen.logreg_100k_20k()
    off, idx, val, label = datagen.generate(spec)
    a = oracle.CRS(spec.m, spec.n, off, idx, val)
    A = ctx.matrix(spec.m, spec.n, off, idx, val)
    kw = dict(num_iter=20, reg_type="L2", reg_param=1e-3)
    kz = dict(kw, w0=np.zeros(spec.n))
    r = fv.logreg_lbfgs(A, label, trace=True, **kz)
    ro = oracle.logreg_lbfgs(a, label, nthreads=8, **kz)
    assert r["n_iter"] == ro["n_iter"] == 20
    assert np.array_equal(r["trace"][:, 1], ro["trace"][:, 1])
    assert abs(r["loss"] - ro["loss"]) <= 1e-6 * abs(ro["loss"])
    assert np.max(np.abs(r["w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    for storage in ("f32", "bf16"):
        rs = fv.logreg_lbfgs(A, label, storage=storage, **kz)
        assert abs(rs["loss"] - ro["loss"]) <= 1e-3 * abs(ro["loss"]), storage
    r1 = fv.logreg_lbfgs(A, label, trace=True, **kw)
    ro1 = oracle.logreg_lbfgs(a, label, nthreads=8, **kw)
    assert r1["n_iter"] == ro1["n_iter"] == 20
    assert np.array_equal(r1["trace"][:, 1], ro1["trace"][:, 1])
    assert abs(r1["loss"] - ro1["loss"]) <= 2e-5 * abs(ro1["loss"])
