"""GPU parity of the row-panel backward product (A^T r on FP32 / BF16 values).

The panel layout regroups the entries of frequent columns by stretches of
rows; it changes only the summation order of the transposed product, so it is
held to the same bar as the plain FP32 path: against the FP64 oracle on the
FP32- (BF16-) rounded values, within 2e-5 of each column's absolute sum, and
bit-identical from run to run.
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


def _zipf(m, n, lam=30.0, seed=3):
    from frovedis_gb300 import datagen
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=lam, seed=seed))
    return oracle.CRS(m, n, off, idx, val), label


def _rounded(a, storage):
    # the device rounds FP64 values straight to FP32 / BF16 (nearest even);
    # rounding to BF16 through FP32 would round twice and differ on ties
    if storage == "f32":
        v = a.val.astype(np.float32).astype(np.float64)
    else:
        d = np.ascontiguousarray(a.val, dtype=np.float64).view(np.uint64)
        keep = np.uint64(45)  # 52 - 7 mantissa bits (normal range)
        d = ((d + ((d >> keep) & np.uint64(1)) + np.uint64((1 << 44) - 1)) >> keep) << keep
        v = d.view(np.float64)
    return oracle.CRS(a.m, a.n, a.off, a.idx, v)


def _colabs(a, r):
    return oracle.spmv(oracle.transpose(oracle.CRS(a.m, a.n, a.off, a.idx, np.abs(a.val))), np.abs(r))


def _check_trans_mv(A, a, rng, storage, vec="f32"):
    r = rng.standard_normal(a.m).astype(np.float32)
    ref = oracle.spmv(oracle.transpose(_rounded(a, storage)), r.astype(np.float64))
    tol = 2e-5 * (_colabs(a, r.astype(np.float64)) + 1e-30)
    # FP64 vectors on FP32 values: r is the same FP32-representable vector
    got = A.trans_mv(r.astype(np.float64) if vec == "f64" else r, storage=storage, vec=vec).astype(np.float64)
    assert np.all(np.abs(got - ref) <= tol), (storage, vec, np.max(np.abs(got - ref) / (tol + 1e-300)))
    return got


@pytest.mark.parametrize("rows,mpp", [(512, 1.0), (1000, 2.0), (4, 0.5), (8192, 1.0)])
def test_panel_trans_mv_matches_oracle(ctx, rows, mpp):
    # 20,000 x 3,000 Zipf(1.1) columns: hot columns by the hundred, a long cold
    # tail; 1000 does not divide the rows (ragged last panel); 4-row panels put
    # every hot column's entries in thousands of one- or two-entry segments
    a, _ = _zipf(20000, 3000)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.set_panels(rows, mpp)
    info = A.panel_info()
    assert info[0] == rows and info[1] == (a.m + rows - 1) // rows
    assert info[2] > 0 and 0 < info[3] <= a.off[-1]
    rng = np.random.default_rng(rows)
    for storage in ("f32", "bf16"):
        _check_trans_mv(A, a, rng, storage)
    # FP64 vectors take the FP32-vector kernels' output path (FP64 result)
    _check_trans_mv(A, a, rng, "f32", vec="f64")


def test_panel_split_hot_and_cold(ctx):
    # min_per_panel between the column counts splits the columns: both parts
    # contribute and the result matches the plain transposed product
    a, _ = _zipf(30000, 5000, seed=5)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    counts = np.bincount(a.idx, minlength=a.n)
    A.set_panels(1024, 3.0)
    rows, npan, nhot, E = A.panel_info()
    thresh = int(np.ceil(3.0 * npan))
    assert nhot == int(np.sum(counts >= thresh))
    assert E == int(np.sum(counts[counts >= thresh]))
    assert 0 < E < a.off[-1]
    rng = np.random.default_rng(1)
    got = _check_trans_mv(A, a, rng, "f32")
    A.set_panels(0)
    assert A.panel_info()[0] == 0
    r = rng.standard_normal(a.m).astype(np.float32)
    A.set_panels(1024, 3.0)
    p1 = A.trans_mv(r, storage="f32", vec="f32").astype(np.float64)
    A.set_panels(0)
    p0 = A.trans_mv(r, storage="f32", vec="f32").astype(np.float64)
    tol = 2e-5 * (_colabs(a, r.astype(np.float64)) + 1e-30)
    assert np.all(np.abs(p1 - p0) <= 2 * tol)
    assert got.shape == (a.n,)


def test_panel_long_segments(ctx):
    # column 0 in every row and column 1 in every other row: their segments in a
    # 4096-row panel hold 4096 and 2048 entries, split into pieces that the CTA
    # adds in order after its barrier; an empty panel stretch (rows without
    # entries) and a column with no entries at all
    rng = np.random.default_rng(7)
    m, n = 20000, 600
    rows = []
    for i in range(m):
        if 8000 <= i < 9000:
            rows.append(np.zeros(0, np.int64))
            continue
        extra = rng.choice(np.arange(2, n - 1), rng.integers(0, 12), replace=False)
        base = [0] + ([1] if i % 2 == 0 else [])
        rows.append(np.sort(np.concatenate([base, extra])))
    off = np.concatenate([[0], np.cumsum([len(x) for x in rows])]).astype(np.int32)
    idx = np.concatenate(rows).astype(np.int32)
    val = rng.standard_normal(int(off[-1]))
    a = oracle.CRS(m, n, off, idx, val)
    A = ctx.matrix(m, n, off, idx, val)
    A.set_panels(4096, 1.0)
    info = A.panel_info()
    assert info[2] >= 2
    for storage in ("f32", "bf16"):
        got = _check_trans_mv(A, a, rng, storage)
        assert got[n - 1] == 0.0


def test_panel_deterministic(ctx):
    a, _ = _zipf(25000, 2000, seed=11)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.set_panels(256, 1.0)
    r = np.random.default_rng(2).standard_normal(a.m).astype(np.float32)
    y0 = A.trans_mv(r, storage="bf16", vec="f32")
    for _ in range(3):
        assert np.array_equal(A.trans_mv(r, storage="bf16", vec="f32"), y0)


def test_panel_bad_rows(ctx):
    a, _ = _zipf(2000, 300)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    with pytest.raises(fv.FvgError):
        A.set_panels(6)  # not a multiple of 4
    A.set_panels(1 << 20)  # more than shared memory holds: refused when the layout is built
    with pytest.raises(fv.FvgError):
        A.trans_mv(np.ones(a.m, np.float32), storage="f32", vec="f32")


def test_panel_unaligned_device_vector(ctx):
    # a device r that is not 16-byte aligned is staged element by element
    torch = pytest.importorskip("torch")
    a, _ = _zipf(20000, 3000, seed=4)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.set_panels(512, 1.0)
    rng = np.random.default_rng(5)
    r = rng.standard_normal(a.m).astype(np.float32)
    buf = torch.zeros(a.m + 1, dtype=torch.float32, device="cuda")
    buf[1:] = torch.from_numpy(r).cuda()
    y = torch.zeros(a.n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    A.trans_mv_device(buf.data_ptr() + 4, y.data_ptr(), storage="f32", vec="f32")
    got = y.cpu().numpy().astype(np.float64)
    ref = oracle.spmv(oracle.transpose(_rounded(a, "f32")), r.astype(np.float64))
    assert np.all(np.abs(got - ref) <= 2e-5 * (_colabs(a, r.astype(np.float64)) + 1e-30))


@pytest.mark.parametrize("storage", ["f32", "bf16"])
def test_panel_eval_matches_fp64(ctx, storage):
    # the fused evaluation with the panel backward pass: loss and gradient
    # against FP64 arithmetic on the same rounded values
    a, label = _zipf(24000, 1500, seed=8)
    ar = _rounded(a, storage)
    B = ctx.matrix(a.m, a.n, ar.off, ar.idx, ar.val)
    rng = np.random.default_rng(9)
    w = rng.standard_normal(a.n) * 0.2
    g64, l64 = fv.logreg_eval(B, label, w, b=0.3, intercept=True)
    B.set_panels(512, 1.0)
    assert B.panel_info()[2] > 0
    g, loss = fv.logreg_eval(B, label, w, b=0.3, intercept=True, storage=storage)
    scale = oracle.spmv(oracle.transpose(oracle.CRS(a.m, a.n, a.off, a.idx, np.abs(ar.val))), np.ones(a.m))
    assert abs(loss - l64) <= 1e-5 * abs(l64)
    assert np.max(np.abs(g[:-1] - g64[:-1]) / (scale + 1.0)) <= 1e-5
    assert abs(g[-1] - g64[-1]) <= 1e-5 * a.m


def test_panel_lbfgs_close_to_oracle(ctx):
    a, label = _zipf(40000, 2000, seed=12)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=20, reg_type="L2", reg_param=1e-3, w0=np.zeros(a.n))
    ro = oracle.logreg_lbfgs(a, label, nthreads=8, **kw)
    A.set_panels(1024, 1.0)
    for storage in ("f32", "bf16"):
        r = fv.logreg_lbfgs(A, label, storage=storage, **kw)
        assert abs(r["loss"] - ro["loss"]) <= 1e-3 * abs(ro["loss"]), storage
    assert A.panel_info()[2] > 0


# ------------------------------------------------------------ forward head
def _eval_check(A, a_rounded, label, storage, rng, sw=None):
    """FP32/BF16 evaluation against FP64 arithmetic on the same rounded values."""
    B = A
    w = rng.standard_normal(a_rounded.n) * 0.2
    g, loss = fv.logreg_eval(B, label, w, b=0.3, intercept=True, storage=storage, sample_weight=sw)
    g64, l64 = oracle.logreg_eval(a_rounded, label, w, b=0.3, intercept=True, sw=sw)
    absa = oracle.CRS(a_rounded.m, a_rounded.n, a_rounded.off, a_rounded.idx, np.abs(a_rounded.val))
    scale = oracle.spmv(oracle.transpose(absa), np.ones(a_rounded.m))
    assert abs(loss - l64) <= 1e-5 * abs(l64), (storage, loss, l64)
    assert np.max(np.abs(g[:-1] - g64[:-1]) / (scale + 1.0)) <= 1e-5, storage
    assert abs(g[-1] - g64[-1]) <= 1e-5 * a_rounded.m, storage


@pytest.mark.parametrize("storage", ["f32", "bf16"])
@pytest.mark.parametrize("head,panels", [(64, 0), (700, 512), (1500, 0)])
def test_head_eval_matches_fp64(ctx, storage, head, panels):
    # the forward head (the most frequent columns from shared memory, the rest
    # of each row through the CRS pass whose epilogue adds both); 1500 = every
    # column: the tail holds no entries and its pass only applies the epilogue
    a, label = _zipf(24000, 1500, seed=21)
    ar = _rounded(a, storage)
    B = ctx.matrix(a.m, a.n, ar.off, ar.idx, ar.val)
    B.set_head(head)
    B.set_panels(panels, 1.0)
    cols, ent = B.head_info()
    counts = np.bincount(a.idx, minlength=a.n)
    assert cols == head
    assert ent == int(np.sort(counts)[::-1][:head].sum())
    _eval_check(B, ar, label, storage, np.random.default_rng(head), sw=np.random.default_rng(3).uniform(0.5, 2, a.m))


def test_head_long_rows_and_empty_rows(ctx):
    # rows with more than 512 head entries are summed in pieces (added in
    # order after the CTA's barrier); empty rows and rows without tail entries
    rng = np.random.default_rng(22)
    m, n = 9000, 3000
    rows = []
    for i in range(m):
        if i % 97 == 0:
            rows.append(np.zeros(0, np.int64))
        elif i % 1000 == 5:
            rows.append(np.sort(rng.choice(n, 2600, replace=False)))
        else:
            k = rng.integers(1, 40)
            rows.append(np.sort(rng.choice(n, k, replace=False, p=None)))
    off = np.concatenate([[0], np.cumsum([len(x) for x in rows])]).astype(np.int32)
    idx = np.concatenate(rows).astype(np.int32)
    val = np.abs(rng.standard_normal(int(off[-1])))
    ar = _rounded(oracle.CRS(m, n, off, idx, val), "f32")
    label = np.where(rng.random(m) < 0.5, 1.0, -1.0)
    B = ctx.matrix(m, n, ar.off, ar.idx, ar.val)
    B.set_head(2048)
    assert B.head_info()[0] == 2048
    _eval_check(B, ar, label, "f32", rng)


def test_head_deterministic_and_errors(ctx):
    a, label = _zipf(20000, 2000, seed=23)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    A.set_head(300)
    w = np.random.default_rng(1).standard_normal(a.n) * 0.1
    g0, l0 = fv.logreg_eval(A, label, w, storage="bf16")
    for _ in range(3):
        g, l = fv.logreg_eval(A, label, w, storage="bf16")
        assert np.array_equal(g, g0) and l == l0
    A.set_head(1 << 20)  # more columns than shared memory holds: refused when the head is built
    with pytest.raises(fv.FvgError):
        fv.logreg_eval(A, label, w, storage="f32")
    A.set_head(0)
    assert A.head_info() == (0, 0)


def test_head_lbfgs_close_to_oracle(ctx):
    a, label = _zipf(40000, 2000, seed=24)
    A = ctx.matrix(a.m, a.n, a.off, a.idx, a.val)
    kw = dict(num_iter=20, reg_type="L2", reg_param=1e-3, w0=np.zeros(a.n))
    ro = oracle.logreg_lbfgs(a, label, nthreads=8, **kw)
    A.set_head(500)
    A.set_panels(1024, 1.0)
    for storage in ("f32", "bf16"):
        r = fv.logreg_lbfgs(A, label, storage=storage, **kw)
        assert abs(r["loss"] - ro["loss"]) <= 1e-3 * abs(ro["loss"]), storage
    assert A.head_info()[0] == 500


@pytest.mark.parametrize("master", ["f32", "bf16"])
def test_panels_and_head_on_lower_precision_uploads(ctx, master):
    # matrices uploaded with FP32 or BF16 values: the panel, cold, head and tail
    # copies are filled from that plane (their FP32 plane converted from BF16)
    a, label = _zipf(24000, 1500, seed=31)
    ar = _rounded(a, master)
    if master == "f32":
        vals = ar.val.astype(np.float32)
    else:
        vals = (ar.val.astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
    B = ctx.matrix(a.m, a.n, ar.off, ar.idx, vals)
    B.set_panels(512, 1.0)
    B.set_head(300)
    rng = np.random.default_rng(32)
    storages = ("f32",) if master == "f32" else ("bf16", "f32")
    for storage in storages:
        r = rng.standard_normal(a.m).astype(np.float32)
        ref = oracle.spmv(oracle.transpose(ar), r.astype(np.float64))
        got = B.trans_mv(r, storage=storage, vec="f32").astype(np.float64)
        assert np.all(np.abs(got - ref) <= 2e-5 * (_colabs(ar, r.astype(np.float64)) + 1e-30)), storage
        _eval_check(B, ar, label, storage, rng)
    assert B.panel_info()[2] > 0 and B.head_info()[0] == 300
