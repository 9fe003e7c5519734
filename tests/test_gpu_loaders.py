"""GPU loaders of the reference's CRS files (text, libsvm, binary directory)
against the oracle restatement, which converts numbers with the C library's
strtoll / strtod / strtof exactly as the reference does.

Bar: bit-exact — row offsets, column ids, every value's bit pattern (FP64
and FP32), labels and the column count."""
import numpy as np
import pytest

import oracle
from _golden import crs_text, golden

fv = pytest.importorskip("frovedis_gb300")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fv.Context(0)
    yield c
    c.close()


def same_bits(a, b, as_float=False):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float32 if as_float else np.float64).astype(np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_tutorial_text_and_binary_files(ctx, tmp_path):
    g = golden()
    p = tmp_path / "data"
    p.write_text(g["tut_spmv"]["raw_text"])
    A = ctx.load_text(p)
    off, idx, val = A.get_crs()
    assert (A.m, A.n) == (g["tut_spmv"]["m"], g["tut_spmv"]["n"])
    assert off.tolist() == g["tut_spmv"]["off"] and idx.tolist() == g["tut_spmv"]["idx"]
    assert val.tolist() == g["tut_spmv"]["val"]
    assert A.spmv(np.ones(A.n)).tolist() == g["tut_spmv"]["expected_y_ones"]
    d = tmp_path / "data_binary"
    d.mkdir()
    rf = g["tut_binary"]["raw_files"]
    for k in ("nums", "type"):
        (d / k).write_text(rf[k])
    for k in ("val", "idx", "off"):
        (d / k).write_bytes(bytes.fromhex(rf[k]))
    B = ctx.load_binary(d)
    off, idx, val = B.get_crs()
    assert off.tolist() == g["tut_binary"]["off"] and idx.tolist() == g["tut_binary"]["idx"]
    toff, tidx, tval = B.get_transpose()
    assert crs_text(oracle.CRS(B.n, B.m, toff, tidx, tval)) == g["tut_binary"]["expected_transpose_text"]
    with pytest.raises(fv.FvgError, match="idx type mismatch"):
        ctx.load_binary(d, idx_type="int32_t")


def _number_tokens(rng, k):
    """Values in the forms a file may hold: shortest repr (up to 17 digits:
    past the exact fast path), fixed and exponent forms, integers, signs,
    subnormals, huge exponents, hex and inf."""
    out = []
    for _ in range(k):
        x = float(rng.standard_normal() * 10.0 ** rng.integers(-8, 9))
        f = rng.integers(0, 12)
        if f == 0: out.append(repr(x))
        elif f == 1: out.append("%.3e" % x)
        elif f == 2: out.append("%g" % x)
        elif f == 3: out.append(str(int(x * 100)))
        elif f == 4: out.append("%.6f" % x)
        elif f == 5: out.append("+%.4f" % abs(x))
        elif f == 6: out.append("%.5E" % x)
        elif f == 7: out.append("-.%d" % rng.integers(1, 1000))
        elif f == 8: out.append("%d." % rng.integers(0, 50))
        elif f == 9: out.append(["1e-320", "4.9e-324", "1.7976931348623157e308", "1e400", "-0"][rng.integers(0, 5)])
        elif f == 10: out.append(["0x1.8p1", "inf", "-INF", "nan", "0.1000000000000000055511151231257827"][rng.integers(0, 5)])
        else: out.append("%.17g" % x)
    return out


def _write_crs(path, rng, m, n, label=False, one_based=False, crlf=False, trailing_newline=True):
    lines = []
    for r in range(m):
        k = rng.integers(0, min(n, 12) + 1)
        cols = np.sort(rng.choice(n, k, replace=False)) + (1 if one_based else 0)
        toks = [f"{c}:{v}" for c, v in zip(cols, _number_tokens(rng, k))]
        sep = " " if rng.random() < 0.7 else "\t"
        line = sep.join(toks)
        if label:
            line = (str(rng.integers(0, 2) * 2 - 1) if rng.random() < 0.8 else repr(rng.random())) + " " + line
        if rng.random() < 0.2:
            line = "  " + line + "  "
        lines.append(line)
    nl = "\r\n" if crlf else "\n"
    text = nl.join(lines) + (nl if trailing_newline else "")
    path.write_bytes(text.encode())


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("variant", ["plain", "crlf", "no_trailing_newline"])
def test_text_loader_bit_exact(ctx, tmp_path, dtype, variant):
    rng = np.random.default_rng(["plain", "crlf", "no_trailing_newline"].index(variant) * 2 + (dtype == "f32"))
    p = tmp_path / "m.txt"
    _write_crs(p, rng, 400, 60, crlf=variant == "crlf", trailing_newline=variant != "no_trailing_newline")
    as_float = dtype == "f32"
    off, idx, val, m, n = oracle.load_text(str(p), as_float=as_float)
    A = ctx.load_text(p, dtype=dtype)
    goff, gidx, gval = A.get_crs()
    assert (A.m, A.n) == (m, n)
    assert np.array_equal(goff, off) and np.array_equal(gidx, idx)
    assert same_bits(gval, val, as_float)
    B = ctx.load_text(p, dtype=dtype, num_col=n + 7)  # explicit column count
    assert B.n == n + 7


@pytest.mark.parametrize("origin,one_based", [(0, True), (0, False), (1, False), (2, True)])
def test_libsvm_loader_bit_exact(ctx, tmp_path, origin, one_based):
    rng = np.random.default_rng(origin * 2 + one_based)
    p = tmp_path / "m.svm"
    _write_crs(p, rng, 300, 40, label=True, one_based=one_based)
    off, idx, val, m, n, lab = oracle.load_libsvm(str(p), origin=origin)
    A, glab = ctx.load_libsvm(p, index_origin=origin)
    goff, gidx, gval = A.get_crs()
    assert (A.m, A.n) == (m, n)
    assert np.array_equal(goff, off) and np.array_equal(gidx, idx)
    assert same_bits(gval, val) and same_bits(glab, lab)


def test_loader_edge_cases(ctx, tmp_path):
    p = tmp_path / "e.txt"
    p.write_bytes(b"")
    A = ctx.load_text(p)
    assert (A.m, A.n, A.nnz) == (0, 0, 0)
    p.write_bytes(b"\n\n3:1.5\n\n")  # empty rows around one entry
    off, idx, val, m, n = oracle.load_text(str(p))
    A = ctx.load_text(p)
    goff, gidx, gval = A.get_crs()
    assert (A.m, A.n) == (m, n) == (4, 4)
    assert np.array_equal(goff, off) and np.array_equal(gidx, idx) and same_bits(gval, val)


@pytest.mark.parametrize("text", [b"1:2.0 junk\n", b"1:2:3\n", b"a:1\n", b"1:\n", b"1:2.0x\n", b"1 :2\n"])
def test_loader_rejects_malformed_lines(ctx, tmp_path, text):
    p = tmp_path / "bad.txt"
    p.write_bytes(text)
    with pytest.raises(fv.FvgError):
        ctx.load_text(p)


def test_binary_loader_types(ctx, tmp_path):
    rng = np.random.default_rng(3)
    m, n = 200, 50
    lens = rng.integers(0, 9, m)
    off = np.concatenate([[0], np.cumsum(lens)])
    idx = np.concatenate([np.sort(rng.choice(n, k, replace=False)) for k in lens])
    val = rng.standard_normal(off[-1])
    for vt, it, ot, vdt in (("double", "int32_t", "uint64_t", "f64"), ("float", "uint64_t", "int64_t", "f32")):
        d = tmp_path / f"bin_{it}_{ot}"
        d.mkdir()
        (d / "nums").write_text(f"{m}\n{n}\n")
        (d / "type").write_text(f"{vt}\n{it}\n{ot}\n")
        np.asarray(val, dtype=np.float64 if vt == "double" else np.float32).tofile(d / "val")
        np.asarray(idx, dtype={"int32_t": np.int32, "uint64_t": np.uint64}[it]).tofile(d / "idx")
        np.asarray(off, dtype={"uint64_t": np.uint64, "int64_t": np.int64}[ot]).tofile(d / "off")
        A = ctx.load_binary(d, dtype=vdt, idx_type=it, off_type=ot)
        goff, gidx, gval = A.get_crs()
        assert np.array_equal(goff, off) and np.array_equal(gidx, idx)
        assert same_bits(gval, val.astype(np.float32) if vdt == "f32" else val, vdt == "f32")
        with pytest.raises(fv.FvgError, match="type mismatch"):
            ctx.load_binary(d, dtype="f64" if vdt == "f32" else "f32", idx_type=it, off_type=ot)
