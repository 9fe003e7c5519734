"""The C++ API (include/frovedis_gb300.hpp): a program written against the
reference's class and function names (tests/cpp/api_check.cpp) compiles,
links against libfvg.so, and on a GPU gives the oracle's results.

Tolerances as in test_gpu_parity: layouts bit for bit, FP64 products rel
1e-12, FP32 products rel 2e-5, trained models rel 1e-6 (loss) / 1e-5
(weights); the L-BFGS iteration count must match exactly."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from frovedis_gb300 import build as fb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "api_check.cpp")


def compile_check(out_dir):
    lib = fb.build()
    exe = os.path.join(str(out_dir), "api_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-o", exe, "-L", os.path.dirname(lib), "-lfvg", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_api_compiles_and_links(tmp_path):
    assert os.access(compile_check(tmp_path), os.X_OK)


def _write_input(path, a, x, label):
    with open(path, "w") as f:
        f.write(f"{a.m} {a.n} {a.nnz}\n")
        for arr in (a.off, a.idx):
            f.write(" ".join(str(int(v)) for v in arr) + "\n")
        for arr in (a.val, x, label):
            f.write(" ".join(repr(float(v)) for v in arr) + "\n")


def _read_output(path):
    out = {}
    for line in open(path):
        parts = line.split()
        out[parts[0]] = np.array([float(v) for v in parts[1:]])
    return out


def close(a, b, rtol):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    return np.max(np.abs(a - b) / (np.abs(b) + 1.0)) <= rtol if a.size else True


@pytest.mark.gpu
def test_cpp_api_matches_oracle(tmp_path):
    from frovedis_gb300 import datagen
    m, n = 4000, 300
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=15.0, seed=4))
    a = oracle.CRS(m, n, off, idx, val)
    x = np.random.default_rng(9).standard_normal(n)
    inp, outp = tmp_path / "in.txt", tmp_path / "out.txt"
    _write_input(inp, a, x, label)
    exe = compile_check(tmp_path)
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    o = _read_output(outp)

    assert close(o["crs_mv"], oracle.spmv(a, x), 1e-12)
    t = oracle.transpose(a)
    assert np.array_equal(o["t_off"], t.off) and np.array_equal(o["t_idx"], t.idx)
    assert np.array_equal(o["t_val"], t.val)
    assert list(o["t_shape"]) == [n, m]
    w, _, _ = oracle.ell_build(a)
    assert int(o["ell_width"][0]) == w
    assert close(o["ell_mv"], oracle.ell_spmv(a, x), 1e-12)
    assert close(o["ell_trans"], oracle.ell_trans_mv(a, label), 1e-12)
    perm, joff, _, _ = oracle.jds_build(a)
    assert np.array_equal(o["jds_perm"], perm) and np.array_equal(o["jds_off"], joff)
    assert close(o["jds_mv"], oracle.jds_spmv(a, x), 1e-12)
    assert close(o["hyb_mv"], oracle.hyb_spmv(a, x), 1e-12)
    assert int(o["hyb_crs_rows"][0]) == oracle.hyb_build(a)["crs_rows"]
    X = x[:, None] * np.arange(1, 4)[None, :] + np.arange(3)[None, :]
    assert close(o["spmm"], oracle.spmm(a, X).ravel(), 1e-12)
    assert close(o["crs_mv_f32"], oracle.spmv_f32(a, x.astype(np.float32)), 2e-5)
    assert o["mismatch_throws"][0] == 1

    ro = oracle.logreg_lbfgs(a, label, num_iter=20, reg_type="L2", reg_param=1e-3, intercept=True)
    assert int(o["lbfgs_n_iter"][0]) == ro["n_iter"]
    assert np.max(np.abs(o["lbfgs_w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    assert abs(o["lbfgs_b"][0] - ro["b"]) <= 1e-5 * max(1.0, abs(ro["b"]))
    pb = oracle.predict_probability(a, ro["w"], ro["b"])
    assert np.max(np.abs(o["lbfgs_prob"] - pb)) <= 1e-6
    agree = np.mean(o["lbfgs_pred"] == np.where(pb >= 0.5, 1.0, -1.0))
    assert agree >= 0.999
    rh = oracle.logreg_lbfgs(a, label, num_iter=20, reg_type="ZERO", reg_param=1e-3, intercept=True, fmt="HYBRID")
    assert np.max(np.abs(o["lbfgs_hyb_w"] - rh["w"])) <= 1e-5 * max(1.0, np.max(np.abs(rh["w"])))
    assert abs(o["lbfgs_hyb_b"][0] - rh["b"]) <= 1e-5 * max(1.0, abs(rh["b"]))
    assert o["lbfgs_jds_throws"][0] == 1
    rs = oracle.logreg_sgd(a, label, num_iter=15, alpha=0.05, mini_batch_fraction=0.3, reg_type="L2",
                           reg_param=1e-2, intercept=True, b0=1.0)
    assert int(o["sgd_n_iter"][0]) == rs["n_iter"]
    assert np.max(np.abs(o["sgd_w"] - rs["w"])) <= 1e-5 * max(1.0, np.max(np.abs(rs["w"])))
    assert abs(o["sgd_b"][0] - rs["b"]) <= 1e-5 * max(1.0, abs(rs["b"]))

    cls = (np.arange(m) % 5).astype(np.float64)
    rm = oracle.softmax_train(a, cls, 5, num_iter=12, alpha=0.05, reg_param=1e-3, reg_type="L2", tol=0.0)
    assert int(o["mlr_n_iter"][0]) == rm["n_iter"]
    W = o["mlr_w"].reshape(n, 5)
    # 12 unnormalised gradient steps grow |W| to ~25: rounding differences
    # of the summation order reach ~1e-9 of that
    assert np.max(np.abs(W - rm["W"])) <= 1e-8 * max(1.0, np.max(np.abs(rm["W"])))
    P = oracle.softmax_probability(a, rm["W"], rm["b"])
    assert np.max(np.abs(o["mlr_prob"].reshape(m, 5) - P)) <= 1e-7
    assert np.mean(o["mlr_pred"] == np.argmax(P, 1)) >= 0.999
    assert np.max(np.abs(o["mlr_maxprob"] - P.max(1))) <= 1e-7

    # save (operator<< with the stream's default 6 significant digits) and
    # reload: the text loader gives what the oracle's strtod gives
    toff, tidx, tval, tm, tn = oracle.load_text(str(outp) + ".dir.txt")
    assert np.array_equal(o["load_text_off"], toff) and np.array_equal(o["load_text_idx"], tidx)
    assert np.array_equal(o["load_text_val"], tval)
    assert np.array_equal(o["load_bin_val"], a.val) and list(o["load_bin_shape"]) == [m, n]
    soff, sidx, sval, sm, sn, slab = oracle.load_libsvm(str(outp) + ".dir.svm")
    assert np.array_equal(o["load_svm_idx"], sidx) and np.array_equal(o["load_svm_label"], slab)
    assert list(o["load_svm_shape"]) == [sm, sn]

    # estimator (logistic_regression::_fit): the lbfgs solver is
    # logistic_regression_with_lbfgs::train from w = 1, b = 1
    re = oracle.logreg_lbfgs(a, label, num_iter=30, reg_type="L2", reg_param=1e-3, intercept=True)
    assert int(o["est_n_iter"][0]) == re["n_iter"]
    assert np.max(np.abs(o["est_w"] - re["w"])) <= 1e-5 * max(1.0, np.max(np.abs(re["w"])))
    pe = np.where(oracle.predict_probability(a, o["est_w"], o["est_b"][0]) >= 0.5, 1.0, -1.0)
    assert abs(o["est_score"][0] - np.mean(pe == label)) <= 1e-6
    assert np.max(np.abs(o["est_text_w"] - o["est_w"])) <= 1e-11 * max(1.0, np.max(np.abs(o["est_w"])))
    assert np.array_equal(o["est_bin_w"], o["est_w"]) and o["est_pred_same"][0] == 1
    assert o["estm_is_mult"][0] == 1
    rm2 = oracle.softmax_train(a, cls, 5, num_iter=10, alpha=0.05, reg_param=0.01, reg_type="ZERO")
    assert int(o["estm_n_iter"][0]) == rm2["n_iter"]
    assert np.max(np.abs(o["estm_w"] - rm2["W"].ravel())) <= 1e-8 * max(1.0, np.max(np.abs(rm2["W"])))
    assert np.array_equal(o["estm_bin_w"], o["estm_w"]) and o["estm_pred_same"][0] == 1
    assert o["estm_text_classes"][0] == 5 and o["estm_lbfgs_throws"][0] == 1

    # the GLM family: initial intercept 0 for SGD, isIntercept for L-BFGS
    y = o["reg_y"]

    def wclose(got, ref):
        return np.max(np.abs(got - ref)) <= 1e-5 * max(1.0, np.max(np.abs(ref)))
    r = oracle.logreg_sgd(a, y, loss="linear", num_iter=20, alpha=1e-4, mini_batch_fraction=0.3, reg_type="ZERO",
                          intercept=True, tol=0.0)
    assert wclose(o["lin_sgd_w"], r["w"]) and abs(o["lin_sgd_b"][0] - r["b"]) <= 1e-5 * max(1.0, abs(r["b"]))
    assert int(o["lin_sgd_n_iter"][0]) == r["n_iter"] == 20
    assert np.max(np.abs(o["lin_pred"] - (a.to_dense() @ o["lin_sgd_w"] + o["lin_sgd_b"][0]))) <= 1e-9
    r = oracle.logreg_lbfgs(a, y, loss="linear", num_iter=25, hist_size=10, reg_type="ZERO", intercept=True)
    assert wclose(o["lin_lbfgs_w"], r["w"]) and int(o["lin_lbfgs_n_iter"][0]) == r["n_iter"]
    r = oracle.logreg_sgd(a, y, loss="linear", num_iter=20, alpha=1e-4, reg_type="L1", reg_param=1e-3, tol=0.0)
    assert wclose(o["lasso_sgd_w"], r["w"])
    r = oracle.logreg_lbfgs(a, y, loss="linear", num_iter=25, reg_type="L2", reg_param=1e-2, intercept=True)
    assert wclose(o["ridge_lbfgs_w"], r["w"])
    r = oracle.logreg_sgd(a, label, loss="hinge", num_iter=30, alpha=0.05, reg_type="L2", reg_param=1e-2,
                          intercept=True, tol=0.0)
    assert wclose(o["svm_sgd_w"], r["w"])
    score = a.to_dense() @ o["svm_sgd_w"] + o["svm_sgd_b"][0]
    assert np.max(np.abs(o["svm_score"] - score)) <= 1e-9
    assert np.array_equal(o["svm_pred"], np.where(o["svm_score"] > 0, 1.0, -1.0))
    r = oracle.logreg_lbfgs(a, label, loss="hinge", num_iter=25, reg_type="L1", reg_param=1e-2, intercept=True)
    assert wclose(o["svm_lbfgs_w"], r["w"]) and int(o["svm_lbfgs_n_iter"][0]) == r["n_iter"]
    r = oracle.logreg_sgd(a, y, loss="eps", eps=0.1, num_iter=20, alpha=0.01, reg_type="ZERO", intercept=True,
                          tol=0.0)
    assert wclose(o["svr_eps_w"], r["w"])
    r = oracle.logreg_sgd(a, y, loss="sqeps", eps=0.05, num_iter=20, alpha=1e-4, reg_type="L2", reg_param=1e-3,
                          tol=0.0)
    assert wclose(o["svr_sqeps_w"], r["w"])
    assert o["svm_jds_throws"][0] == 1
    assert np.max(np.abs(o["lin_loaded_w"] - o["lin_sgd_w"])) <= 1e-11 * max(1.0, np.max(np.abs(o["lin_sgd_w"])))
    assert o["svm_loaded_same"][0] == 1

    rs = oracle.logreg_sgd(a, label, shrink=True, num_iter=15, alpha=0.05, mini_batch_fraction=0.3, reg_type="L2",
                           reg_param=1e-2, intercept=True, tol=0.0)
    assert wclose(o["shrink_w"], rs["w"]) and abs(o["shrink_b"][0] - rs["b"]) <= 1e-5 * max(1.0, abs(rs["b"]))
    assert int(o["shrink_n_iter"][0]) == rs["n_iter"] == 15
    # estimator: initial model (w = 1, b = fit_intercept) as logistic_regression::_fit builds it
    rs = oracle.logreg_sgd(a, label, shrink=True, num_iter=12, alpha=0.05, reg_type="L1", reg_param=1e-3,
                           intercept=True, b0=1.0)
    assert wclose(o["est_shrink_w"], rs["w"]) and int(o["est_shrink_n_iter"][0]) == rs["n_iter"]


# ---------------------------------------------------------------------------
# The distributed containers (crs_matrix / dvector on one rank) and the
# INTEGRATION.md binding: its C++ block is pasted into tests/cpp/dist_check.cpp
# verbatim, where it specialises logistic_regression_with_lbfgs::train for
# crs_matrix<double,int,int>.
DIST_SRC = os.path.join(ROOT, "tests", "cpp", "dist_check.cpp")


def integration_binding():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text.index("## The binding a frovedis maintainer would add (C++)")
    start = text.index("```cpp\n", sec) + len("```cpp\n")
    return text[start:text.index("```", start)]


def compile_dist(out_dir):
    lib = fb.build()
    src = os.path.join(str(out_dir), "dist_check.cpp")
    code = open(DIST_SRC).read()
    assert "// @@BINDING@@" in code
    with open(src, "w") as f:
        f.write(code.replace("// @@BINDING@@", integration_binding()))
    exe = os.path.join(str(out_dir), "dist_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), src,
           "-o", exe, "-L", os.path.dirname(lib), "-lfvg", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_integration_binding_compiles(tmp_path):
    assert "logistic_regression_with_lbfgs::train(crs_matrix<double,int,int>& data" in integration_binding()
    assert os.access(compile_dist(tmp_path), os.X_OK)


@pytest.mark.gpu
def test_distributed_overloads_and_binding_match_oracle(tmp_path):
    from frovedis_gb300 import datagen
    m, n = 3000, 250
    off, idx, val, label = datagen.generate(datagen.Spec(m=m, n=n, lam=12.0, seed=6))
    a = oracle.CRS(m, n, off, idx, val)
    inp, outp = tmp_path / "in.txt", tmp_path / "out.txt"
    with open(inp, "w") as f:
        f.write(f"{m} {n} {a.nnz}\n")
        for arr in (a.off, a.idx):
            f.write(" ".join(str(int(v)) for v in arr) + "\n")
        for arr in (a.val, label):
            f.write(" ".join(repr(float(v)) for v in arr) + "\n")
    exe = compile_dist(tmp_path)
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    o = _read_output(outp)
    kw = dict(num_iter=15, reg_type="L2", reg_param=1e-3)
    ro = oracle.logreg_lbfgs(a, label, w0=np.zeros(n), **kw)
    # the binding and the library's own overload make the same call
    assert np.array_equal(o["binding_w"], o["own_w"])
    assert int(o["binding_iter"][0]) == int(o["own_iter"][0]) == ro["n_iter"]
    assert np.max(np.abs(o["binding_w"] - ro["w"])) <= 1e-5 * max(1.0, np.max(np.abs(ro["w"])))
    rd = oracle.logreg_lbfgs(a, label, intercept=True, **kw)
    assert np.max(np.abs(o["defaults_w"] - rd["w"])) <= 1e-5 * max(1.0, np.max(np.abs(rd["w"])))
    assert abs(o["defaults_b"][0] - rd["b"]) <= 1e-5 * max(1.0, abs(rd["b"]))
    assert np.array_equal(o["moved_w"], o["defaults_w"]) and o["moved_cleared"][0] == 1
    rs = oracle.logreg_sgd(a, label, num_iter=10, alpha=0.05, reg_type="L2", reg_param=1e-2, intercept=True)
    assert np.max(np.abs(o["sgd_w"] - rs["w"])) <= 1e-5 * max(1.0, np.max(np.abs(rs["w"])))
    assert abs(o["sgd_b"][0] - rs["b"]) <= 1e-5 * max(1.0, abs(rs["b"]))
