"""CPU oracle — test infrastructure only.

ctypes bindings to ``oracle/_build/liboracle.so``, the plain C++ restatement
of the reference's sparse logistic-regression path (``oracle.cpp``).  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this package; the product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

FMT = {"CRS": 0, "JDS": 1, "ELL": 2, "HYBRID": 3}
REG = {"ZERO": 0, "L1": 1, "L2": 2}
# GLM loss kinds (ml/glm/gradient.hpp): logistic_gradient, linear_gradient,
# hinge_gradient, epsilon_insensitive, squared_epsilon_insensitive.
LOSS = {"logistic": 0, "linear": 1, "hinge": 2, "eps": 3, "sqeps": 4}

_i64 = C.c_int64
_int = C.c_int
_dbl = C.c_double
_p = C.c_void_p


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (g++ only)."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "oracle.cpp")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        L = _lib
        sig = {
            "orc_crs_spmv_f64": [_i64, _i64, _p, _p, _p, _p, _p],
            "orc_crs_spmv_f32": [_i64, _i64, _p, _p, _p, _p, _p],
            "orc_crs_transpose_f64": [_i64, _i64, _p, _p, _p, _p, _p, _p],
            "orc_crs_spmm_f64": [_i64, _i64, _p, _p, _p, _p, _i64, _p],
            "orc_ell_build_f64": [_i64, _i64, _p, _p, _p, _p, _p],
            "orc_ell_spmv_f64": [_i64, _i64, _i64, _p, _p, _p, _p],
            "orc_ell_trans_mv_f64": [_i64, _i64, _i64, _p, _p, _p, _p],
            "orc_jds_build_f64": [_i64, _i64, _p, _p, _p, _p, _p, _p, _p, _p],
            "orc_jds_spmv_f64": [_i64, _i64, _p, _p, _p, _p, _p],
            "orc_hyb_info": [_i64, _i64, _p, _p, _p, _i64, _p],
            "orc_hyb_build_f64": [_i64, _i64, _p, _p, _p, _i64, _p, _p, _p, _p, _p, _p, _p],
            "orc_hyb_spmv_f64": [_i64, _i64, _p, _p, _p, _i64, _p, _p],
            "orc_fmt_mv_f64": [_int, _int, _i64, _i64, _p, _p, _p, _p, _p],
            "orc_glm_dloss_f64": [_int, _dbl, _i64, _p, _p, _p, _p],
            "orc_glm_eval_f64": [_int, _i64, _i64, _p, _p, _p, _p, _p, _p, _dbl, _int, _p, _int, _int,
                                 _p, _p, _int, _dbl],
            "orc_glm_lbfgs_f64": [_int, _i64, _i64, _p, _p, _p, _p, _p, _p, _int, _int, _i64, _i64, _dbl,
                                  _int, _int, _dbl, _p, _p, _p, _p, _p, _int, _int, _dbl],
            "orc_glm_sgd_f64": [_int, _i64, _i64, _p, _p, _p, _p, _p, _p, _int, _int, _i64, _dbl, _dbl,
                                _dbl, _int, _int, _dbl, _p, _p, _p, _p, _int, _int, _dbl],
            "orc_predict_probability_f64": [_i64, _i64, _p, _p, _p, _p, _dbl, _p],
            "orc_softmax_train_f64": [_i64, _i64, _p, _p, _p, _p, _p, _i64, _i64, _dbl, _dbl, _int, _int, _dbl,
                                      _p, _p, _p],
            "orc_softmax_probability_f64": [_i64, _i64, _p, _p, _p, _p, _p, _i64, _int, _p],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = None
        L.orc_problem_create.argtypes = [_int, _i64, _i64, _p, _p, _p, _p, _p, _p, _int, _int, _int, _dbl]
        L.orc_problem_create.restype = _p
        L.orc_problem_lbfgs.argtypes = [_p, _i64, _i64, _dbl, _int, _int, _dbl, _p, _p, _p, _p, _p, _int]
        L.orc_problem_lbfgs.restype = _int
        L.orc_problem_destroy.argtypes = [_p]
        L.orc_problem_destroy.restype = None
        L.orc_softmax_lbfgs_f64.argtypes = [_i64, _i64, _p, _p, _p, _p, _p, _i64, _i64, _i64, _dbl, _int, _dbl,
                                            _p, _p, _p, _p]
        L.orc_softmax_lbfgs_f64.restype = _int
        L.orc_ell_width.argtypes = [_i64, _p]
        L.orc_ell_width.restype = _i64
        L.orc_glm_lbfgs_f64.restype = _int
        L.orc_glm_sgd_f64.restype = _int
        L.orc_softmax_train_f64.restype = _int
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_p)


class CRS:
    """Host CRS matrix (int32 off/idx, float64 values) handed to the oracle."""

    def __init__(self, m, n, off, idx, val):
        self.m, self.n = int(m), int(n)
        self.off = np.ascontiguousarray(off, dtype=np.int32)
        self.idx = np.ascontiguousarray(idx, dtype=np.int32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        assert self.off.shape[0] == self.m + 1

    @property
    def nnz(self):
        return int(self.off[-1])

    def args(self):
        return (self.m, self.n, _ptr(self.off), _ptr(self.idx), _ptr(self.val))

    def to_dense(self):
        d = np.zeros((self.m, self.n))
        for r in range(self.m):
            for p in range(self.off[r], self.off[r + 1]):
                d[r, self.idx[p]] += self.val[p]
        return d


def spmv(a: CRS, x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.m)
    lib().orc_crs_spmv_f64(*a.args(), _ptr(x), _ptr(y))
    return y


def spmv_f32(a: CRS, x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    v = a.val.astype(np.float32)
    y = np.zeros(a.m, dtype=np.float32)
    lib().orc_crs_spmv_f32(a.m, a.n, _ptr(a.off), _ptr(a.idx), _ptr(v), _ptr(x), _ptr(y))
    return y


def transpose(a: CRS) -> CRS:
    toff = np.zeros(a.n + 1, dtype=np.int32)
    tidx = np.zeros(a.nnz, dtype=np.int32)
    tval = np.zeros(a.nnz)
    lib().orc_crs_transpose_f64(*a.args(), _ptr(toff), _ptr(tidx), _ptr(tval))
    return CRS(a.n, a.m, toff, tidx, tval)


def spmm(a: CRS, X) -> np.ndarray:
    X = np.ascontiguousarray(X, dtype=np.float64)
    k = X.shape[1]
    Y = np.zeros((a.m, k))
    lib().orc_crs_spmm_f64(*a.args(), _ptr(X), k, _ptr(Y))
    return Y


def ell_build(a: CRS):
    w = lib().orc_ell_width(a.m, _ptr(a.off))
    eidx = np.zeros(a.m * w, dtype=np.int32)
    ev = np.zeros(a.m * w)
    lib().orc_ell_build_f64(*a.args(), _ptr(eidx), _ptr(ev))
    return w, eidx, ev


def ell_spmv(a: CRS, x) -> np.ndarray:
    w, eidx, ev = ell_build(a)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.m)
    lib().orc_ell_spmv_f64(a.m, a.n, w, _ptr(eidx), _ptr(ev), _ptr(x), _ptr(y))
    return y


def ell_trans_mv(a: CRS, v) -> np.ndarray:
    w, eidx, ev = ell_build(a)
    v = np.ascontiguousarray(v, dtype=np.float64)
    y = np.zeros(a.n)
    lib().orc_ell_trans_mv_f64(a.m, a.n, w, _ptr(eidx), _ptr(ev), _ptr(v), _ptr(y))
    return y


def jds_build(a: CRS):
    perm = np.zeros(a.m, dtype=np.int32)
    maxlen = int(np.max(np.diff(a.off))) if a.m else 0
    joff = np.zeros(maxlen + 2, dtype=np.int64)
    jidx = np.zeros(a.nnz, dtype=np.int32)
    jval = np.zeros(a.nnz)
    nd = np.zeros(1, dtype=np.int64)
    lib().orc_jds_build_f64(*a.args(), _ptr(perm), _ptr(joff), _ptr(jidx), _ptr(jval), _ptr(nd))
    nd = int(nd[0])
    return perm, joff[: nd + 1], jidx, jval


def jds_spmv(a: CRS, x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.m)
    lib().orc_jds_spmv_f64(*a.args(), _ptr(x), _ptr(y))
    return y


def hyb_build(a: CRS, thr: int = 256):
    info = np.zeros(5, dtype=np.int64)
    lib().orc_hyb_info(*a.args(), thr, _ptr(info))
    nd, crows, cnnz, jnnz, plen = (int(v) for v in info)
    perm = np.zeros(max(plen, 1), dtype=np.int32)
    joff = np.zeros(nd + 1, dtype=np.int64)
    jidx = np.zeros(max(jnnz, 1), dtype=np.int32)
    jval = np.zeros(max(jnnz, 1))
    coff = np.zeros(crows + 1, dtype=np.int64)
    cidx = np.zeros(max(cnnz, 1), dtype=np.int32)
    cval = np.zeros(max(cnnz, 1))
    lib().orc_hyb_build_f64(*a.args(), thr, _ptr(perm), _ptr(joff), _ptr(jidx), _ptr(jval), _ptr(coff),
                            _ptr(cidx), _ptr(cval))
    return dict(perm=perm[:plen], joff=joff, jidx=jidx[:jnnz], jval=jval[:jnnz], coff=coff,
                cidx=cidx[:cnnz], cval=cval[:cnnz], crs_rows=crows)


def hyb_spmv(a: CRS, x, thr: int = 256) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.m)
    lib().orc_hyb_spmv_f64(*a.args(), thr, _ptr(x), _ptr(y))
    return y


def fmt_mv(a: CRS, fmt: str, x, trans: bool = False) -> np.ndarray:
    """Forward (``A x``) or backward (``A^T x``) product as the glm path does it."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(a.n if trans else a.m)
    lib().orc_fmt_mv_f64(FMT[fmt], int(trans), *a.args(), _ptr(x), _ptr(y))
    return y


def glm_dloss(label, wtx, loss="logistic", eps=0.0):
    """``<kind>_gradient::compute_dloss`` on one vector: (dloss, sumloss)."""
    label = np.ascontiguousarray(label, dtype=np.float64)
    wtx = np.ascontiguousarray(wtx, dtype=np.float64)
    d = np.zeros(len(wtx))
    s = np.zeros(1)
    lib().orc_glm_dloss_f64(LOSS[loss], float(eps), len(wtx), _ptr(label), _ptr(wtx), _ptr(d), _ptr(s))
    return d, float(s[0])


def logistic_dloss(label, wtx):
    return glm_dloss(label, wtx)


def _splits(a: CRS, splits):
    if splits is None:
        return np.array([0, a.m], dtype=np.int64), 1
    s = np.ascontiguousarray(splits, dtype=np.int64)
    return s, len(s) - 1


def logreg_eval(a: CRS, label, w, b=0.0, sw=None, intercept=False, fmt="CRS", splits=None, nthreads=1,
                loss="logistic", eps=0.0):
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = np.ones(a.m) if sw is None else np.ascontiguousarray(sw, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    sp, P = _splits(a, splits)
    g = np.zeros(a.n + 1)
    out = np.zeros(1)
    lib().orc_glm_eval_f64(FMT[fmt], *a.args(), _ptr(label), _ptr(sw), _ptr(w), float(b), int(intercept),
                           _ptr(sp), P, nthreads, _ptr(g), _ptr(out), LOSS[loss], float(eps))
    return g, float(out[0])


def logreg_lbfgs(a: CRS, label, num_iter=1000, alpha=0.01, hist_size=10, reg_param=0.01, reg_type="ZERO",
                 intercept=False, tol=0.001, fmt="CRS", sw=None, w0=None, b0=None, splits=None, nthreads=1,
                 l2_no_eta=False, loss="logistic", eps=0.0):
    """``logistic_regression_with_lbfgs::train`` semantics (``loss`` selects
    the other GLMs' gradient); returns a dict."""
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = np.ones(a.m) if sw is None else np.ascontiguousarray(sw, dtype=np.float64)
    w = np.ones(a.n) if w0 is None else np.array(w0, dtype=np.float64)
    b = np.array([(1.0 if intercept else 0.0) if b0 is None else float(b0)])
    sp, P = _splits(a, splits)
    n_iter = np.zeros(1, dtype=np.int64)
    fl = np.zeros(1)
    trace = np.zeros(4 * num_iter)
    rc = lib().orc_glm_lbfgs_f64(FMT[fmt], *a.args(), _ptr(label), _ptr(sw), _ptr(sp), P, nthreads,
                                 num_iter, hist_size, reg_param, REG[reg_type], int(intercept), tol,
                                 _ptr(w), _ptr(b), _ptr(n_iter), _ptr(fl), _ptr(trace), int(l2_no_eta),
                                 LOSS[loss], float(eps))
    if rc != 0:
        raise ValueError(f"oracle lbfgs rejected the arguments (code {rc})")
    it = int(n_iter[0])
    return dict(w=w, b=float(b[0]), n_iter=it, loss=float(fl[0]), trace=trace.reshape(-1, 4)[:it])


class Problem:
    """An L-BFGS problem built once (per-rank matrices and transposed copies,
    rows split like MPI ranks) for repeated oracle runs whose timing covers
    the training loop alone."""

    def __init__(self, a: CRS, label, sw=None, fmt="CRS", splits=None, nthreads=1, loss="logistic", eps=0.0):
        self.n = a.n
        self._label = np.ascontiguousarray(label, dtype=np.float64)
        self._sw = np.ones(a.m) if sw is None else np.ascontiguousarray(sw, dtype=np.float64)
        sp, P = _splits(a, splits)
        self.h = lib().orc_problem_create(FMT[fmt], *a.args(), _ptr(self._label), _ptr(self._sw), _ptr(sp), P,
                                          nthreads, LOSS[loss], float(eps))
        if not self.h:
            raise ValueError("oracle problem rejected the arguments")

    def lbfgs(self, num_iter=1000, hist_size=10, reg_param=0.01, reg_type="ZERO", intercept=False, tol=0.001,
              w0=None, b0=None, l2_no_eta=False):
        w = np.ones(self.n) if w0 is None else np.array(w0, dtype=np.float64)
        b = np.array([(1.0 if intercept else 0.0) if b0 is None else float(b0)])
        n_iter = np.zeros(1, dtype=np.int64)
        fl = np.zeros(1)
        trace = np.zeros(4 * num_iter)
        rc = lib().orc_problem_lbfgs(self.h, num_iter, hist_size, reg_param, REG[reg_type], int(intercept), tol,
                                     _ptr(w), _ptr(b), _ptr(n_iter), _ptr(fl), _ptr(trace), int(l2_no_eta))
        if rc != 0:
            raise ValueError(f"oracle lbfgs rejected the arguments (code {rc})")
        it = int(n_iter[0])
        return dict(w=w, b=float(b[0]), n_iter=it, loss=float(fl[0]), trace=trace.reshape(-1, 4)[:it])

    def close(self):
        if self.h:
            lib().orc_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def logreg_sgd(a: CRS, label, num_iter=1000, alpha=0.01, mini_batch_fraction=1.0, reg_param=0.01,
               reg_type="ZERO", intercept=False, tol=0.001, fmt="CRS", sw=None, w0=None, b0=None, splits=None,
               nthreads=1, l2_no_eta=False, loss="logistic", eps=0.0, shrink=False):
    """``logistic_regression_with_sgd::train`` semantics (``loss`` selects the
    other GLMs' gradient; ``shrink`` the shrink::logistic_regression_with_sgd
    driver); returns a dict."""
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = np.ones(a.m) if sw is None else np.ascontiguousarray(sw, dtype=np.float64)
    w = np.ones(a.n) if w0 is None else np.array(w0, dtype=np.float64)
    # initModel(numFeatures): intercept 0 (logistic_regression_with_sgd.hpp:300)
    b = np.array([0.0 if b0 is None else float(b0)])
    sp, P = _splits(a, splits)
    n_iter = np.zeros(1, dtype=np.int64)
    fl = np.zeros(1)
    rc = lib().orc_glm_sgd_f64(FMT[fmt], *a.args(), _ptr(label), _ptr(sw), _ptr(sp), P, nthreads, num_iter,
                               alpha, mini_batch_fraction, reg_param, REG[reg_type], int(intercept), tol,
                               _ptr(w), _ptr(b), _ptr(n_iter), _ptr(fl), int(l2_no_eta) | (2 if shrink else 0),
                               LOSS[loss], float(eps))
    if rc != 0:
        raise ValueError(f"oracle sgd rejected the arguments (code {rc})")
    return dict(w=w, b=float(b[0]), n_iter=int(n_iter[0]), loss=float(fl[0]))


def softmax_train(a: CRS, label, K, num_iter=1000, alpha=0.01, reg_param=0.01, reg_type="ZERO", intercept=False,
                  tol=0.001, sw=None, W0=None, b0=None):
    """``multinomial_logistic_regression::train`` semantics (CRS); returns a dict
    with W (n, K), b (K), n_iter.  Labels are class ids 0..K-1."""
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = None if sw is None else np.ascontiguousarray(sw, dtype=np.float64)
    W = np.zeros((a.n, K)) if W0 is None else np.array(W0, dtype=np.float64, order="C")
    b = np.zeros(K) if b0 is None else np.array(b0, dtype=np.float64)
    n_iter = np.zeros(1, dtype=np.int64)
    rc = lib().orc_softmax_train_f64(*a.args(), _ptr(label), _ptr(sw), K, num_iter, alpha, reg_param, REG[reg_type],
                                     int(intercept), tol, _ptr(W), _ptr(b), _ptr(n_iter))
    if rc != 0:
        raise ValueError(f"oracle softmax rejected the arguments (code {rc})")
    return dict(W=W, b=b, n_iter=int(n_iter[0]))


def softmax_lbfgs(a: CRS, label, K, num_iter=100, hist_size=10, reg_param=0.01, reg_type="ZERO", tol=0.001,
                  sw=None, W0=None):
    """Multinomial logistic regression by L-BFGS: the reference's softmax
    gradient (softmax_gradient_descent.hpp:119-136) with its L-BFGS driver,
    the cross-entropy as the line search's loss, no intercept.  Returns W
    (n, K), n_iter, loss and the per-iteration trace."""
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = None if sw is None else np.ascontiguousarray(sw, dtype=np.float64)
    W = np.zeros((a.n, K)) if W0 is None else np.array(W0, dtype=np.float64).reshape(a.n, K)
    W = np.ascontiguousarray(W)
    n_iter = np.zeros(1, dtype=np.int64)
    fl = np.zeros(1)
    trace = np.zeros(4 * num_iter)
    rc = lib().orc_softmax_lbfgs_f64(*a.args(), _ptr(label), _ptr(sw), int(K), num_iter, hist_size, reg_param,
                                     REG[reg_type], tol, _ptr(W), _ptr(n_iter), _ptr(fl), _ptr(trace))
    if rc != 0:
        raise ValueError(f"oracle softmax lbfgs rejected the arguments (code {rc})")
    it = int(n_iter[0])
    return dict(W=W, n_iter=it, loss=float(fl[0]), trace=trace.reshape(-1, 4)[:it])


def softmax_probability(a: CRS, W, b, intercept=False) -> np.ndarray:
    W = np.ascontiguousarray(W, dtype=np.float64)
    K = W.shape[1]
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros((a.m, K))
    lib().orc_softmax_probability_f64(*a.args(), _ptr(W), _ptr(b), K, int(intercept), _ptr(out))
    return out


def predict_probability(a: CRS, w, b=0.0) -> np.ndarray:
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.zeros(a.m)
    lib().orc_predict_probability_f64(*a.args(), _ptr(w), float(b), _ptr(out))
    return out


def text_rank_splits(data: bytes, P: int):
    """Rows each of P ranks gets when the reference loads a text file with
    ``make_dvector_loadline`` (core/dvector.cc:198-300): rank r reads bytes
    [each*r-1, each*(r+1)-1) and owns the lines whose preceding newline lies
    in its range (rank 0 also owns the first line).  Returns P+1 row splits."""
    size = len(data)
    each = -(-size // P)
    starts = [0] + [i + 1 for i, ch in enumerate(data) if ch == 0x0A and i + 1 < size]
    owner = []
    for s in starts:
        if s == 0:
            owner.append(0)
            continue
        d = s - 1  # the newline before the line
        r = 0
        for q in range(P):
            lo = 0 if q == 0 else min(each * q - 1, size)
            hi = size if q == P - 1 else min(each * (q + 1) - 1, size)
            if lo <= d < hi:
                r = q
                break
        owner.append(r)
    counts = [owner.count(q) for q in range(P)]
    sp = [0]
    for c in counts:
        sp.append(sp[-1] + c)
    return sp


# ------------------------------------------------------------------ loaders
# Restatement of the reference's CRS file loaders, driving the C library's
# strtoll / strtod / strtof through ctypes so that every number is converted
# exactly as the reference converts it.
_libc = None


def _c():
    global _libc
    if _libc is None:
        _libc = C.CDLL(None)
        _libc.strtoll.restype = C.c_longlong
        _libc.strtoll.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_int]
        _libc.strtod.restype = C.c_double
        _libc.strtod.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        _libc.strtof.restype = C.c_float
        _libc.strtof.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    return _libc


def _getlines(data: bytes):
    """std::getline over a file: a last line without newline counts."""
    parts = data.split(b"\n")
    if parts and parts[-1] == b"":
        parts.pop()
    return parts


def _parseline(line: bytes, idx, val, as_float):
    """make_crs_matrix_local_parseline (matrix/crs_matrix.hpp:665-679)."""
    lc = _c()
    buf = C.create_string_buffer(line + b"\0\0")
    s = C.addressof(buf)
    end = C.c_void_p()
    while C.string_at(s, 1) != b"\0":
        pos = lc.strtoll(s, C.byref(end), 10)
        if end.value == s:
            break
        idx.append(pos)
        s = end.value + 1
        v = (lc.strtof if as_float else lc.strtod)(s, C.byref(end))
        val.append(v)
        s = end.value


def load_text(path, num_col=None, as_float=False):
    """make_crs_matrix_local_load (crs_matrix.hpp:757-775, x86 branch):
    returns (off, idx, val, num_row, num_col)."""
    off, idx, val = [0], [], []
    for line in _getlines(open(path, "rb").read()):
        _parseline(line, idx, val, as_float)
        off.append(len(val))
    if num_col is None:
        num_col = (max(idx) + 1) if idx else 0
    dt = np.float32 if as_float else np.float64
    return (np.array(off, dtype=np.int64), np.array(idx, dtype=np.int64), np.array(val, dtype=dt), len(off) - 1,
            num_col)


def load_libsvm(path, origin=0, as_float=False):
    """make_crs_matrix_local_loadlibsvm (crs_matrix.hpp:863-899): origin as
    IndexOrigin (0 AUTO, 1 ZERO_ORIG, 2 ONE_ORIG); returns (off, idx, val,
    num_row, num_col, label)."""
    lc = _c()
    off, idx, val, label = [0], [], [], []
    for line in _getlines(open(path, "rb").read()):
        buf = C.create_string_buffer(line + b"\0")
        s = C.addressof(buf)
        end = C.c_void_p()
        label.append((lc.strtof if as_float else lc.strtod)(s, C.byref(end)))  # loadlibsvm_extract_label
        _parseline(line[end.value - s:], idx, val, as_float)
        off.append(len(val))
    num_col = max(idx) + 1  # taken before the origin adjustment
    idx = np.array(idx, dtype=np.int64)
    if origin == 2 or (origin == 0 and idx.min() > 0):
        idx = idx - 1
    dt = np.float32 if as_float else np.float64
    return (np.array(off, dtype=np.int64), idx, np.array(val, dtype=dt), len(off) - 1, num_col,
            np.array(label, dtype=np.float64))


def load_binary(path, val_dtype=np.float64, idx_dtype=np.uint64, off_dtype=np.uint64):
    """make_crs_matrix_local_loadbinary (crs_matrix.hpp:565-603), native byte
    order: returns (off, idx, val, num_row, num_col)."""
    m, n = (int(x) for x in open(os.path.join(path, "nums")).read().split()[:2])
    val = np.fromfile(os.path.join(path, "val"), dtype=val_dtype)
    idx = np.fromfile(os.path.join(path, "idx"), dtype=idx_dtype).astype(np.int64)
    off = np.fromfile(os.path.join(path, "off"), dtype=off_dtype).astype(np.int64)
    return off, idx, val, m, n
