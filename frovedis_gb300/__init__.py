"""frovedis_gb300 — GB300 sparse logistic-regression path behind a C ABI.

Python bindings (ctypes) to ``libfvg.so`` (include/fvg.h).  They mirror the
reference's local-matrix operators and trainer entry points:

* ``Matrix.spmv / trans_mv / spmm``  — operator*(crs/ell/jds/hybrid, vector),
  trans_mv, operator*(crs, rowmajor)   (frovedis matrix/*.hpp)
* ``logreg_lbfgs`` / ``logreg_sgd``  — logistic_regression_with_{lbfgs,sgd}::
  train main APIs (ml/glm/logistic_regression_with_*.hpp)
* ``logreg_eval``                    — gradient_descent::compute_gradient
* ``predict_probability``            — logistic_regression_model::predict_probability

There is no CPU fallback: every call runs the CUDA library, and loading
fails with an error when it cannot be built or loaded.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

F64, F32, BF16 = 0, 1, 2
CRS, JDS, ELL, HYBRID = 0, 1, 2, 3
FORMATS = {"CRS": CRS, "JDS": JDS, "ELL": ELL, "HYBRID": HYBRID}
REG = {"ZERO": 0, "L1": 1, "L2": 2}
# fvg_loss: the GLM family's compute_dloss kinds (ml/glm/gradient.hpp)
LOSS = {"logistic": 0, "linear": 1, "hinge": 2, "eps": 3, "sqeps": 4}
SPLIT = 3
DTYPES = {"f64": F64, "f32": F32, "bf16": BF16, "split": SPLIT}

_p = C.c_void_p
_i64 = C.c_int64
_int = C.c_int
_dbl = C.c_double


class FvgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fvg status {code}: {msg}")
        self.code = code


class GlmParams(C.Structure):
    _fields_ = [("num_iteration", C.c_int64), ("alpha", C.c_double), ("hist_size", C.c_int64),
                ("reg_param", C.c_double), ("reg_type", C.c_int32), ("intercept", C.c_int32),
                ("convergence_tol", C.c_double), ("mat_type", C.c_int32), ("mini_batch_fraction", C.c_double),
                ("num_partitions", C.c_int32), ("storage", C.c_int32), ("refine", C.c_int32),
                ("refine_stall", C.c_double), ("l2_no_eta", C.c_int32), ("use_graph", C.c_int32),
                ("trace", C.POINTER(C.c_double)), ("row_splits", C.POINTER(C.c_int64)),
                ("loss", C.c_int32), ("epsilon", C.c_double)]


EXPORTS = [
    "fvg_ctx_create", "fvg_ctx_destroy", "fvg_ctx_last_error", "fvg_ctx_stream", "fvg_ctx_synchronize",
    "fvg_ctx_set_profiling", "fvg_ctx_get_profile", "fvg_ctx_reset_profile", "fvg_ctx_kernel_launches",
    "fvg_matrix_create_crs", "fvg_matrix_destroy", "fvg_matrix_info", "fvg_matrix_prepare",
    "fvg_matrix_add_storage", "fvg_matrix_device_bytes", "fvg_matrix_get_transpose", "fvg_matrix_get_ell",
    "fvg_matrix_get_jds", "fvg_matrix_get_hybrid", "fvg_spmv", "fvg_trans_mv", "fvg_spmm",
    "fvg_glm_params_default", "fvg_logreg_lbfgs", "fvg_logreg_sgd", "fvg_logreg_eval",
    "fvg_logreg_predict_probability", "fvg_spmv_no_alloc", "fvg_logreg_lbfgs_batched",
    "fvg_multinomial_train", "fvg_multinomial_probability",
    "fvg_matrix_get_crs", "fvg_matrix_load_text", "fvg_matrix_load_libsvm", "fvg_matrix_get_labels",
    "fvg_matrix_load_binary", "fvg_glm_lbfgs", "fvg_glm_sgd", "fvg_glm_lbfgs_batched", "fvg_glm_eval",
    "fvg_logreg_shrink_sgd", "fvg_matrix_set_panels", "fvg_matrix_panel_info", "fvg_matrix_set_head",
    "fvg_matrix_head_info", "fvg_ctx_set_wait_limit", "fvg_debug_inject_alloc_failure", "fvg_matrix_autotune",
    "fvg_multinomial_lbfgs", "fvg_logreg_lbfgs_multi", "fvg_glm_lbfgs_multi",
]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_needed: bool = True):
    """Loads libfvg.so, building it first when it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise FvgError(-1, f"{_build.LIB} is missing; run frovedis_gb300.build.build()")
    L = C.CDLL(_build.LIB)
    sig = {
        "fvg_ctx_create": ([_int, C.POINTER(_p)], _int),
        "fvg_ctx_destroy": ([_p], None),
        "fvg_ctx_last_error": ([_p], C.c_char_p),
        "fvg_ctx_stream": ([_p], _p),
        "fvg_ctx_synchronize": ([_p], _int),
        "fvg_ctx_set_profiling": ([_p, _int], _int),
        "fvg_ctx_get_profile": ([_p, C.c_char_p, C.POINTER(_dbl), C.POINTER(_i64)], _int),
        "fvg_ctx_reset_profile": ([_p], _int),
        "fvg_ctx_kernel_launches": ([_p], _i64),
        "fvg_ctx_set_wait_limit": ([_p, _i64], _int),
        "fvg_matrix_autotune": ([_p, _p, _int, _p, _int, _p, _p, _i64, C.POINTER(_i64)], _int),
        "fvg_debug_inject_alloc_failure": ([_i64], None),
        "fvg_matrix_create_crs": ([_p, _i64, _i64, _p, _p, _p, _int, _int, C.POINTER(_p)], _int),
        "fvg_matrix_destroy": ([_p], None),
        "fvg_matrix_info": ([_p, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)], _int),
        "fvg_matrix_prepare": ([_p, _p, _int, _int], _int),
        "fvg_matrix_add_storage": ([_p, _p, _int], _int),
        "fvg_matrix_set_panels": ([_p, _p, _i64, _dbl], _int),
        "fvg_matrix_panel_info": ([_p, _p, C.POINTER(_i64)], _int),
        "fvg_matrix_set_head": ([_p, _p, _i64], _int),
        "fvg_matrix_head_info": ([_p, _p, C.POINTER(_i64)], _int),
        "fvg_matrix_device_bytes": ([_p], _i64),
        "fvg_matrix_get_transpose": ([_p, _p, _p, _p, _p], _int),
        "fvg_matrix_get_ell": ([_p, _p, C.POINTER(_i64), _p, _p], _int),
        "fvg_matrix_get_jds": ([_p, _p, C.POINTER(_i64), _p, _p, _p, _p], _int),
        "fvg_matrix_get_hybrid": ([_p, _p, _p, _p, _p, _p, _p, _p, _p, _p], _int),
        "fvg_spmv": ([_p, _p, _int, _int, _int, _p, _p, _int], _int),
        "fvg_trans_mv": ([_p, _p, _int, _int, _int, _p, _p, _int], _int),
        "fvg_spmm": ([_p, _p, _int, _int, _int, _p, _i64, _p, _int], _int),
        "fvg_glm_params_default": ([C.POINTER(GlmParams)], None),
        "fvg_logreg_lbfgs": ([_p, _p, _p, _p, C.POINTER(GlmParams), _p, C.POINTER(_dbl), C.POINTER(_i64),
                              C.POINTER(_dbl)], _int),
        "fvg_logreg_sgd": ([_p, _p, _p, _p, C.POINTER(GlmParams), _p, C.POINTER(_dbl), C.POINTER(_i64),
                            C.POINTER(_dbl)], _int),
        "fvg_logreg_eval": ([_p, _p, _int, _int, _p, _p, _p, _dbl, _int, _p, C.POINTER(_dbl)], _int),
        "fvg_logreg_predict_probability": ([_p, _p, _p, _dbl, _p], _int),
        "fvg_spmv_no_alloc": ([_p, _p, _int, _int, _p, _p], _int),
        "fvg_logreg_lbfgs_batched": ([_p, _p, _p, _p, C.POINTER(GlmParams), _i64, _p, _p, _p, _p, _p], _int),
        "fvg_multinomial_train": ([_p, _p, _p, _p, C.POINTER(GlmParams), _i64, _p, _p, C.POINTER(_i64)], _int),
        "fvg_multinomial_lbfgs": ([_p, _p, _p, _p, C.POINTER(GlmParams), _i64, _p, C.POINTER(_i64), C.POINTER(_dbl)],
                                  _int),
        "fvg_multinomial_probability": ([_p, _p, _p, _p, _i64, _int, _p], _int),
        "fvg_matrix_get_crs": ([_p, _p, _p, _p, _p], _int),
        "fvg_matrix_load_text": ([_p, C.c_char_p, _int, _i64, C.POINTER(_p)], _int),
        "fvg_matrix_load_libsvm": ([_p, C.c_char_p, _int, _int, C.POINTER(_p)], _int),
        "fvg_matrix_get_labels": ([_p, _p], _int),
        "fvg_matrix_load_binary": ([_p, C.c_char_p, _int, C.c_char_p, C.c_char_p, C.POINTER(_p)], _int),
        "fvg_glm_lbfgs": ([_p, _p, _p, _p, C.POINTER(GlmParams), _p, C.POINTER(_dbl), C.POINTER(_i64),
                           C.POINTER(_dbl)], _int),
        "fvg_glm_sgd": ([_p, _p, _p, _p, C.POINTER(GlmParams), _p, C.POINTER(_dbl), C.POINTER(_i64),
                         C.POINTER(_dbl)], _int),
        "fvg_glm_lbfgs_batched": ([_p, _p, _p, _p, C.POINTER(GlmParams), _i64, _p, _p, _p, _p, _p], _int),
        "fvg_logreg_lbfgs_multi": ([_p, _i64, _p, _p, _p, C.POINTER(GlmParams), _i64, _p, _p, _p, _p, _p], _int),
        "fvg_glm_lbfgs_multi": ([_p, _i64, _p, _p, _p, C.POINTER(GlmParams), _i64, _p, _p, _p, _p, _p], _int),
        "fvg_logreg_shrink_sgd": ([_p, _p, _p, _p, C.POINTER(GlmParams), _p, C.POINTER(_dbl), C.POINTER(_i64),
                                   C.POINTER(_dbl)], _int),
        "fvg_glm_eval": ([_p, _p, _int, _int, _int, _dbl, _p, _p, _p, _dbl, _int, _p, C.POINTER(_dbl)], _int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_p)


def _fmt(f):
    return FORMATS[f] if isinstance(f, str) else int(f)


def _dt(d):
    return DTYPES[d] if isinstance(d, str) else int(d)


class Context:
    """One GPU, one CUDA stream (fvg_ctx)."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = _p()
        rc = self.L.fvg_ctx_create(device, C.byref(h))
        if rc != 0:
            raise FvgError(rc, "fvg_ctx_create failed (is a CUDA GPU visible?)")
        self.h = h

    def check(self, rc):
        if rc != 0:
            raise FvgError(rc, self.L.fvg_ctx_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.fvg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self) -> int:
        return self.L.fvg_ctx_stream(self.h) or 0

    def synchronize(self):
        self.check(self.L.fvg_ctx_synchronize(self.h))

    def set_profiling(self, on: bool):
        self.check(self.L.fvg_ctx_set_profiling(self.h, int(on)))

    def profile(self, name: str):
        ms = _dbl()
        n = _i64()
        self.check(self.L.fvg_ctx_get_profile(self.h, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def reset_profile(self):
        self.check(self.L.fvg_ctx_reset_profile(self.h))

    @property
    def kernel_launches(self) -> int:
        return int(self.L.fvg_ctx_kernel_launches(self.h))

    def set_wait_limit(self, polls=-1):
        """Poll budget of the kernels' bounded device-side waits (< 0: the
        defaults; 0: a wait that is not complete at once gives up)."""
        self.check(self.L.fvg_ctx_set_wait_limit(self.h, int(polls)))

    def matrix(self, m, n, off, idx, val, on_device=False):
        return Matrix(self, m, n, off, idx, val, on_device=on_device)

    def _wrap(self, h, dt):
        M = Matrix.__new__(Matrix)
        M.ctx = self
        M.h = h
        M.master = dt
        r, c = _i64(), _i64()
        self.check(self.L.fvg_matrix_info(h, C.byref(r), C.byref(c), None))
        M.m, M.n = r.value, c.value
        M._keep = None
        return M

    def load_text(self, path, dtype="f64", num_col=-1):
        """make_crs_matrix_local_load: "col:value" lines parsed on the device."""
        h = _p()
        self.check(self.L.fvg_matrix_load_text(self.h, str(path).encode(), _dt(dtype), int(num_col), C.byref(h)))
        return self._wrap(h, _dt(dtype))

    def load_libsvm(self, path, dtype="f64", index_origin=0):
        """make_crs_matrix_local_loadlibsvm (index_origin 0 AUTO, 1 ZERO_ORIG,
        2 ONE_ORIG); returns (matrix, labels)."""
        h = _p()
        self.check(self.L.fvg_matrix_load_libsvm(self.h, str(path).encode(), _dt(dtype), int(index_origin),
                                                 C.byref(h)))
        M = self._wrap(h, _dt(dtype))
        lab = np.zeros(M.m)
        self.check(self.L.fvg_matrix_get_labels(M.h, _ptr(lab)))
        return M, lab

    def load_binary(self, path, dtype="f64", idx_type="uint64_t", off_type="uint64_t"):
        """make_crs_matrix_local_loadbinary (type names as in the type file)."""
        h = _p()
        self.check(self.L.fvg_matrix_load_binary(self.h, str(path).encode(), _dt(dtype), idx_type.encode(),
                                                 off_type.encode(), C.byref(h)))
        return self._wrap(h, _dt(dtype))


class Matrix:
    """Device CRS matrix (fvg_matrix) with derived layouts built on demand."""

    def __init__(self, ctx: Context, m, n, off, idx, val, on_device=False):
        self.ctx = ctx
        self.m, self.n = int(m), int(n)
        if on_device:  # (off, idx, val, dtype) are device pointers
            offp, idxp, valp, dt = off, idx, val[0], val[1]
        else:
            off = np.ascontiguousarray(off, dtype=np.int32)
            idx = np.ascontiguousarray(idx, dtype=np.int32)
            if isinstance(val, np.ndarray) and val.dtype == np.float32:
                dt = F32
            elif isinstance(val, np.ndarray) and val.dtype == np.uint16:  # raw bf16 bits
                dt = BF16
            else:
                val = np.ascontiguousarray(val, dtype=np.float64)
                dt = F64
            val = np.ascontiguousarray(val)
            self._keep = (off, idx, val)
            offp, idxp, valp = _ptr(off), _ptr(idx), _ptr(val)
        h = _p()
        ctx.check(ctx.L.fvg_matrix_create_crs(ctx.h, self.m, self.n, offp, idxp, valp, dt, int(on_device),
                                              C.byref(h)))
        self.h = h
        self._keep = None
        self.master = dt

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.fvg_matrix_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nnz(self):
        z = _i64()
        self.ctx.check(self.ctx.L.fvg_matrix_info(self.h, None, None, C.byref(z)))
        return z.value

    def prepare(self, fmt="CRS", transpose=True):
        self.ctx.check(self.ctx.L.fvg_matrix_prepare(self.ctx.h, self.h, _fmt(fmt), int(transpose)))

    def add_storage(self, storage):
        self.ctx.check(self.ctx.L.fvg_matrix_add_storage(self.ctx.h, self.h, _dt(storage)))

    def set_panels(self, rows=-1, min_per_panel=0.0):
        """Row-panel layout of the FP32/BF16 backward product: rows < 0 picks it
        from the matrix, 0 turns it off, > 0 forces panels of that height."""
        self.ctx.check(self.ctx.L.fvg_matrix_set_panels(self.ctx.h, self.h, int(rows), float(min_per_panel)))

    def set_head(self, columns=-1):
        """Forward head of the FP32/BF16 forward product: columns < 0 picks it
        from the matrix, 0 turns it off, > 0 forces that many columns."""
        self.ctx.check(self.ctx.L.fvg_matrix_set_head(self.ctx.h, self.h, int(columns)))

    def autotune(self, storage="split", label=None, reps=3):
        """Times the candidate training layouts (fvg_matrix_autotune) and
        leaves the fastest set on the matrix.  Returns (best, tried): dicts
        with format (name), head (bool), panel_min (0 = panels off) and
        eval_ms; train with mat_type=best["format"]."""
        class _Choice(C.Structure):
            _fields_ = [("format", C.c_int32), ("head", C.c_int32), ("panel_min", C.c_double),
                        ("eval_ms", C.c_double)]
        names = {v: k for k, v in FORMATS.items()}
        best = _Choice()
        tried = (_Choice * 32)()
        n = _i64()
        lab = None if label is None else np.ascontiguousarray(label, dtype=np.float64)
        self.ctx.check(self.ctx.L.fvg_matrix_autotune(self.ctx.h, self.h, _dt(storage), _ptr(lab), int(reps),
                                                      C.byref(best), tried, 32, C.byref(n)))

        def d(ch):
            return {"format": names[ch.format], "head": bool(ch.head), "panel_min": ch.panel_min,
                    "eval_ms": ch.eval_ms}
        return d(best), [d(tried[i]) for i in range(min(n.value, 32))]

    def head_info(self):
        """(columns in the head, their entries); zeros when unused."""
        info = (_i64 * 2)()
        self.ctx.check(self.ctx.L.fvg_matrix_head_info(self.ctx.h, self.h, info))
        return tuple(int(v) for v in info)

    def panel_info(self):
        """(rows per panel, panels, columns in the panels, their entries); zeros when unused."""
        info = (_i64 * 4)()
        self.ctx.check(self.ctx.L.fvg_matrix_panel_info(self.ctx.h, self.h, info))
        return tuple(int(v) for v in info)

    @property
    def device_bytes(self):
        return int(self.ctx.L.fvg_matrix_device_bytes(self.h))

    # --- products -------------------------------------------------------
    def _product(self, fn, x, nout, fmt, storage, vec):
        vd = np.float64 if _dt(vec) == F64 else np.float32
        x = np.ascontiguousarray(x, dtype=vd)
        y = np.zeros(nout, dtype=vd)
        self.ctx.check(fn(self.ctx.h, self.h, _fmt(fmt), _dt(storage), _dt(vec), _ptr(x), _ptr(y), 0))
        return y

    def spmv(self, x, fmt="CRS", storage="f64", vec="f64"):
        return self._product(self.ctx.L.fvg_spmv, x, self.m, fmt, storage, vec)

    def trans_mv(self, x, fmt="CRS", storage="f64", vec="f64"):
        return self._product(self.ctx.L.fvg_trans_mv, x, self.n, fmt, storage, vec)

    def spmv_device(self, xptr, yptr, fmt="CRS", storage="f64", vec="f64"):
        self.ctx.check(self.ctx.L.fvg_spmv(self.ctx.h, self.h, _fmt(fmt), _dt(storage), _dt(vec), xptr, yptr, 1))

    def trans_mv_device(self, xptr, yptr, fmt="CRS", storage="f64", vec="f64"):
        self.ctx.check(self.ctx.L.fvg_trans_mv(self.ctx.h, self.h, _fmt(fmt), _dt(storage), _dt(vec), xptr, yptr,
                                               1))

    def spmm_device(self, xptr, k, yptr, fmt="CRS", storage="f64", vec="f64"):
        """Y = A X with X (num_col x k) and Y (num_row x k) row-major device arrays."""
        self.ctx.check(self.ctx.L.fvg_spmm(self.ctx.h, self.h, _fmt(fmt), _dt(storage), _dt(vec), xptr, int(k), yptr,
                                           1))

    def spmm(self, X, fmt="CRS", storage="f64", vec="f64"):
        vd = np.float64 if _dt(vec) == F64 else np.float32
        X = np.ascontiguousarray(X, dtype=vd)
        k = X.shape[1]
        Y = np.zeros((self.m, k), dtype=vd)
        self.ctx.check(self.ctx.L.fvg_spmm(self.ctx.h, self.h, _fmt(fmt), _dt(storage), _dt(vec), _ptr(X), k,
                                           _ptr(Y), 0))
        return Y

    # --- derived layouts (host copies) ----------------------------------
    def get_crs(self):
        """(off, idx, val) of the uploaded matrix (values as FP64)."""
        z = self.nnz
        off = np.zeros(self.m + 1, dtype=np.int32)
        idx = np.zeros(max(z, 1), dtype=np.int32)
        val = np.zeros(max(z, 1))
        self.ctx.check(self.ctx.L.fvg_matrix_get_crs(self.ctx.h, self.h, _ptr(off), _ptr(idx), _ptr(val)))
        return off, idx[:z], val[:z]

    def get_transpose(self):
        toff = np.zeros(self.n + 1, dtype=np.int32)
        tidx = np.zeros(max(self.nnz, 1), dtype=np.int32)
        tval = np.zeros(max(self.nnz, 1))
        self.ctx.check(self.ctx.L.fvg_matrix_get_transpose(self.ctx.h, self.h, _ptr(toff), _ptr(tidx), _ptr(tval)))
        z = self.nnz
        return toff, tidx[:z], tval[:z]

    def get_ell(self):
        w = _i64()
        self.ctx.check(self.ctx.L.fvg_matrix_get_ell(self.ctx.h, self.h, C.byref(w), None, None))
        cells = self.m * w.value
        eidx = np.zeros(max(cells, 1), dtype=np.int32)
        ev = np.zeros(max(cells, 1))
        self.ctx.check(self.ctx.L.fvg_matrix_get_ell(self.ctx.h, self.h, C.byref(w), _ptr(eidx), _ptr(ev)))
        return w.value, eidx[:cells], ev[:cells]

    def get_jds(self):
        nd = _i64()
        self.ctx.check(self.ctx.L.fvg_matrix_get_jds(self.ctx.h, self.h, C.byref(nd), None, None, None, None))
        z = self.nnz
        perm = np.zeros(max(self.m, 1), dtype=np.int32)
        joff = np.zeros(nd.value + 1, dtype=np.int64)
        jidx = np.zeros(max(z, 1), dtype=np.int32)
        jval = np.zeros(max(z, 1))
        self.ctx.check(self.ctx.L.fvg_matrix_get_jds(self.ctx.h, self.h, C.byref(nd), _ptr(perm), _ptr(joff),
                                                     _ptr(jidx), _ptr(jval)))
        return perm[: self.m if z else 0], joff, jidx[:z], jval[:z]

    def get_hybrid(self):
        info = np.zeros(5, dtype=np.int64)
        L = self.ctx.L
        self.ctx.check(L.fvg_matrix_get_hybrid(self.ctx.h, self.h, _ptr(info), None, None, None, None, None, None,
                                               None))
        nd, crows, cnnz, jnnz, plen = (int(v) for v in info)
        perm = np.zeros(max(self.m, 1), dtype=np.int32)
        joff = np.zeros(nd + 1, dtype=np.int64)
        jidx = np.zeros(max(jnnz, 1), dtype=np.int32)
        jval = np.zeros(max(jnnz, 1))
        coff = np.zeros(crows + 1, dtype=np.int64)
        cidx = np.zeros(max(cnnz, 1), dtype=np.int32)
        cval = np.zeros(max(cnnz, 1))
        self.ctx.check(L.fvg_matrix_get_hybrid(self.ctx.h, self.h, _ptr(info), _ptr(perm), _ptr(joff), _ptr(jidx),
                                               _ptr(jval), _ptr(coff), _ptr(cidx), _ptr(cval)))
        return dict(perm=perm[:plen], joff=joff, jidx=jidx[:jnnz], jval=jval[:jnnz], coff=coff,
                    cidx=cidx[:cnnz], cval=cval[:cnnz], crs_rows=crows)


_ALIASES = {"num_iter": "num_iteration", "numIteration": "num_iteration", "fmt": "mat_type",
            "regParam": "reg_param", "hist": "hist_size", "tol": "convergence_tol", "eps": "epsilon"}


def glm_params(**kw) -> GlmParams:
    p = GlmParams()
    load().fvg_glm_params_default(C.byref(p))
    fields = {f[0] for f in GlmParams._fields_}
    for k, v in kw.items():
        k = _ALIASES.get(k, k)
        if k not in fields:
            raise TypeError(f"unknown training parameter {k!r}")
        if k in ("reg_type",) and isinstance(v, str):
            v = REG[v]
        if k in ("loss",) and isinstance(v, str):
            v = LOSS[v]
        if k in ("mat_type",):
            v = _fmt(v)
        if k in ("storage",):
            v = _dt(v)
        setattr(p, k, v)
    return p


def _train(fn, mat: Matrix, label, sample_weight=None, w0=None, b0=None, trace=False, row_splits=None,
           sgd=False, **kw):
    ctx = mat.ctx
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = None if sample_weight is None else np.ascontiguousarray(sample_weight, dtype=np.float64)
    icpt = bool(kw.get("intercept", False))
    w = np.ones(mat.n) if w0 is None else np.array(w0, dtype=np.float64)  # weight init = 1 (linear_model.hpp:310)
    # initial intercept: the SGD trainers build initModel(numFeatures) (0), the
    # L-BFGS ones initModel(numFeatures, isIntercept)
    # (logistic_regression_with_sgd.hpp:300, logistic_regression_with_lbfgs.hpp:301)
    b = C.c_double((0.0 if sgd or not icpt else 1.0) if b0 is None else float(b0))
    kw["intercept"] = int(icpt)
    p = glm_params(**kw)
    tr = None
    if trace:
        tr = np.zeros(4 * p.num_iteration)
        p.trace = tr.ctypes.data_as(C.POINTER(C.c_double))
    sp = None
    if row_splits is not None:
        sp = np.ascontiguousarray(row_splits, dtype=np.int64)
        p.num_partitions = len(sp) - 1
        p.row_splits = sp.ctypes.data_as(C.POINTER(C.c_int64))
    n_iter = _i64()
    loss = _dbl()
    ctx.check(fn(ctx.h, mat.h, _ptr(label), _ptr(sw), C.byref(p), _ptr(w), C.byref(b), C.byref(n_iter),
                 C.byref(loss)))
    out = dict(w=w, b=b.value, n_iter=n_iter.value, loss=loss.value)
    if trace:
        out["trace"] = tr.reshape(-1, 4)[: n_iter.value]
    return out


def logreg_lbfgs(mat: Matrix, label, **kw):
    """logistic_regression_with_lbfgs::train (defaults as in the reference)."""
    return _train(mat.ctx.L.fvg_logreg_lbfgs, mat, label, **kw)


def logreg_lbfgs_batched(mat: Matrix, label, reg_params, sample_weight=None, w0=None, b0=None, _fn=None, **kw):
    """k L-BFGS trainings on one matrix, model j with reg_param = reg_params[j]
    (fvg_logreg_lbfgs_batched).  w0: (k, n) initial weights (default all 1),
    b0: (k,) initial intercepts.  Returns w (k, n), b, n_iter, loss (k,)."""
    ctx = mat.ctx
    lam = np.ascontiguousarray(reg_params, dtype=np.float64)
    k = len(lam)
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = None if sample_weight is None else np.ascontiguousarray(sample_weight, dtype=np.float64)
    icpt = bool(kw.get("intercept", False))
    # order="C": a copy of a broadcast view would otherwise keep its column-major memory order
    w = (np.ones((k, mat.n)) if w0 is None
         else np.array(np.broadcast_to(w0, (k, mat.n)), dtype=np.float64, order="C"))
    b = (np.full(k, 1.0 if icpt else 0.0) if b0 is None
         else np.array(np.broadcast_to(b0, (k,)), dtype=np.float64, order="C"))
    kw["intercept"] = int(icpt)
    p = glm_params(**kw)
    n_iter = np.zeros(k, dtype=np.int64)
    loss = np.zeros(k)
    fn = ctx.L.fvg_logreg_lbfgs_batched if _fn is None else _fn
    ctx.check(fn(ctx.h, mat.h, _ptr(label), _ptr(sw), C.byref(p), k, _ptr(lam), _ptr(w), _ptr(b), _ptr(n_iter),
                 _ptr(loss)))
    return dict(w=w, b=b, n_iter=n_iter, loss=loss)


def logreg_lbfgs_multi(mats, labels, reg_params, sample_weights=None, w0=None, b0=None, _fn=None, **kw):
    """The batched trainer over several datasets in one launch
    (fvg_logreg_lbfgs_multi): the k models of every dataset, model (d, j) on
    mats[d] with reg_param = reg_params[j].  w0[d]: (k, n_d) initial weights
    of dataset d (default all 1), b0: (nd, k) initial intercepts.  Returns
    w (a list of (k, n_d) arrays), b, n_iter, loss ((nd, k) arrays)."""
    mats = list(mats)
    nd = len(mats)
    ctx = mats[0].ctx
    lam = np.ascontiguousarray(reg_params, dtype=np.float64)
    k = len(lam)
    labs = [np.ascontiguousarray(l, dtype=np.float64) for l in labels]
    sws = None if sample_weights is None else [
        None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in sample_weights]
    icpt = bool(kw.get("intercept", False))
    ns = [m.n for m in mats]
    wflat = np.empty(sum(k * n for n in ns))
    o = 0
    for d, n in enumerate(ns):
        wd = np.ones((k, n)) if w0 is None else np.broadcast_to(np.asarray(w0[d], dtype=np.float64), (k, n))
        wflat[o:o + k * n] = wd.reshape(-1)
        o += k * n
    b = (np.full((nd, k), 1.0 if icpt else 0.0) if b0 is None
         else np.array(np.broadcast_to(b0, (nd, k)), dtype=np.float64, order="C"))
    kw["intercept"] = int(icpt)
    p = glm_params(**kw)
    n_iter = np.zeros((nd, k), dtype=np.int64)
    loss = np.zeros((nd, k))
    mh = (_p * nd)(*[m.h for m in mats])
    lh = (_p * nd)(*[_ptr(x) for x in labs])
    sh = None if sws is None else (_p * nd)(*[_ptr(x) for x in sws])
    fn = ctx.L.fvg_logreg_lbfgs_multi if _fn is None else _fn
    ctx.check(fn(ctx.h, nd, mh, lh, sh, C.byref(p), k, _ptr(lam), _ptr(wflat), _ptr(b), _ptr(n_iter), _ptr(loss)))
    w, o = [], 0
    for n in ns:
        w.append(wflat[o:o + k * n].reshape(k, n))
        o += k * n
    return dict(w=w, b=b, n_iter=n_iter, loss=loss)


def glm_lbfgs_multi(mats, labels, reg_params, loss="linear", **kw):
    """The multi-dataset batched trainer for any GLM loss (fvg_glm_lbfgs_multi)."""
    return logreg_lbfgs_multi(mats, labels, reg_params, loss=loss, _fn=mats[0].ctx.L.fvg_glm_lbfgs_multi, **kw)


def multinomial_lbfgs(mat: Matrix, label, nclasses, sample_weight=None, W0=None, trace=False, **kw):
    """Multinomial logistic regression by L-BFGS (fvg_multinomial_lbfgs): the
    reference's softmax gradient with the binary trainers' L-BFGS loop and the
    cross-entropy as the line search's loss; no intercept.  W0 (n, nclasses)
    defaults to zeros.  Returns W, n_iter, loss (and trace)."""
    ctx = mat.ctx
    K = int(nclasses)
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = None if sample_weight is None else np.ascontiguousarray(sample_weight, dtype=np.float64)
    W = np.zeros((mat.n, K)) if W0 is None else np.array(W0, dtype=np.float64).reshape(mat.n, K)
    W = np.ascontiguousarray(W)
    p = glm_params(**kw)
    tr = None
    if trace:
        tr = np.zeros(4 * p.num_iteration)
        p.trace = tr.ctypes.data_as(C.POINTER(C.c_double))
    n_iter = _i64()
    loss = _dbl()
    ctx.check(ctx.L.fvg_multinomial_lbfgs(ctx.h, mat.h, _ptr(label), _ptr(sw), C.byref(p), K, _ptr(W),
                                          C.byref(n_iter), C.byref(loss)))
    out = dict(W=W, n_iter=n_iter.value, loss=loss.value)
    if trace:
        out["trace"] = tr.reshape(-1, 4)[: n_iter.value]
    return out


def multinomial_train(mat: Matrix, label, nclasses, sample_weight=None, W0=None, b0=None, **kw):
    """multinomial_logistic_regression::train (fvg_multinomial_train).  label:
    class ids 0..nclasses-1; W0 (n, nclasses) and b0 (nclasses,) default to
    zeros as in the reference's model constructor.  Returns W, b, n_iter."""
    ctx = mat.ctx
    K = int(nclasses)
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = None if sample_weight is None else np.ascontiguousarray(sample_weight, dtype=np.float64)
    W = np.zeros((mat.n, K)) if W0 is None else np.array(W0, dtype=np.float64, order="C")
    b = np.zeros(K) if b0 is None else np.array(b0, dtype=np.float64, order="C")
    kw["intercept"] = int(bool(kw.get("intercept", False)))
    p = glm_params(**kw)
    n_iter = _i64()
    ctx.check(ctx.L.fvg_multinomial_train(ctx.h, mat.h, _ptr(label), _ptr(sw), C.byref(p), K, _ptr(W), _ptr(b),
                                          C.byref(n_iter)))
    return dict(W=W, b=b, n_iter=n_iter.value)


def multinomial_probability(mat: Matrix, W, b, intercept=False):
    W = np.ascontiguousarray(W, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    K = W.shape[1]
    out = np.zeros((mat.m, K))
    mat.ctx.check(mat.ctx.L.fvg_multinomial_probability(mat.ctx.h, mat.h, _ptr(W), _ptr(b), K, int(intercept),
                                                        _ptr(out)))
    return out


def logreg_sgd(mat: Matrix, label, **kw):
    """logistic_regression_with_sgd::train (defaults as in the reference)."""
    return _train(mat.ctx.L.fvg_logreg_sgd, mat, label, sgd=True, **kw)


def logreg_shrink_sgd(mat: Matrix, label, **kw):
    """shrink::logistic_regression_with_sgd::train (fvg_logreg_shrink_sgd)."""
    return _train(mat.ctx.L.fvg_logreg_shrink_sgd, mat, label, sgd=True, **kw)


def glm_lbfgs(mat: Matrix, label, loss="linear", **kw):
    """The GLM family's L-BFGS trainers (fvg_glm_lbfgs): loss "linear" with
    reg_type ZERO / L2 / L1 = linear_regression / ridge_regression / lasso
    _with_lbfgs, "hinge" = svm_with_lbfgs, "logistic" as logreg_lbfgs."""
    return _train(mat.ctx.L.fvg_glm_lbfgs, mat, label, loss=loss, **kw)


def glm_sgd(mat: Matrix, label, loss="linear", **kw):
    """The GLM family's SGD trainers (fvg_glm_sgd): "linear" (linear / ridge /
    lasso), "hinge" (svm_with_sgd), "eps" / "sqeps" (svm_regression_with_sgd
    with SVRLossType EPS / SQEPS and ``epsilon``)."""
    return _train(mat.ctx.L.fvg_glm_sgd, mat, label, sgd=True, loss=loss, **kw)


def glm_lbfgs_batched(mat: Matrix, label, reg_params, loss="linear", **kw):
    """k GLM L-BFGS trainings on one matrix (fvg_glm_lbfgs_batched)."""
    return logreg_lbfgs_batched(mat, label, reg_params, loss=loss, _fn=mat.ctx.L.fvg_glm_lbfgs_batched, **kw)


def logreg_eval(mat: Matrix, label, w, b=0.0, intercept=False, sample_weight=None, fmt="CRS", storage="f64",
                loss=None, epsilon=0.0):
    """One loss/gradient evaluation: fvg_logreg_eval, or fvg_glm_eval when a
    loss kind is named."""
    label = np.ascontiguousarray(label, dtype=np.float64)
    sw = None if sample_weight is None else np.ascontiguousarray(sample_weight, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    g = np.zeros(mat.n + 1)
    out = _dbl()
    L = mat.ctx.L
    if loss is None:
        st = L.fvg_logreg_eval(mat.ctx.h, mat.h, _fmt(fmt), _dt(storage), _ptr(label), _ptr(sw), _ptr(w), float(b),
                               int(intercept), _ptr(g), C.byref(out))
    else:
        st = L.fvg_glm_eval(mat.ctx.h, mat.h, _fmt(fmt), _dt(storage), LOSS[loss] if isinstance(loss, str) else loss,
                            float(epsilon), _ptr(label), _ptr(sw), _ptr(w), float(b), int(intercept), _ptr(g),
                            C.byref(out))
    mat.ctx.check(st)
    return g, out.value


glm_eval = logreg_eval


def predict_probability(mat: Matrix, w, b=0.0):
    w = np.ascontiguousarray(w, dtype=np.float64)
    out = np.zeros(mat.m)
    mat.ctx.check(mat.ctx.L.fvg_logreg_predict_probability(mat.ctx.h, mat.h, _ptr(w), float(b), _ptr(out)))
    return out


def bf16_bits(x) -> np.ndarray:
    """Round-to-nearest-even FP64/FP32 → bf16 bit patterns (uint16)."""
    f = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    rounding = ((f >> 16) & 1) + 0x7FFF
    return ((f + rounding) >> 16).astype(np.uint16)
