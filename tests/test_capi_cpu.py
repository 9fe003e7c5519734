"""CPU-only checks of the C-ABI library: it builds for sm_103a, loads without
a GPU, exports every entry point include/fvg.h declares, and fails cleanly
(status, no crash) when no GPU is present."""
import ctypes
import os
import re

import pytest

import frovedis_gb300 as fv
from frovedis_gb300 import build as fb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "fvg.h")).read()
    return re.findall(r"FVG_API\s+[\w\s\*]+?\b(fvg_\w+)\s*\(", src)


def test_library_builds_and_loads():
    path = fb.build()
    assert os.path.exists(path)
    ctypes.CDLL(path)


def test_exports_match_header():
    names = _declared()
    assert len(names) >= 25
    L = ctypes.CDLL(fb.build())
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(fv.EXPORTS)


def test_glm_params_defaults_match_reference():
    # logistic_regression_with_lbfgs.hpp:8-25 / glm_config defaults (common.hpp:33-47)
    p = fv.glm_params()
    assert p.num_iteration == 1000 and p.alpha == 0.01 and p.hist_size == 10
    assert p.reg_param == 0.01 and p.reg_type == 0 and p.intercept == 0
    assert p.convergence_tol == 0.001 and p.mat_type == 0 and p.mini_batch_fraction == 1.0


def test_null_arguments_are_rejected_without_gpu():
    L = fv.load()
    out = ctypes.c_void_p()
    assert L.fvg_ctx_create(0, None) == 1  # FVG_ERR_INVALID_ARG
    assert L.fvg_ctx_synchronize(None) == 1
    assert L.fvg_matrix_info(None, None, None, None) == 1
    assert L.fvg_spmv(None, None, 0, 0, 0, None, None, 0) == 1
    assert L.fvg_logreg_lbfgs(None, None, None, None, None, None, None, None, None) == 1
    # a missing GPU is a status code, not a crash
    rc = L.fvg_ctx_create(0, ctypes.byref(out))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert rc != 0 and not out.value


def test_bf16_rounding_helper():
    import numpy as np
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3])
    b = fv.bf16_bits(x)
    back = (b.astype(np.uint32) << 16).view(np.float32)
    assert np.all(np.abs(back - x) <= np.abs(x) * 2 ** -8)
