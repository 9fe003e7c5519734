"""Synthetic power-law sparse logistic-regression data (host generator).

The reference's own benchmark data (Criteo CTR) is not available, so seeded
synthetic inputs with the shapes and value distributions of the benchmark
configurations stand in for it.  The generator is C++ (synth.cpp), threaded,
and deterministic per row, so the GPU path and the CPU baseline read the same
bytes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_OUT = os.path.join(os.path.dirname(_HERE), "_build")
LIB = os.path.join(_OUT, "libfvg_synth.so")
_lib = None


class SynCfg(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("seed", C.c_uint64), ("len_kind", C.c_int32),
                ("lam", C.c_double), ("s_len", C.c_double), ("len_cap", C.c_int64), ("total_nnz", C.c_int64),
                ("col_kind", C.c_int32), ("s_col", C.c_double), ("val_kind", C.c_int32),
                ("val_sigma", C.c_double), ("wstar_sd", C.c_double), ("nthreads", C.c_int32)]


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "synth.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        os.makedirs(_OUT, exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", src,
                        "-o", LIB + ".tmp"], check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.syn_lengths.argtypes = [C.POINTER(SynCfg), C.c_void_p]
        _lib.syn_lengths.restype = C.c_int64
        _lib.syn_fill.argtypes = [C.POINTER(SynCfg), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.syn_fill.restype = C.c_int
    return _lib


@dataclass
class Spec:
    m: int
    n: int
    seed: int = 0
    len_kind: str = "poisson"   # "poisson" (1+Poisson(lam)) | "zipf" (rescaled to nnz)
    lam: float = 39.0
    s_len: float = 1.3
    len_cap: int = 0
    total_nnz: int = 0
    col_kind: str = "zipf"      # "zipf" | "uniform"
    s_col: float = 1.1
    val_kind: str = "absnormal"  # "absnormal" | "normal" | "lognormal"
    val_sigma: float = 0.5
    wstar_sd: float = 1.0 / np.sqrt(40.0)
    labels: bool = True


def generate(spec: Spec, nthreads: int = 0):
    """Returns (off int32[m+1], idx int32[nnz], val float64[nnz], label float64[m] or None)."""
    c = SynCfg(spec.m, spec.n, spec.seed, 0 if spec.len_kind == "poisson" else 1, spec.lam, spec.s_len,
               spec.len_cap, spec.total_nnz, 0 if spec.col_kind == "zipf" else 1, spec.s_col,
               {"absnormal": 0, "normal": 1, "lognormal": 2}[spec.val_kind], spec.val_sigma, spec.wstar_sd,
               nthreads)
    L = lib()
    lens = np.zeros(spec.m, dtype=np.int32)
    nnz = L.syn_lengths(C.byref(c), lens.ctypes.data_as(C.c_void_p))
    if nnz < 0 or nnz >= 2 ** 31:
        raise ValueError(f"bad synthetic config (nnz={nnz})")
    off = np.zeros(spec.m + 1, dtype=np.int32)
    idx = np.zeros(max(nnz, 1), dtype=np.int32)
    val = np.zeros(max(nnz, 1), dtype=np.float64)
    label = np.zeros(spec.m, dtype=np.float64) if spec.labels else None
    rc = L.syn_fill(C.byref(c), lens.ctypes.data_as(C.c_void_p), off.ctypes.data_as(C.c_void_p),
                    idx.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p),
                    None if label is None else label.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise ValueError("synthetic fill failed")
    return off, idx[:nnz], val[:nnz], label


# The benchmark configurations (seed 0), restated as concrete generators.
def logreg_100k_20k(scale: float = 1.0) -> Spec:
    """L2 logistic regression, 100,000 x 20,000, nnz/row 1+Poisson(39), Zipf(1.1) columns, |N(0,1)| values."""
    return Spec(m=int(100_000 * scale), n=20_000, lam=39.0, col_kind="zipf", s_col=1.1, val_kind="absnormal",
                wstar_sd=1.0 / np.sqrt(40.0))


def spmv_2m_80m(scale: float = 1.0) -> Spec:
    """SpMV kernel bench, 2,000,000^2, 80M nonzeros, Zipf(1.3) row lengths (cap 20,000), uniform columns."""
    m = int(2_000_000 * scale)
    return Spec(m=m, n=m, len_kind="zipf", s_len=1.3, len_cap=20_000, total_nnz=int(80_000_000 * scale),
                col_kind="uniform", val_kind="normal", labels=False)


def logreg_10m_1m(scale: float = 1.0) -> Spec:
    """Mixed-precision LR at scale: 10,000,000 x 1,000,000, nnz/row 1+Poisson(59), Zipf(1.1), lognormal(0,0.5)."""
    return Spec(m=int(10_000_000 * scale), n=max(1000, int(1_000_000 * scale)), lam=59.0, col_kind="zipf",
                s_col=1.1, val_kind="lognormal", val_sigma=0.5, wstar_sd=1.0 / np.sqrt(60.0))


def regpath_datasets(count: int = 16, scale: float = 1.0):
    """Batched regularisation path: `count` datasets with 500,000 columns,
    rows ~ U[10,000, 2,000,000] (seeded), nnz/row 1+Poisson(49), Zipf(1.2)
    columns, |N(0,1)| values; dataset i uses seed 100 + i."""
    rng = np.random.default_rng(2024)
    rows = rng.integers(10_000, 2_000_001, size=16)[:count]
    return [Spec(m=max(100, int(r * scale)), n=max(1000, int(500_000 * scale)), seed=100 + i, lam=49.0,
                 col_kind="zipf", s_col=1.2, val_kind="absnormal", wstar_sd=1.0 / np.sqrt(50.0))
            for i, r in enumerate(rows)]
