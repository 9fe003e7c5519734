"""Host check of the integer FP64 -> (FP32, BF16 residual) split
(frovedis_gb300/csrc/split_bits.h) that builds the split-storage planes:
hi must be the FP32 rounding of x and lo the BF16 rounding (nearest, ties
to even) of the exact x - hi, bit for bit, over random values of every
exponent the fast path takes and the rounding boundaries (FP32 ties, carries
into the next binade, overflow, BF16 ties)."""
import math
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bf16_bits(r):
    """BF16 rounding (nearest, ties to even) of a finite double, as bits."""
    if r == 0.0:
        return 0x8000 if math.copysign(1.0, r) < 0 else 0
    sign = 0x8000 if r < 0 else 0
    m, e = math.frexp(abs(r))          # |r| = m * 2^e, m in [0.5, 1)
    q = round(m * 256.0)               # exact product; round() is half-to-even
    if q == 256:
        q, e = 128, e + 1
    return sign | ((e - 1 + 127) << 7) | (q & 127)


def _ref(x):
    with np.errstate(over="ignore"):  # values that round past the FP32 range
        h = np.float32(x)
    hb = int(h.view(np.uint32))
    if np.isinf(h):
        return hb, 0
    return hb, _bf16_bits(float(x) - float(h))


def _values(rng):
    vals = []
    for e in range(-60, 128):
        m = rng.uniform(1.0, 2.0, 6)
        s = rng.choice([-1.0, 1.0], 6)
        vals += list(s * m * 2.0 ** e)
    top = rng.integers(0, 1 << 23, 400)
    for t in top:
        for low in (1 << 28, (1 << 28) - 1, (1 << 28) + 1, 0, 1, (1 << 29) - 1, 3 << 26, 5 << 20):
            e = int(rng.integers(-60, 128))
            bits = ((e + 1023) << 52) | (int(t) << 29) | low
            vals.append(float(np.array([bits], np.uint64).view(np.float64)[0]))
    for e in (0, 5, -60, 127):  # the largest fraction rounding up: next binade (or infinity)
        for low in ((1 << 28) + 1, 1 << 28):
            bits = ((e + 1023) << 52) | (((1 << 23) - 1) << 29) | low
            vals.append(float(np.array([bits], np.uint64).view(np.float64)[0]))
            vals.append(-vals[-1])
    for t in range(0, 64):  # residuals whose BF16 rounding is a tie
        for low in ((0x81 << 8) | 0x80, (0x82 << 8) | 0x80, 0x180, 0x3):
            bits = ((10 + 1023) << 52) | (t << 29) | low
            vals.append(float(np.array([bits], np.uint64).view(np.float64)[0]))
    return np.array(vals, np.float64)


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    d = tmp_path_factory.mktemp("split_bits")
    out = str(d / "split_bits_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I",
           os.path.join(ROOT, "frovedis_gb300", "csrc"), os.path.join(ROOT, "tests", "cpp", "split_bits_check.cpp"),
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_split_bits_match_exact_rounding(exe, tmp_path):
    x = _values(np.random.default_rng(5))
    inp, outp = tmp_path / "x.bin", tmp_path / "o.bin"
    x.tofile(inp)
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    o = np.fromfile(outp, np.uint32).reshape(-1, 3)
    assert o.shape[0] == x.size
    assert o[:, 2].all()  # every value lies in the fast path's range
    bad = [(float(v), int(a), int(b), _ref(v)) for v, a, b in zip(x, o[:, 0], o[:, 1]) if (int(a), int(b)) != _ref(v)]
    assert not bad, bad[:5]


def test_split_bits_declines_outside_range(exe, tmp_path):
    x = np.array([0.0, -0.0, 5e-324, 2.0 ** -61, 2.0 ** -1022, 2.0 ** 128, -2.0 ** 200, np.inf, -np.inf, np.nan])
    inp, outp = tmp_path / "x.bin", tmp_path / "o.bin"
    x.tofile(inp)
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    o = np.fromfile(outp, np.uint32).reshape(-1, 3)
    assert not o[:, 2].any()
