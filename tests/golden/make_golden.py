"""Regenerates tests/golden/golden.json from the reference's own fixtures.

Reads (never writes) the reference tree whose path is the required first
argument (``python tests/golden/make_golden.py <frovedis source tree>``) and
extracts, as data:

* the tutorial SpMV fixture ``doc/tutorial/src/tut3.2.1-1/data`` (also as
  raw text, for the loaders) and its
  documented result (``doc/tutorial/tutorial.md``, block after "The result of
  the program should be"), also used for ELL/JDS/hybrid by ``tut3.2.2``;
* the binary CRS fixture ``doc/tutorial/src/tut3.2.1-2/data_binary``
  (nums/val/idx/off/type, also as raw files) and its documented transpose (tutorial.md, block
  after "It should be:");
* the glm fixtures ``test/ml/test2.1-1`` (SGD) and ``test/ml/test2.1-2``
  (L-BFGS) of logistic regression, ``test1.1-*`` (linear regression),
  ``test1.2-*`` (lasso), ``test1.3-*`` (ridge) and ``test2.2-*`` (SVM), each
  ``-1`` SGD and ``-2`` L-BFGS: data/label text, the trainer, the
  hyper-parameters and expected outputs written in their ``test.cc``, plus
  the raw bytes-per-line layout needed to reproduce the 4-rank row split of
  ``mpirun -np 4`` (test/ml/exec.sh).

Run:  python tests/golden/make_golden.py [/path/to/reference]
"""
import json
import os
import re
import struct
import sys


def parse_crs_text(text):
    """0-based "col:val" lines (crs_matrix.hpp:664-690)."""
    off, idx, val = [0], [], []
    for line in text.split("\n")[:-1] if text.endswith("\n") else text.split("\n"):
        for item in line.split():
            c, v = item.split(":")
            idx.append(int(c))
            val.append(float(v))
        off.append(len(idx))
    ncol = (max(idx) + 1) if idx else 0
    return dict(m=len(off) - 1, n=ncol, off=off, idx=idx, val=val)


def indented_block_after(md, marker, start=0):
    pos = md.index(marker, start)
    lines = md[pos:].split("\n")[1:]
    out, started = [], False
    for ln in lines:
        if ln.startswith("    ") and ln.strip():
            out.append(ln.strip())
            started = True
        elif started and not ln.strip():
            break
        elif started:
            break
    return out


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <path of the frovedis source tree>")
    ref = sys.argv[1]
    tut = os.path.join(ref, "doc", "tutorial")
    md = open(os.path.join(tut, "tutorial.md")).read()
    g = {}

    # --- tutorial SpMV (tut3.2.1-1, tut3.2.2) ---
    data = open(os.path.join(tut, "src", "tut3.2.1-1", "data")).read()
    g["tut_spmv"] = parse_crs_text(data)
    g["tut_spmv"]["raw_text"] = data  # the file itself, for the loader tests
    g["tut_spmv"]["expected_y_ones"] = [
        float(v) for v in indented_block_after(md, "The result of the program should be:",
                                               md.index("src/tut3.2.1-1/tut.cc"))]

    # --- tutorial binary CRS + transpose (tut3.2.1-2) ---
    d = os.path.join(tut, "src", "tut3.2.1-2", "data_binary")
    nums = open(os.path.join(d, "nums")).read().split()
    types = open(os.path.join(d, "type")).read().split()
    assert types == ["double", "uint64_t", "uint64_t"], types
    raw_val = open(os.path.join(d, "val"), "rb").read()
    raw_idx = open(os.path.join(d, "idx"), "rb").read()
    raw_off = open(os.path.join(d, "off"), "rb").read()
    val = list(struct.unpack("<%dd" % (len(raw_val) // 8), raw_val))
    idx = list(struct.unpack("<%dQ" % (len(raw_idx) // 8), raw_idx))
    off = list(struct.unpack("<%dQ" % (len(raw_off) // 8), raw_off))
    g["tut_binary"] = dict(m=int(nums[0]), n=int(nums[1]), off=off, idx=idx, val=val, type=types)
    g["tut_binary"]["raw_files"] = {  # the directory itself, for the loader tests
        "nums": open(os.path.join(d, "nums")).read(), "type": open(os.path.join(d, "type")).read(),
        "val": raw_val.hex(), "idx": raw_idx.hex(), "off": raw_off.hex()}
    tr = indented_block_after(md, "It should be:", md.index("src/tut3.2.1-2/tut.cc"))
    g["tut_binary"]["expected_transpose_text"] = tr

    # --- glm tests ---
    trainers = {"logistic_regression": ("logistic", None), "linear_regression": ("linear", "ZERO"),
                "lasso": ("linear", "L1"), "ridge_regression": ("linear", "L2"), "svm": ("hinge", None)}
    for name in ("test2.1-1", "test2.1-2", "test1.1-1", "test1.1-2", "test1.2-1", "test1.2-2", "test1.3-1",
                 "test1.3-2", "test2.2-1", "test2.2-2"):
        td = os.path.join(ref, "test", "ml", name)
        raw = open(os.path.join(td, "data"), "rb").read()
        src = open(os.path.join(td, "test.cc")).read()
        labels = [float(x) for x in open(os.path.join(td, "label")).read().split()]
        ent = parse_crs_text(raw.decode())
        ent["label"] = labels
        ent["data_bytes_hex"] = raw.hex()
        for key in ("num_iteration", "alpha", "minibatch_fraction", "regParam", "hist_size"):
            mm = re.search(r"\b%s\s*=\s*([0-9.eE+-]+)\s*;" % key, src)
            if mm:
                ent[key] = float(mm.group(1))
        mm = re.search(r"bool intercept\s*=\s*(true|false)", src)
        ent["intercept"] = mm.group(1) == "true"
        mm = re.search(r"auto model = (\w+)_with_(sgd|lbfgs)::train", src)
        ent["trainer"] = mm.group(1) + "_with_" + mm.group(2)
        ent["loss"], reg = trainers[mm.group(1)]
        mm = re.search(r"RegType rt\s*=\s*(\w+)", src)
        ent["reg_type"] = mm.group(1) if mm else reg
        for key in ("expected_out", "expected_out_p", "expected_out_pb"):
            # the live (not commented-out) initialiser
            mm = re.search(r"(?m)^\s*std::vector<double>\s+" + key + r"\s*=\s*\{([^}]*)\}", src)
            if mm:
                ent[key] = [float(x) for x in mm.group(1).split(",")]
        mm = re.search(r"double tol\s*=\s*([0-9.eE+-]+)", src)
        ent["rms_tol"] = float(mm.group(1))
        ent["solver"] = "sgd" if "with_sgd" in src else "lbfgs"
        g[name] = ent
    ex = open(os.path.join(ref, "test", "ml", "exec.sh")).read()
    mm = re.search(r"mpirun\s+-np\s+(\d+)", ex)
    g["glm_test_ranks"] = int(mm.group(1))

    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(out, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    main()
