"""Loading and materialising the golden fixtures of tests/golden/.

A case describes one VSIPL fftm call (kind, precision, plan arguments and the
input/output views).  `build_case` recreates its blocks from the stored seeds
(or the stored inputs); `check_output` compares an output block with the
reference's, whole or through the stored sample.
"""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

import pyoracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_meta = None
_arrays = None


def meta():
    global _meta
    if _meta is None:
        with open(os.path.join(GOLDEN, "fftm_cases.json")) as f:
            _meta = json.load(f)
    return _meta


def arrays():
    global _arrays
    if _arrays is None:
        _arrays = dict(np.load(os.path.join(GOLDEN, "fftm_cases.npz")))
    return _arrays


def cases():
    return meta()["cases"]


def ref_tests():
    with open(os.path.join(GOLDEN, "ref_testcases.json")) as f:
        return json.load(f)


def dtype_of(case):
    return np.float32 if case["prec"] == "f" else np.float64


def make_cview(spec, dtype):
    n = spec["block"]
    if spec["split"]:
        buf = np.zeros(n, dtype)
        im = np.zeros(n, dtype)
        if spec["seed"] is not None:
            buf[:] = O.fill(n, spec["seed"], spec["dist"], dtype)
            im[:] = O.fill(n, spec["seed"] + 1, spec["dist"], dtype)
    else:
        buf = np.zeros(2 * n, dtype)
        im = None
        if spec["seed"] is not None:
            buf[:] = O.fill(2 * n, spec["seed"], spec["dist"], dtype)
    return O.CView(buf, spec["off"], spec["cs"], spec["cl"], spec["rs"], spec["rl"], im)


def make_rview(spec, dtype):
    buf = np.zeros(spec["block"], dtype)
    if spec["seed"] is not None:
        buf[:] = O.fill(spec["block"], spec["seed"], spec["dist"], dtype)
    return O.RView(buf, spec["off"], spec["cs"], spec["cl"], spec["rs"], spec["rl"])


def block_arrays(v):
    if isinstance(v, O.CView) and v.split:
        return np.concatenate([v.buf, v.im])
    return v.buf.copy()


def _load_input(view, stored):
    if isinstance(view, O.CView) and view.split:
        n = view.buf.size
        view.buf[:] = stored[:n]
        view.im[:] = stored[n:]
    else:
        view.buf[:] = stored


def build_case(case):
    """Return (x_view, y_view_or_None) with the case's input data in place."""
    dtype = dtype_of(case)
    kind = case["kind"]
    if kind in ("ccop", "ccip"):
        x = make_cview(case["x"], dtype)
        if case.get("stored_input"):
            _load_input(x, arrays()[case["id"] + "__in"])
        if kind == "ccip" or case.get("alias"):
            return x, None
        return x, make_cview(case["y"], dtype)
    if kind == "rcop":
        x = make_rview(case["x"], dtype)
        if case.get("stored_input"):
            x.buf[:] = arrays()[case["id"] + "__in"]
        return x, make_cview(case["y"], dtype)
    z = make_cview(case["x"], dtype)
    if case.get("stored_input"):
        _load_input(z, arrays()[case["id"] + "__in"])
    return z, make_rview(case["y"], dtype)


def output_block(case, x, y):
    if case["kind"] == "ccip" or case.get("alias"):
        return block_arrays(x)
    return block_arrays(y)


def sha256(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def reference_values(case):
    """(indices, values) of the reference output block available in the fixture."""
    A = arrays()
    if case["stored_output"]:
        v = A[case["id"] + "__out"]
        return np.arange(v.size), v
    return A[case["id"] + "__sidx"], A[case["id"] + "__sval"]


def log2n(case):
    n = case["N"] if (case["major"] == 0) else case["M"]
    if case["kind"] in ("rcop", "crop"):
        n = max(n // 2, 2)
    return max(1.0, float(np.log2(max(n, 2))))


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.sqrt(np.sum(b * b))
    num = np.sqrt(np.sum((a - b) ** 2))
    return float(num / den) if den > 0 else float(num)
