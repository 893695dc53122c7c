"""Loading and materialising the golden fixtures of tests/golden/.

A case describes one VSIPL fftm call (kind, precision, plan arguments and the
input/output views), or -- with "single" set -- one single-FFT call on
vectors, stored as a one-row view (col_length 1, the vector's stride as
row_stride); "shared" puts y in x's block.  `build_case` recreates its blocks from the stored seeds
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
_fft_meta = None
_fft_arrays = None


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


def fft_meta():
    global _fft_meta
    if _fft_meta is None:
        with open(os.path.join(GOLDEN, "fft_cases.json")) as f:
            _fft_meta = json.load(f)
    return _fft_meta


def fft_arrays():
    global _fft_arrays
    if _fft_arrays is None:
        _fft_arrays = dict(np.load(os.path.join(GOLDEN, "fft_cases.npz")))
    return _fft_arrays


def fft_cases():
    return fft_meta()["cases"]


def fft_kats():
    with open(os.path.join(GOLDEN, "fft_kat.json")) as f:
        return json.load(f)


def arrays_of(case):
    return fft_arrays() if case.get("single") else arrays()


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
    A = arrays_of(case)
    if kind in ("ccop", "ccip"):
        x = make_cview(case["x"], dtype)
        if case.get("stored_input"):
            _load_input(x, A[case["id"] + "__in"])
        if kind == "ccip" or case.get("alias"):
            return x, None
        if case.get("shared"):
            ys = case["y"]
            return x, O.CView(x.buf, ys["off"], ys["cs"], ys["cl"], ys["rs"], ys["rl"], x.im)
        return x, make_cview(case["y"], dtype)
    if kind == "rcop":
        x = make_rview(case["x"], dtype)
        if case.get("stored_input"):
            x.buf[:] = A[case["id"] + "__in"]
        return x, make_cview(case["y"], dtype)
    z = make_cview(case["x"], dtype)
    if case.get("stored_input"):
        _load_input(z, A[case["id"] + "__in"])
    return z, make_rview(case["y"], dtype)


def output_block(case, x, y):
    if case["kind"] == "ccip" or case.get("alias") or case.get("shared"):
        return block_arrays(x)
    return block_arrays(y)


def sha256(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def reference_values(case):
    """(indices, values) of the reference output block available in the fixture."""
    A = arrays_of(case)
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


# ------------------------------------------------------------------ single-FFT known-answer tests
def cplx(pairs) -> np.ndarray:
    a = np.asarray(pairs, np.float64).reshape(-1, 2)
    return a[:, 0] + 1j * a[:, 1]


def kat_views(t):
    """(x view, y view or None) of a single-FFT known-answer test with its
    input in place: dense vectors in blocks of `block` elements, or -- for
    ccfftop_sc -- x and y bound on one block at (offset, stride) xbind / ybind."""
    dtype = np.float32 if t["prec"] == "f" else np.float64
    n, kind = t["n"], t["kind"]
    xin = t["x"] if isinstance(t["x"], np.ndarray) else cplx(t["x"])
    if kind == "rcop":
        x = O.RView(np.zeros(t["block"], dtype), 0, n, 1, 1, n)
        x.set(np.asarray(xin).real[None, :])
        z = O.CView(np.zeros(2 * t["block"], dtype), 0, n // 2 + 1, 1, 1, n // 2 + 1)
        return x, z
    if kind == "crop":
        z = O.CView(np.zeros(2 * t["block"], dtype), 0, n // 2 + 1, 1, 1, n // 2 + 1)
        z.set(np.asarray(xin)[None, :])
        y = O.RView(np.zeros(t["block"], dtype), 0, n, 1, 1, n)
        return z, y
    if t.get("shared"):
        buf = np.zeros(2 * t["block"], dtype)
        xo, xs = t["xbind"]
        yo, ys = t["ybind"]
        x = O.CView(buf, xo, n * xs, 1, xs, n)
        y = O.CView(buf, yo, n * ys, 1, ys, n)
        x.set(np.asarray(xin)[None, :])
        return x, y
    x = O.CView(np.zeros(2 * t["block"], dtype), 0, n, 1, 1, n)
    x.set(np.asarray(xin)[None, :])
    if kind == "ccip":
        return x, None
    return x, O.CView(np.zeros(2 * t["block"], dtype), 0, n, 1, 1, n)


def kat_run(t, plan):
    """Run a known-answer test through `plan`, any object with the single-FFT
    methods ccfftop / ccfftip / rcfftop / crfftop taking one-row views;
    returns the output vector (complex128)."""
    x, y = kat_views(t)
    k = t["kind"]
    if k == "ccop":
        plan.ccfftop(x, y)
        return y.get()[0]
    if k == "ccip":
        plan.ccfftip(x)
        return x.get()[0]
    if k == "rcop":
        plan.rcfftop(x, y)
        return y.get()[0]
    plan.crfftop(x, y)
    return y.get()[0].astype(np.complex128)


# ------------------------------------------------------------------ k-omega pipeline cases
_kw_meta = None
_kw_arrays = None


def komega_cases():
    global _kw_meta
    if _kw_meta is None:
        with open(os.path.join(GOLDEN, "komega_cases.json")) as f:
            _kw_meta = json.load(f)
    return _kw_meta["cases"]


def komega_arrays():
    global _kw_arrays
    if _kw_arrays is None:
        _kw_arrays = dict(np.load(os.path.join(GOLDEN, "komega_cases.npz")))
    return _kw_arrays


def komega_views(c):
    """Fresh (data, freq, gram, scale) of a k-omega case: data Nsens x Nts rows
    of pitch `pitch` at offset `doff` (host-exact U[-1,1) stream, seed
    1000 + seed), freq Nsens x (Nts/2 + 1) interleaved, column-major ("col",
    as kw.c creates it) or row-major, gram the same shape at offset `goff`
    holding |U[-1,1)| (seed 2000 + seed)."""
    Ns, Nt, pitch, doff, goff = c["Nsens"], c["Nts"], c["pitch"], c["doff"], c["goff"]
    Nf = Nt // 2 + 1
    data = O.RView(O.fill(doff + Ns * pitch, 1000 + c["seed"], 0, np.float32), doff, pitch, Ns, 1, Nt)
    fbuf = np.zeros(2 * Ns * Nf, np.float32)
    freq = O.CView(fbuf, 0, 1, Ns, Ns, Nf) if c["freq"] == "col" else O.CView(fbuf, 0, Nf, Ns, 1, Nf)
    gbuf = np.abs(O.fill(goff + Ns * Nf, 2000 + c["seed"], 0, np.float32))
    gram = O.RView(gbuf, goff, 1, Ns, Ns, Nf) if c["gram"] == "col" else O.RView(gbuf, goff, Nf, Ns, 1, Nf)
    return data, freq, gram, np.float32(c["scale"])


def komega_reference(c, name):
    """(indices, values) of the reference's output block `name` (data_out,
    freq_out or gram_out) available in the fixture."""
    A = komega_arrays()
    k = c["id"] + "__" + name
    if k in A:
        return np.arange(A[k].size), A[k]
    return A[k + "__idx"], A[k + "__val"]
