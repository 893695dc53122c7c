"""Running golden cases through the GPU library's C ABI (test helper)."""
from __future__ import annotations

import numpy as np

import golden_cases as G
import jvsip_gb300 as J
import pyoracle as O

KIND = dict(ccop=J.KIND_CCOP, ccip=J.KIND_CCIP, rcop=J.KIND_RCOP, crop=J.KIND_CROP)


def _view(b, v, single):
    if single:
        # a one-row view stands for the vector of its row
        return b.vview(v.off, v.row_stride, v.row_length)
    return b.view(v.off, v.col_stride, v.col_length, v.row_stride, v.row_length)


def _bind(v, admit, single=False):
    b = J.CBlock(v.buf, v.im) if isinstance(v, O.CView) else J.RBlock(v.buf)
    view = _view(b, v, single)
    if admit:
        b.admit(True)
    return b, view


def run_case_gpu(case, admit: bool):
    """Run a golden case through the library; returns (out_block, in_block_before)."""
    x, y = G.build_case(case)
    before = G.output_block(case, x, y).copy()
    single = bool(case.get("single"))
    bx, vx = _bind(x, admit, single)
    if y is None:
        by, vy = bx, vx
    elif case.get("shared"):
        by, vy = bx, _view(bx, y, single)
    else:
        by, vy = _bind(y, admit, single)
    if single:
        p = J.FFT(KIND[case["kind"]], case["N"], case["scale"], case["dir"], G.dtype_of(case))
    else:
        p = J.FFTM(KIND[case["kind"]], case["M"], case["N"], case["scale"], case["dir"], case["major"],
                   G.dtype_of(case))
    try:
        k = case["kind"]
        if single:
            if k == "ccop":
                p.ccfftop(vx, vx if case.get("alias") else vy)
            elif k == "ccip":
                p.ccfftip(vx)
            elif k == "rcop":
                p.rcfftop(vx, vy)
            else:
                p.crfftop(vx, vy)
        elif k == "ccop":
            p.ccfftmop(vx, vx if case.get("alias") else vy)
        elif k == "ccip":
            p.ccfftmip(vx)
        elif k == "rcop":
            p.rcfftmop(vx, vy)
        else:
            p.crfftmop(vx, vy)
    finally:
        for b in {id(bx): bx, id(by): by}.values():
            if admit:
                b.release(True)
        for v in {id(vx): vx, id(vy): vy}.values():
            v.destroy()
        for b in {id(bx): bx, id(by): by}.values():
            b.destroy()
        p.destroy()
    return G.output_block(case, x, y), before


def view_mask(case):
    """Boolean mask over the output block: True where the output view writes."""
    x, y = G.build_case(case)
    out_spec = case["x"] if (case["kind"] == "ccip" or case.get("alias")) else case["y"]
    dtype = G.dtype_of(case)
    if case["kind"] == "crop":
        v = G.make_rview(out_spec, dtype)
        m = np.zeros(v.buf.size, bool)
        m[v.index()] = True
        return m
    v = G.make_cview(out_spec, dtype)
    if case.get("shared"):
        v = G.make_cview(dict(case["x"]) | {k: out_spec[k] for k in ("off", "cs", "cl", "rs", "rl")}, dtype)
    idx = v.index()
    if v.split:
        m = np.zeros(2 * v.buf.size, bool)
        m[idx] = True
        m[v.buf.size + idx] = True
        return m
    m = np.zeros(v.buf.size, bool)
    m[2 * idx] = True
    m[2 * idx + 1] = True
    return m


def tolerance(case):
    return (1e-6 if case["prec"] == "f" else 1e-14) * G.log2n(case)
