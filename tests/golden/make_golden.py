"""Generate the golden fixtures under tests/golden/ from the jvsip reference.

Run where the reference sources are, with JVSIP_REFERENCE naming the
reference checkout (the directory holding c_VSIP_src/ and c_VSIP_testing/):

    JVSIP_REFERENCE=<checkout> python tests/golden/make_golden.py

It writes
  ref_testcases.json  -- the reference's own fftm known-answer tests, parsed
                         from c_VSIP_testing/ccfftm{op,ip}_{f,d}.h: the 8x4
                         strided/offset input, the create/bind arguments and
                         the 4-decimal expected outputs;
  fftm_cases.json     -- a catalogue of seeded cases (sizes, views, strides,
  fftm_cases.npz         directions, scales, split/interleaved, in-place,
                         aliasing, real<->complex) with the output blocks the
                         reference library (oracle/_ref/libvsip_ref.so, built
                         from the reference sources by oracle/Makefile.ref)
                         produced for them.

Inputs are regenerated from (seed, dist) by the shared SplitMix64 stream
(oracle/fftm_oracle.c); dist 0 (U[-1,1)) uses integer arithmetic and one exact
scaling only, so it is bit-identical on every host and is used for every
case whose input is not stored.  Cases with N(0,1) inputs store them.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import pyoracle as O  # noqa: E402
import pyref as R  # noqa: E402

REF = os.environ.get("JVSIP_REFERENCE", "")
if not REF or not os.path.isdir(REF):
    sys.exit("set JVSIP_REFERENCE to the jvsip reference checkout (the directory holding c_VSIP_src/)")
# outputs up to this size are stored whole; larger ones as a hash plus a sample
FULL_OUTPUT_BYTES = 40 * 1024


# ------------------------------------------------------------------ reference tests
def parse_ref_tests():
    cases = []
    for fname in ("ccfftmop_f.h", "ccfftmip_f.h", "ccfftmop_d.h", "ccfftmip_d.h"):
        path = os.path.join(REF, "c_VSIP_testing", fname)
        text = open(path).read()
        prec = fname[-3]
        kind = "ccop" if "ccfftmop" in fname else "ccip"
        blocks = re.split(r"\{\s*/\*\s*8 by 4\s*\*/", text)[1:]
        line0 = 1
        for blk in blocks:
            arrays = {}
            for name in ("rdta", "idta", "rdta0", "idta0"):
                m = re.search(r"\b%s\[32\]\s*=\s*\{([^}]*)\}" % name, blk)
                arrays[name] = [float(v) for v in m.group(1).replace("\n", " ").split(",")]
            m = re.search(r"vsip_ccfftm(?:op|ip)_create_[fd]\(([^)]*)\)", blk)
            args = [a.strip() for a in m.group(1).split(",")]
            M, N = int(args[0]), int(args[1])
            scale = float(eval(args[2]))
            d = -1 if args[3] == "VSIP_FFT_FWD" else 1
            major = 0 if args[4] == "VSIP_ROW" else 1
            m = re.search(r"vsip_cmbind_[fd]\(block,([^)]*)\)", blk)
            o, cs, cl, rs, rl = [int(v) for v in m.group(1).split(",")]
            line = text[: text.index(blk)].count("\n") + 1
            cases.append(dict(file="c_VSIP_testing/" + fname, line=line, prec=prec, kind=kind,
                              M=M, N=N, scale=scale, dir=d, major=major, block=1000,
                              bind=[o, cs, cl, rs, rl],
                              x_re=arrays["rdta"], x_im=arrays["idta"],
                              gold_re=arrays["rdta0"], gold_im=arrays["idta0"], tol_meansq=2e-4))
            line0 = line
    return cases


# ------------------------------------------------------------------ seeded cases
def cview_spec(M, N, major=0, off=0, cs=None, rs=None, block=None, split=False, seed=None, dist=0):
    """Complex view spec. Default: dense VSIPL-created layout for `major`."""
    if cs is None or rs is None:
        cs, rs = (N, 1) if major == 0 else (1, M)
    if block is None:
        idx_max = off + max(0, (M - 1) * cs) + max(0, (N - 1) * rs)
        idx_min = off + min(0, (M - 1) * cs) + min(0, (N - 1) * rs)
        assert idx_min >= 0
        block = idx_max + 1
    return dict(block=block, split=split, off=off, cs=cs, cl=M, rs=rs, rl=N, seed=seed, dist=dist)


def rview_spec(M, N, major=0, off=0, cs=None, rs=None, block=None, seed=None, dist=0):
    if cs is None or rs is None:
        cs, rs = (N, 1) if major == 0 else (1, M)
    if block is None:
        block = off + max(0, (M - 1) * cs) + max(0, (N - 1) * rs) + 1
    return dict(block=block, off=off, cs=cs, cl=M, rs=rs, rl=N, seed=seed, dist=dist)


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


def catalogue():
    C = []

    def cc(cid, prec, kind, M, N, major, d, scale, x, y=None, alias=False):
        C.append(dict(id=cid, prec=prec, kind=kind, M=M, N=N, major=major, dir=d, scale=scale,
                      x=x, y=y, alias=alias))

    # configuration 1 (plain 64 x 1024 ROW, U[-1,1) seed 1) and its inverse round trip
    for p in ("f", "d"):
        cc(f"cfg1_{p}_fwd", p, "ccop", 64, 1024, 0, -1, 1.0, cview_spec(64, 1024, seed=1), cview_spec(64, 1024))
        cc(f"cfg1_{p}_inv", p, "ccop", 64, 1024, 0, 1, 1.0 / 1024, cview_spec(64, 1024, seed=1), cview_spec(64, 1024))
    # configuration 2 sample: 1000-point transforms down 64 columns of a row-major 1000 x 64 matrix
    cc("cfg2col_f", "f", "ccop", 1000, 64, 1, -1, 1.0, cview_spec(1000, 64, major=0, seed=3), cview_spec(1000, 64, major=0))
    cc("cfg2col_d", "d", "ccop", 1000, 16, 1, -1, 1.0, cview_spec(1000, 16, major=0, seed=3), cview_spec(1000, 16, major=0))
    # configuration 3 sample: 4096-point rows, forward op, inverse in place
    for p in ("f", "d"):
        cc(f"cfg3_{p}_fwd", p, "ccop", 8, 4096, 0, -1, 1.0, cview_spec(8, 4096, seed=4), cview_spec(8, 4096))
        cc(f"cfg3_{p}_inv_ip", p, "ccip", 8, 4096, 0, 1, 1.0 / 4096, cview_spec(8, 4096, seed=4))
    # radix coverage (2,3,4,5,7,8 and their mixes), both directions, both precisions
    lengths = [2, 3, 4, 5, 6, 7, 8, 9, 12, 15, 16, 20, 25, 27, 32, 45, 49, 60, 64, 96, 120, 125,
               128, 192, 210, 243, 256, 343, 384, 500, 512, 625, 640, 729, 768, 1000, 1024, 1152,
               1536, 2048, 2187, 2401, 3125, 4096, 6000, 8192, 16384]
    for i, n in enumerate(lengths):
        rows = 3 if n <= 4096 else 2
        for p in ("f", "d"):
            d = -1 if i % 2 == 0 else 1
            cc(f"len{n}_{p}", p, "ccop", rows, n, 0, d, 1.0 if d == -1 else 1.0 / n,
               cview_spec(rows, n, seed=100 + i), cview_spec(rows, n))
    # lengths with unsupported prime factors: DFT fallback and recursion
    for i, n in enumerate([11, 13, 22, 88, 136, 143, 165, 242, 1009, 2 * 3 * 5 * 7 * 11]):
        for p in ("f", "d"):
            cc(f"prime{n}_{p}", p, "ccop", 2, n, 0, -1 if i % 2 else 1, 1.0,
               cview_spec(2, n, seed=200 + i), cview_spec(2, n))
    # column major transforms of assorted lengths
    for i, n in enumerate([16, 60, 96, 1024]):
        cc(f"col{n}_f", "f", "ccop", n, 5, 1, -1, 1.0, cview_spec(n, 5, seed=300 + i), cview_spec(n, 5))
        cc(f"colcm{n}_d", "d", "ccip", n, 3, 1, 1, 0.5, cview_spec(n, 3, major=1, seed=310 + i))
    # strided / offset / negative-stride views (in and out), split blocks, in place
    for p in ("f", "d"):
        cc(f"strided_row_{p}", p, "ccop", 6, 96, 0, -1, 1.0,
           cview_spec(6, 96, off=7, cs=205, rs=2, seed=400),
           cview_spec(6, 96, off=5 * 97 + 3, cs=-97, rs=1, block=6 * 97 + 10))
        cc(f"strided_col_{p}", p, "ccop", 60, 4, 1, 1, 1.0 / 60,
           cview_spec(60, 4, off=4 + 3 * 190, cs=3, rs=-190, block=4 + 59 * 3 + 3 * 190 + 1, seed=401),
           cview_spec(60, 4, off=0, cs=1, rs=61))
        cc(f"revrow_ip_{p}", p, "ccip", 4, 128, 0, -1, 1.0,
           cview_spec(4, 128, off=127, cs=128, rs=-1, block=512, seed=410))
        cc(f"split_row_{p}", p, "ccop", 5, 240, 0, 1, 1.0,
           cview_spec(5, 240, split=True, seed=420), cview_spec(5, 240, split=True))
        cc(f"split_col_ip_{p}", p, "ccip", 48, 7, 1, -1, 2.0,
           cview_spec(48, 7, off=2, cs=9, rs=1, block=2 + 47 * 9 + 7, split=True, seed=430))
        # x and y are the same view (the reference copies x to y first, VI_ccfftmop_f_def.h:26)
        cc(f"alias_{p}", p, "ccop", 4, 1000, 0, -1, 1.0, cview_spec(4, 1000, seed=440), None, alias=True)
    # configuration 4 sample: rows scaled by 10^u, u ~ U(-3,3) (inputs stored)
    cc("cfg4_f", "f", "ccop", 4, 1024, 0, -1, 1.0,
       cview_spec(4, 1024, seed=5, dist=1) | {"rowscale": True}, cview_spec(4, 1024))
    # real <-> complex (configuration 2 sample 16 x 1536 and more)
    R_ = []

    def rc(cid, prec, M, N, major, scale, x, z):
        R_.append(dict(id=cid, prec=prec, kind="rcop", M=M, N=N, major=major, dir=-1, scale=scale, x=x, y=z))

    def cr(cid, prec, M, N, major, scale, z, x):
        R_.append(dict(id=cid, prec=prec, kind="crop", M=M, N=N, major=major, dir=1, scale=scale, x=z, y=x))

    for p in ("f", "d"):
        nr = 4 if p == "f" else 2
        rc(f"cfg2rc_{p}", p, nr, 1536, 0, 1.0, rview_spec(nr, 1536, seed=2, dist=1), cview_spec(nr, 769))
        cr(f"cfg2cr_{p}", p, nr, 1536, 0, 1.0 / 1536, cview_spec(nr, 769, seed=22, dist=1), rview_spec(nr, 1536))
        for i, n in enumerate([4, 6, 10, 16, 22, 30, 96, 250, 1000, 2048, 4096]):
            rc(f"rc{n}_{p}", p, 3, n, 0, 1.0 if i % 2 == 0 else 0.5, rview_spec(3, n, seed=500 + i), cview_spec(3, n // 2 + 1))
            cr(f"cr{n}_{p}", p, 3, n, 0, 1.0 / n, cview_spec(3, n // 2 + 1, seed=520 + i), rview_spec(3, n))
        rc(f"rccol_{p}", p, 120, 5, 1, 1.0, rview_spec(120, 5, major=0, seed=540), cview_spec(61, 5))
        cr(f"crcol_{p}", p, 120, 5, 1, 1.0 / 120, cview_spec(61, 5, seed=541), rview_spec(120, 5, major=0))
        rc(f"rcstr_{p}", p, 4, 64, 0, 1.0, rview_spec(4, 64, off=3, cs=131, rs=2, seed=550),
           cview_spec(4, 33, off=1, cs=40, rs=1))
        cr(f"crstr_{p}", p, 4, 64, 0, 1.0 / 64, cview_spec(4, 33, off=2, cs=70, rs=2, seed=551),
           rview_spec(4, 64, off=1, cs=65, rs=1))
    return C + R_


def run_case(case, impl):
    """Build the case's blocks, run it through `impl` (pyref.RefPlan or
    pyoracle.Plan) and return (input blocks, output block)."""
    dtype = np.float32 if case["prec"] == "f" else np.float64
    kind = case["kind"]
    kcode = dict(ccop=O.CCOP, ccip=O.CCIP, rcop=O.RCOP, crop=O.CROP)[kind]
    plan = impl(kcode, case["M"], case["N"], case["scale"], case["dir"], case["major"], dtype)
    if kind in ("ccop", "ccip"):
        x = make_cview(case["x"], dtype)
        if case["x"].get("rowscale"):
            u = O.fill(case["x"]["cl"], 55, 0, np.float64) * 3.0
            sc = (10.0 ** u).astype(dtype)
            z = x.get() * sc[:, None]
            x.set(z.astype(np.complex64 if dtype == np.float32 else np.complex128))
        xin = block_arrays(x)
        if kind == "ccip":
            plan.ccfftmip(x)
            return xin, block_arrays(x)
        if case["alias"]:
            plan.ccfftmop(x, x)
            return xin, block_arrays(x)
        y = make_cview(case["y"], dtype)
        plan.ccfftmop(x, y)
        return xin, block_arrays(y)
    if kind == "rcop":
        x = make_rview(case["x"], dtype)
        z = make_cview(case["y"], dtype)
        plan.rcfftmop(x, z)
        return x.buf.copy(), block_arrays(z)
    z = make_cview(case["x"], dtype)
    x = make_rview(case["y"], dtype)
    zin = block_arrays(z)
    plan.crfftmop(z, x)
    return zin, x.buf.copy()


def main():
    R.build()
    out = os.path.join(HERE)
    tcs = parse_ref_tests()
    with open(os.path.join(out, "ref_testcases.json"), "w") as f:
        json.dump(tcs, f, indent=1)
    cases = catalogue()
    arrays = {}
    for c in cases:
        xin, yout = run_case(c, R.RefPlan)
        oin, oout = run_case(c, O.Plan)
        assert np.array_equal(xin, oin)
        c["oracle_bit_exact"] = bool(np.array_equal(yout, oout))
        c["out_sha256"] = hashlib.sha256(np.ascontiguousarray(yout).tobytes()).hexdigest()
        c["out_size"] = int(yout.size)
        c["stored_output"] = bool(yout.nbytes <= FULL_OUTPUT_BYTES)
        if c["stored_output"]:
            arrays[c["id"] + "__out"] = yout
        else:
            # large outputs: a deterministic sample of the reference's values
            idx = np.unique(np.linspace(0, yout.size - 1, 1024).astype(np.int64))
            arrays[c["id"] + "__sidx"] = idx
            arrays[c["id"] + "__sval"] = yout[idx]
        if c["x"].get("dist", 0) != 0 or c["x"].get("rowscale"):
            arrays[c["id"] + "__in"] = xin
            c["stored_input"] = True
    # a checksum of the shared input stream, so drift of the generator is caught
    probe = O.fill(4096, 12345, 0, np.float64)
    meta = dict(generator_probe_sum=float(np.sum(probe * np.arange(4096))), cases=cases,
                source="jvsip reference c_VSIP_src built by oracle/Makefile.ref")
    with open(os.path.join(out, "fftm_cases.json"), "w") as f:
        json.dump(meta, f, indent=1)
    np.savez_compressed(os.path.join(out, "fftm_cases.npz"), **arrays)
    n_exact = sum(c["oracle_bit_exact"] for c in cases)
    print(f"{len(tcs)} reference tests, {len(cases)} seeded cases, oracle bit-exact on {n_exact}")


if __name__ == "__main__":
    main()
