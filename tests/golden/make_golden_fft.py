"""Generate the single-FFT golden fixtures under tests/golden/ from the jvsip
reference's vector FFT (vsip_ccfftop / ccfftip / rcfftop / crfftop).

Run where the reference sources are, with JVSIP_REFERENCE naming the
reference checkout (the directory holding c_VSIP_src/ and c_VSIP_testing/):

    JVSIP_REFERENCE=<checkout> python tests/golden/make_golden_fft.py

It writes
  fft_kat.json        -- the reference's own single-FFT known-answer tests
                         (c_VSIP_testing/ccfftop_f.h, ccfftip_f.h,
                         ccfftop_sc_f.h, iccfftop_f.h, iccfftip_f.h,
                         rcfftop_f.h, crfftop_f.h and their _d twins): the
                         closed-form input those tests build (the inverse DFT
                         of the ramp 0, 1, ..., n-1, restated here from the
                         test's vramp / cos / sin / div steps), the transform,
                         the expected ramp and the reference library's output;
  fft_cases.json      -- seeded single-FFT cases (lengths, directions, scales,
  fft_cases.npz          strided / negative-stride / offset / split vectors,
                         in place, x == y, x and y in one block, real <->
                         complex) with the output blocks the reference library
                         (oracle/_ref/libvsip_ref.so) produced for them.

A single-FFT case is stored in the layout of a one-row fftm case (col_length
1, the vector's stride as row_stride), so the fixtures' readers and the
oracle -- the fftm restatement run with M = 1 -- take it unchanged.  Each case
records whether the oracle reproduced the reference bit for bit.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, HERE)

import pyoracle as O  # noqa: E402
import pyref as R  # noqa: E402
from golden_cases import kat_run  # noqa: E402
from make_golden import block_arrays, cview_spec, make_cview, make_rview, rview_spec  # noqa: E402

FULL_OUTPUT_BYTES = 40 * 1024
KINDS = dict(ccop=O.CCOP, ccip=O.CCIP, rcop=O.RCOP, crop=O.CROP)


# ------------------------------------------------------------------ known-answer tests
def kat_input(n: int) -> np.ndarray:
    """The input of the reference's single-FFT tests (ccfftop_f.h:37-56): the
    inverse DFT of the ramp 0..n-1 in closed form -- x[0] = (n-1)/2,
    x[n/2] = -1/2, x[k] = -1/2 - i cot(pi k/n)/2 and x[n-k] = conj(x[k]) for
    0 < k < n/2."""
    x = np.zeros(n, np.complex128)
    x[0] = (n - 1) / 2.0
    x[n // 2] = -0.5
    k = np.arange(1, n // 2)
    x[k] = -0.5 - 0.5j / np.tan(np.pi * k / n)
    x[n - k] = np.conj(x[k])
    return x


def kat_cases():
    """One entry per (test file, precision, length).  `x` is the input vector
    (complex, or real for rcfftop), `expect` the reference test's expected
    output; the test accepts |y - expect| <= 0.001 elementwise
    (vsip_vclip_f(chk_r,.001,.001,0,1,...) then sum <= .5)."""
    out = []
    for prec in ("f", "d"):
        for n in (8, 16, 22, 24):
            x = kat_input(n)
            ramp = np.arange(n, dtype=np.float64)
            base = dict(prec=prec, n=n, block=24)
            out.append(dict(base, file=f"c_VSIP_testing/ccfftop_{prec}.h", kind="ccop", dir=-1, scale=1.0,
                            x=x, expect=ramp.astype(np.complex128)))
            out.append(dict(base, file=f"c_VSIP_testing/ccfftip_{prec}.h", kind="ccip", dir=-1, scale=1.0,
                            x=x, expect=ramp.astype(np.complex128)))
            # x and y bound on one block of 7*24: x at 72 stride -3, y at 73 stride 2
            out.append(dict(base, file=f"c_VSIP_testing/ccfftop_sc_{prec}.h", kind="ccop", dir=-1, scale=1.0,
                            x=x, expect=ramp.astype(np.complex128), block=168, shared=True,
                            xbind=[72, -3], ybind=[73, 2]))
            out.append(dict(base, file=f"c_VSIP_testing/iccfftop_{prec}.h", kind="ccop", dir=1, scale=1.0,
                            x=np.conj(x), expect=ramp.astype(np.complex128)))
            out.append(dict(base, file=f"c_VSIP_testing/iccfftip_{prec}.h", kind="ccip", dir=1, scale=1.0,
                            x=np.conj(x), expect=ramp.astype(np.complex128)))
            out.append(dict(base, file=f"c_VSIP_testing/rcfftop_{prec}.h", kind="rcop", dir=-1, scale=1.0 / n,
                            x=ramp, expect=np.conj(x)[: n // 2 + 1]))
            out.append(dict(base, file=f"c_VSIP_testing/crfftop_{prec}.h", kind="crop", dir=1, scale=1.0,
                            x=np.conj(x)[: n // 2 + 1], expect=ramp.astype(np.complex128)))
    return out


# ------------------------------------------------------------------ seeded cases
def cvec(n, off=0, stride=1, block=None, split=False, seed=None, dist=0):
    """A complex vector as a one-row view spec."""
    lo = off + min(0, (n - 1) * stride)
    assert lo >= 0
    if block is None:
        block = off + max(0, (n - 1) * stride) + 1
    return cview_spec(1, n, off=off, cs=max(1, abs(n * stride)), rs=stride, block=block, split=split, seed=seed,
                      dist=dist)


def rvec(n, off=0, stride=1, block=None, seed=None, dist=0):
    lo = off + min(0, (n - 1) * stride)
    assert lo >= 0
    if block is None:
        block = off + max(0, (n - 1) * stride) + 1
    return rview_spec(1, n, off=off, cs=max(1, abs(n * stride)), rs=stride, block=block, seed=seed, dist=dist)


def catalogue():
    C = []

    def add(cid, prec, kind, N, d, scale, x, y=None, alias=False, shared=False):
        C.append(dict(id=cid, single=True, prec=prec, kind=kind, M=1, N=N, major=0, dir=d, scale=scale, x=x, y=y,
                      alias=alias, shared=shared))

    lengths = [2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16, 27, 60, 64, 100, 125, 128, 243, 343, 1000, 1024,
               1536, 2048, 2187, 4096, 6000, 8192, 16384, 32768, 65536, 100000, 131072, 196608, 262144,
               1 << 20]
    for i, n in enumerate(lengths):
        for p in ("f", "d"):
            d = -1 if i % 2 == 0 else 1
            add(f"v{n}_{p}", p, "ccop", n, d, 1.0 if d == -1 else 1.0 / n, cvec(n, seed=700 + i), cvec(n))
    for i, n in enumerate([11, 13, 97, 1009, 2310, 4099, 11 * 4096]):
        for p in ("f", "d"):
            add(f"vprime{n}_{p}", p, "ccop", n, -1 if i % 2 else 1, 1.0, cvec(n, seed=760 + i), cvec(n))
    for p in ("f", "d"):
        add(f"vip4096_{p}", p, "ccip", 4096, 1, 1.0 / 4096, cvec(4096, seed=780))
        add(f"vip1000_{p}", p, "ccip", 1000, -1, 2.0, cvec(1000, seed=781))
        add(f"vstride_{p}", p, "ccop", 384, -1, 1.0, cvec(384, off=5, stride=3, seed=782),
            cvec(384, off=383 * 2 + 1, stride=-2, block=384 * 2 + 4))
        add(f"vneg_ip_{p}", p, "ccip", 1024, 1, 1.0, cvec(1024, off=1023, stride=-1, seed=783))
        add(f"vsplit_{p}", p, "ccop", 720, 1, 0.25, cvec(720, split=True, seed=784), cvec(720, off=3, split=True))
        add(f"vsplit_ip_{p}", p, "ccip", 2048, -1, 1.0, cvec(2048, off=1, stride=2, split=True, seed=785))
        add(f"valias_{p}", p, "ccop", 3000, -1, 1.0, cvec(3000, seed=786), None, alias=True)
        # x at even indices, y at odd indices of one block: overlapping spans, disjoint elements
        add(f"vshared_{p}", p, "ccop", 512, -1, 1.0, cvec(512, off=0, stride=2, block=1024, seed=787),
            cvec(512, off=1, stride=2, block=1024), shared=True)
        add(f"vlong_stride_{p}", p, "ccop", 65536, 1, 1.0 / 65536, cvec(65536, off=2, stride=2, seed=788),
            cvec(65536))
        # real <-> complex
        for i, n in enumerate([4, 6, 10, 16, 22, 30, 96, 250, 1000, 2048, 4096, 32768, 65536, 1 << 20]):
            # N(0,1) inputs are stored with the case: only for the short lengths
            dist = 1 if n <= 4096 else 0
            add(f"vrc{n}_{p}", p, "rcop", n, -1, 1.0 if i % 2 == 0 else 0.5, rvec(n, seed=800 + i, dist=dist),
                cvec(n // 2 + 1))
            add(f"vcr{n}_{p}", p, "crop", n, 1, 1.0 / n, cvec(n // 2 + 1, seed=830 + i, dist=dist), rvec(n))
        add(f"vrcstr_{p}", p, "rcop", 512, -1, 1.0, rvec(512, off=3, stride=2, seed=860),
            cvec(257, off=256 * 3 + 1, stride=-3, block=257 * 3 + 2))
        add(f"vcrstr_{p}", p, "crop", 512, 1, 1.0 / 512, cvec(257, off=1, stride=2, seed=861, dist=1),
            rvec(512, off=511 * 2, stride=-2))
        add(f"vrcodd_{p}", p, "rcop", 1000, -1, 1.0, rvec(1000, off=1, seed=862, dist=1),
            cvec(501, split=True))
    return C


def build_views(case):
    """(x, y-or-None) views of a seeded case with the input in place; a shared
    case binds y on x's storage."""
    dtype = np.float32 if case["prec"] == "f" else np.float64
    k = case["kind"]
    if k in ("ccop", "ccip"):
        x = make_cview(case["x"], dtype)
        if k == "ccip" or case["alias"]:
            return x, None
        if case["shared"]:
            ys = case["y"]
            return x, O.CView(x.buf, ys["off"], ys["cs"], ys["cl"], ys["rs"], ys["rl"], x.im)
        return x, make_cview(case["y"], dtype)
    if k == "rcop":
        return make_rview(case["x"], dtype), make_cview(case["y"], dtype)
    return make_cview(case["x"], dtype), make_rview(case["y"], dtype)


def run_case(case, plan):
    """Run through `plan` (single-FFT methods); returns (input block, output block)."""
    x, y = build_views(case)
    xin = block_arrays(x)
    k = case["kind"]
    if k == "ccip":
        plan.ccfftip(x)
        return xin, block_arrays(x)
    if k == "ccop":
        if case["alias"]:
            plan.ccfftop(x, x)
            return xin, block_arrays(x)
        plan.ccfftop(x, y)
        return xin, block_arrays(x if case["shared"] else y)
    if k == "rcop":
        plan.rcfftop(x, y)
        return x.buf.copy(), block_arrays(y)
    plan.crfftop(x, y)
    return xin, y.buf.copy()


class OracleFFT:
    """The oracle (the fftm restatement) as a single-FFT plan: one row, M = 1."""

    def __init__(self, kind, N, scale=1.0, dir=-1, dtype=np.float32):
        self.p = O.Plan(kind, 1, N, scale, dir, O.ROW, dtype)

    def ccfftop(self, x, y):
        self.p.ccfftmop(x, y)

    def ccfftip(self, x):
        self.p.ccfftmip(x)

    def rcfftop(self, x, z):
        self.p.rcfftmop(x, z)

    def crfftop(self, z, x):
        self.p.crfftmop(z, x)


def plan_for(impl, case_or_kat, N):
    t = case_or_kat
    dtype = np.float32 if t["prec"] == "f" else np.float64
    return impl(KINDS[t["kind"]], N, t["scale"], t["dir"], dtype)


def cplx_list(z):
    z = np.asarray(z, np.complex128)
    return [[float(a), float(b)] for a, b in zip(z.real, z.imag)]


def main():
    R.build()
    kats = []
    for t in kat_cases():
        got_ref = kat_run(t, plan_for(R.RefFFT, t, t["n"]))
        got_orc = kat_run(t, plan_for(OracleFFT, t, t["n"]))
        err = float(np.max(np.abs(got_ref - t["expect"])))
        assert err <= 1e-3, (t["file"], t["n"], err)
        e = {k: v for k, v in t.items() if k not in ("x", "expect")}
        e["x"] = cplx_list(t["x"])
        e["expect"] = cplx_list(t["expect"])
        e["ref_out"] = cplx_list(got_ref)
        e["oracle_bit_exact"] = bool(np.array_equal(got_ref, got_orc))
        kats.append(e)
    with open(os.path.join(HERE, "fft_kat.json"), "w") as f:
        json.dump(kats, f, indent=0)
    cases = catalogue()
    arrays = {}
    for c in cases:
        xin, yout = run_case(c, plan_for(R.RefFFT, c, c["N"]))
        oin, oout = run_case(c, plan_for(OracleFFT, c, c["N"]))
        assert np.array_equal(xin, oin)
        c["oracle_bit_exact"] = bool(np.array_equal(yout, oout))
        c["out_sha256"] = hashlib.sha256(np.ascontiguousarray(yout).tobytes()).hexdigest()
        c["out_size"] = int(yout.size)
        c["stored_output"] = bool(yout.nbytes <= FULL_OUTPUT_BYTES)
        if c["stored_output"]:
            arrays[c["id"] + "__out"] = yout
        else:
            idx = np.unique(np.linspace(0, yout.size - 1, 2048).astype(np.int64))
            arrays[c["id"] + "__sidx"] = idx
            arrays[c["id"] + "__sval"] = yout[idx]
        if c["x"].get("dist", 0) != 0:
            arrays[c["id"] + "__in"] = xin
            c["stored_input"] = True
    meta = dict(cases=cases, source="jvsip reference c_VSIP_src (vector FFT) built by oracle/Makefile.ref")
    with open(os.path.join(HERE, "fft_cases.json"), "w") as f:
        json.dump(meta, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "fft_cases.npz"), **arrays)
    n_exact = sum(c["oracle_bit_exact"] for c in cases)
    k_exact = sum(k["oracle_bit_exact"] for k in kats)
    print(f"{len(kats)} known-answer tests (oracle bit-exact on {k_exact}), {len(cases)} seeded cases "
          f"(oracle bit-exact on {n_exact})")


if __name__ == "__main__":
    main()
