"""GPU parity: every golden case through the C ABI of the GPU library, in the
host-staged mode (blocks not admitted) and the device-resident mode (blocks
admitted to device mirrors), against the reference's outputs within
rel-L2 <= 1e-6*log2(N) (_f) / 1e-14*log2(N) (_d); elements outside the output
view must be left untouched; and the reference's own known-answer tests."""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G
import gpu_run as R
import jvsip_gb300 as J
import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("admit", [False, True], ids=["staged", "resident"])
@pytest.mark.parametrize("case", G.cases(), ids=lambda c: c["id"])
def test_golden_case(case, admit):
    out, before = R.run_case_gpu(case, admit)
    idx, ref = G.reference_values(case)
    err = G.rel_l2(out[idx], ref)
    assert err <= R.tolerance(case), f"rel-L2 {err:.3e} > {R.tolerance(case):.3e}"
    mask = R.view_mask(case)
    # nothing outside the output view may change
    assert np.array_equal(out[~mask], before[~mask])


@pytest.mark.parametrize("tc", G.ref_tests(), ids=lambda t: f"{t['file'].split('/')[-1]}:{t['line']}")
def test_reference_known_answer(tc):
    dtype = np.float32 if tc["prec"] == "f" else np.float64
    o, cs, cl, rs, rl = tc["bind"]
    x = O.CView(np.zeros(2 * tc["block"], dtype), o, cs, cl, rs, rl)
    x.set(np.array(tc["x_re"]).reshape(cl, rl) + 1j * np.array(tc["x_im"]).reshape(cl, rl))
    gold = np.array(tc["gold_re"]).reshape(cl, rl) + 1j * np.array(tc["gold_im"]).reshape(cl, rl)
    kind = J.KIND_CCOP if tc["kind"] == "ccop" else J.KIND_CCIP
    p = J.FFTM(kind, tc["M"], tc["N"], tc["scale"], tc["dir"], tc["major"], dtype)
    bx = J.CBlock(x.buf)
    vx = bx.view(o, cs, cl, rs, rl)
    if kind == J.KIND_CCOP:
        y = O.dense_cview(tc["M"], tc["N"], dtype)
        by = J.CBlock(y.buf)
        vy = by.view(0, tc["N"], tc["M"], 1, tc["N"])
        p.ccfftmop(vx, vy)
        got = y.get()
    else:
        p.ccfftmip(vx)
        got = x.get()
    assert float(np.mean(np.abs(got - gold) ** 2)) < tc["tol_meansq"]


def test_plan_attributes_and_schedule():
    p = J.FFTM(J.KIND_RCOP, 4096, 1536, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW)
    a = p.getattr()
    assert (a.input.r, a.input.c, a.output.r, a.output.c) == (4096, 1536, 4096, 769)
    assert a.place == 1 and a.dir == -1 and a.major == 0
    q = J.FFTM(J.KIND_CCIP, 1000, 4096, 0.5, J.VSIP_FFT_INV, J.VSIP_COL)
    a = q.getattr()
    assert a.place == 0 and a.dir == 1 and a.major == 1 and abs(a.scale - 0.5) < 1e-7
    assert int(np.prod(q.passes())) == 1000
    assert q.jofk(1000) == O.jofk(1000)


class _ViewXX(C.Structure):
    _fields_ = [("block", C.c_void_p), ("offset", C.c_ulong), ("stride", C.c_long), ("length", C.c_ulong),
                ("markings", C.c_int)]


class PlanObjF(C.Structure):
    """The leading fields of the plan object, c_VSIP_src/vsip_fftmattributes_f.h:8-38."""
    _fields_ = [("wt", C.c_void_p), ("temp", C.c_void_p), ("index", C.c_void_p), ("pn", C.c_void_p),
                ("p0", C.c_void_p), ("pF", C.c_void_p), ("x", C.c_void_p), ("xx", _ViewXX),
                ("x_r", C.c_void_p), ("x_i", C.c_void_p), ("xp_r", C.c_void_p), ("xp_i", C.c_void_p),
                ("xst", C.c_long), ("yst", C.c_long), ("xpst", C.c_long), ("ypst", C.c_long),
                ("scale", C.c_float), ("N", C.c_ulong), ("M", C.c_ulong), ("MN", C.c_ulong), ("mN", C.c_ulong),
                ("major", C.c_int), ("length", C.c_ulong), ("d", C.c_int), ("type", C.c_int), ("dft", C.c_int),
                ("ntimes", C.c_uint), ("hint", C.c_int), ("stage", C.c_ulong), ("ext_fftm_obj", C.c_void_p)]


def _catalogue_lengths():
    lens = {11, 13, 17, 1009, 768, 1000, 1, 2, 3, 49, 343, 2401, 6000, 13824}
    for c in G.cases():
        if c["kind"] in ("rcop", "crop"):
            lens.add((c["N"] if c["major"] == 0 else c["M"]) // 2)
        else:
            lens.add(c["M"] if c["major"] == 1 else c["N"])
    for c in G.fft_cases():
        lens.add(c["N"] // 2 if c["kind"] in ("rcop", "crop") else c["N"])
    return sorted(n for n in lens if n >= 1)


@pytest.mark.parametrize("n", _catalogue_lengths())
def test_factor_and_digit_reversal_match_the_reference(n):
    # index work: bit-exact against the oracle's VI_nuV / VI_jofk restatement
    p = J.FFTM(J.KIND_CCOP, 2, n, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW)
    obj = PlanObjF.from_address(p.h)
    assert obj.MN == n and obj.mN == 2
    f = O.factor(n)
    assert obj.length == len(f)
    assert obj.dft == (1 if f and f[0][0] == 1 and f[0][2] == n else 0)
    assert p.jofk(n) == O.jofk(n)


def test_caller_quirk_scale_minus_one():
    # example21.c / kw.c pass (..., VSIP_FFT_FWD, 1, VSIP_COL, ...) to ccfftmip_create:
    # scale = -1 and dir = +1; the result must be the inverse transform times -1.
    M, N = 16, 3
    x = O.dense_cview(M, N)
    x.buf[:] = O.fill(x.buf.size, 9, 0)
    p = J.FFTM(J.KIND_CCIP, M, N, -1.0, 1, J.VSIP_COL)
    o = O.Plan(O.CCIP, M, N, -1.0, 1, O.COL)
    xo = O.CView(x.buf.copy(), 0, N, M, 1, N)
    o.ccfftmip(xo)
    b = J.CBlock(x.buf)
    p.ccfftmip(b.view(0, N, M, 1, N))
    assert G.rel_l2(x.buf, xo.buf) < 1e-6 * 4


GENERIC_IDS = {"cfg1_f_fwd", "cfg1_f_inv", "cfg3_f_fwd", "cfg3_f_inv_ip", "len64_f", "len128_f", "len256_f",
               "len512_f", "len1024_f", "len2048_f", "len4096_f", "len8192_f", "cfg4_f", "alias_f"}


@pytest.mark.parametrize("case", [c for c in G.cases() if c["id"] in GENERIC_IDS], ids=lambda c: c["id"])
def test_generic_kernel_on_fast_shapes(case, monkeypatch):
    # the specialised row kernels take these shapes by default; check the
    # general shared-memory kernel on them too
    monkeypatch.setenv("JVSIP_GPU_NO_FAST", "1")
    out, before = R.run_case_gpu(case, True)
    idx, ref = G.reference_values(case)
    assert G.rel_l2(out[idx], ref) <= R.tolerance(case)
