"""The CPU oracle against the reference: every golden case bit for bit (the
multiple-FFT cases, and the single-FFT cases run as one-row fftm calls), the
reference's own fftm known-answer tests (c_VSIP_testing/ccfftm{op,ip}_{f,d}.h)
at their own acceptance level (mean square error < 2e-4), and its single-FFT
known-answer tests (c_VSIP_testing/ccfftop_f.h and the rest) at theirs
(|y - expected| <= 0.001 elementwise)."""
import numpy as np
import pytest

import golden_cases as G
import pyoracle as O

KIND = dict(ccop=O.CCOP, ccip=O.CCIP, rcop=O.RCOP, crop=O.CROP)


def run_oracle(case):
    x, y = G.build_case(case)
    p = O.Plan(KIND[case["kind"]], case["M"], case["N"], case["scale"], case["dir"], case["major"],
               G.dtype_of(case))
    k = case["kind"]
    if k == "ccop":
        p.ccfftmop(x, x if case.get("alias") else y)
    elif k == "ccip":
        p.ccfftmip(x)
    elif k == "rcop":
        p.rcfftmop(x, y)
    else:
        p.crfftmop(x, y)
    return G.output_block(case, x, y)


def test_generator_is_stable():
    probe = O.fill(4096, 12345, 0, np.float64)
    assert float(np.sum(probe * np.arange(4096))) == G.meta()["generator_probe_sum"]


@pytest.mark.parametrize("case", G.cases() + G.fft_cases(), ids=lambda c: c["id"])
def test_oracle_matches_reference_bit_for_bit(case):
    out = run_oracle(case)
    assert out.size == case["out_size"]
    idx, ref = G.reference_values(case)
    assert np.array_equal(out[idx], ref)
    assert G.sha256(out) == case["out_sha256"]


@pytest.mark.parametrize("tc", G.ref_tests(), ids=lambda t: f"{t['file'].split('/')[-1]}:{t['line']}")
def test_oracle_passes_reference_known_answer_tests(tc):
    dtype = np.float32 if tc["prec"] == "f" else np.float64
    o, cs, cl, rs, rl = tc["bind"]
    x = O.CView(np.zeros(2 * tc["block"], dtype), o, cs, cl, rs, rl)
    x.set(np.array(tc["x_re"]).reshape(cl, rl) + 1j * np.array(tc["x_im"]).reshape(cl, rl))
    gold = np.array(tc["gold_re"]).reshape(cl, rl) + 1j * np.array(tc["gold_im"]).reshape(cl, rl)
    kind = O.CCOP if tc["kind"] == "ccop" else O.CCIP
    p = O.Plan(kind, tc["M"], tc["N"], tc["scale"], tc["dir"], tc["major"], dtype)
    if kind == O.CCOP:
        y = O.dense_cview(tc["M"], tc["N"], dtype)
        p.ccfftmop(x, y)
        got = y.get()
    else:
        p.ccfftmip(x)
        got = x.get()
    meansq = float(np.mean(np.abs(got - gold) ** 2))
    assert meansq < tc["tol_meansq"]


class OracleFFT:
    """The oracle as a single-FFT plan: the fftm restatement with one row."""

    def __init__(self, t):
        dtype = np.float32 if t["prec"] == "f" else np.float64
        self.p = O.Plan(KIND[t["kind"]], 1, t["n"], t["scale"], t["dir"], O.ROW, dtype)

    def ccfftop(self, x, y):
        self.p.ccfftmop(x, y)

    def ccfftip(self, x):
        self.p.ccfftmip(x)

    def rcfftop(self, x, z):
        self.p.rcfftmop(x, z)

    def crfftop(self, z, x):
        self.p.crfftmop(z, x)


@pytest.mark.parametrize("t", G.fft_kats(), ids=lambda t: f"{t['file'].split('/')[-1]}:n{t['n']}")
def test_oracle_passes_reference_single_fft_tests(t):
    got = G.kat_run(t, OracleFFT(t))
    assert float(np.max(np.abs(got - G.cplx(t["expect"])))) <= 1e-3
    assert np.array_equal(got, G.cplx(t["ref_out"])) == t["oracle_bit_exact"]


def test_factorisation_and_digit_reversal():
    # VI_nuV orders radices 3,5,7,8,4,2; the cofactor of a stage is its final radix
    assert O.factor(1024) == [(8, 4, 2), (2, 1, 2)]
    assert O.factor(1000) == [(5, 4, 8), (8, 1, 8)]
    assert O.factor(768) == [(3, 2, 256), (8, 3, 4), (4, 1, 4)]
    assert O.factor(11) == [(1, 1, 11)]
    for n in (12, 60, 1000, 1024, 88, 143):
        j = O.jofk(n)
        assert sorted(j) == list(range(n))
