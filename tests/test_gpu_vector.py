"""GPU parity of the single-FFT calls (vsip_ccfftop / ccfftip / rcfftop /
crfftop in _f and _d) through the C ABI: every single-FFT golden case in the
host-staged and device-resident modes against the reference's outputs within
rel-L2 <= 1e-6*log2(N) (_f) / 1e-14*log2(N) (_d), with nothing outside the
output vector changed; the reference's own single-FFT known-answer tests at
their acceptance level (|y - expected| <= 0.001); the plan attributes of
c_VSIP_src/vsip_fft_getattr_f.c; plans with ntimes == 0 captured as CUDA
graphs; and full-size vectors (2^20 to 2^26 points) through round trips,
Parseval and numpy's FFT."""
import numpy as np
import pytest

import golden_cases as G
import gpu_run as R
import jvsip_gb300 as J
import pyoracle as O

pytestmark = pytest.mark.gpu

KIND = dict(ccop=J.KIND_CCOP, ccip=J.KIND_CCIP, rcop=J.KIND_RCOP, crop=J.KIND_CROP)


@pytest.mark.parametrize("admit", [False, True], ids=["staged", "resident"])
@pytest.mark.parametrize("case", G.fft_cases(), ids=lambda c: c["id"])
def test_single_fft_golden_case(case, admit):
    out, before = R.run_case_gpu(case, admit)
    idx, ref = G.reference_values(case)
    err = G.rel_l2(out[idx], ref)
    assert err <= R.tolerance(case), f"rel-L2 {err:.3e} > {R.tolerance(case):.3e}"
    mask = R.view_mask(case)
    assert np.array_equal(out[~mask], before[~mask])


class GpuFFT:
    """The library's single-FFT plan driven with one-row oracle views (the
    known-answer tests' vectors); blocks are bound to the views' storage."""

    def __init__(self, t):
        dtype = np.float32 if t["prec"] == "f" else np.float64
        self.p = J.FFT(KIND[t["kind"]], t["n"], t["scale"], t["dir"], dtype)

    def _run(self, name, *views):
        blocks, vecs = {}, []
        for v in views:
            key = id(v.buf)
            if key not in blocks:
                blocks[key] = J.CBlock(v.buf, v.im) if isinstance(v, O.CView) else J.RBlock(v.buf)
            vecs.append(blocks[key].vview(v.off, v.row_stride, v.row_length))
        try:
            getattr(self.p, name)(*vecs)
        finally:
            for w in vecs:
                w.destroy()
            for b in blocks.values():
                b.destroy()

    def ccfftop(self, x, y):
        self._run("ccfftop", x, y)

    def ccfftip(self, x):
        self._run("ccfftip", x)

    def rcfftop(self, x, z):
        self._run("rcfftop", x, z)

    def crfftop(self, z, x):
        self._run("crfftop", z, x)


@pytest.mark.parametrize("t", G.fft_kats(), ids=lambda t: f"{t['file'].split('/')[-1]}:n{t['n']}")
def test_reference_single_fft_known_answer(t):
    got = G.kat_run(t, GpuFFT(t))
    assert float(np.max(np.abs(got - G.cplx(t["expect"])))) <= 1e-3
    tol = (1e-6 if t["prec"] == "f" else 1e-14) * max(1.0, np.log2(t["n"]))
    assert G.rel_l2(np.concatenate([got.real, got.imag]),
                    np.concatenate([G.cplx(t["ref_out"]).real, G.cplx(t["ref_out"]).imag])) <= tol


def test_attributes_follow_the_reference():
    # c_VSIP_src/vsip_fft_getattr_f.c:18-57
    a = J.FFT(J.KIND_CCOP, 1000, 0.5, J.VSIP_FFT_INV).getattr()
    assert (a.input, a.output, a.place, a.dir) == (1000, 1000, 1, 1) and abs(a.scale - 0.5) < 1e-7
    a = J.FFT(J.KIND_CCIP, 64, 1.0, J.VSIP_FFT_FWD, np.float64).getattr()
    assert (a.input, a.output, a.place, a.dir, a.scale) == (64, 64, 0, -1, 1.0)
    a = J.FFT(J.KIND_RCOP, 1536, 1.0).getattr()
    assert (a.input, a.output, a.place, a.dir) == (1536, 769, 1, -1)
    a = J.FFT(J.KIND_CROP, 1536, 1.0 / 1536, dtype=np.float64).getattr()
    assert (a.input, a.output, a.place, a.dir) == (769, 1536, 1, 1)
    p = J.FFT(J.KIND_CCOP, 1 << 20)
    assert int(np.prod(p.passes())) == 1 << 20


def test_introspection_takes_both_plan_kinds():
    v = J.FFT(J.KIND_CCOP, 1000)
    m = J.FFTM(J.KIND_CCOP, 4, 1000)
    assert v.passes() == m.passes() and int(np.prod(v.passes())) == 1000
    assert int(J.lib().jvsip_fftm_graphs(v.h)) == 0


def test_length_one_and_scale():
    x = np.array([1.5, -2.0, 7.0, 8.0], np.float32)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    p = J.FFT(J.KIND_CCOP, 1, 3.0)
    vx, vy = bx.vview(1, 1, 1), by.vview(1, 1, 1)
    p.ccfftop(vx, vy)
    assert np.array_equal(y, np.array([0, 0, 21.0, 24.0], np.float32))
    for w in (vx, vy):
        w.destroy()
    bx.destroy()
    by.destroy()


@pytest.mark.parametrize("N", [4096, 1 << 18])
def test_many_times_plan_captures_graphs(N):
    g = np.random.default_rng(N)
    x = g.standard_normal(2 * N).astype(np.float32)
    y1, y2 = np.zeros_like(x), np.zeros_like(x)
    bx, b1, b2 = J.CBlock(x), J.CBlock(y1), J.CBlock(y2)
    for b in (bx, b1, b2):
        b.admit(True)
    many = J.FFT(J.KIND_CCOP, N, 1.0, J.VSIP_FFT_FWD, ntimes=0)
    once = J.FFT(J.KIND_CCOP, N, 1.0, J.VSIP_FFT_FWD, ntimes=1)
    vx, v1, v2 = bx.vview(0, 1, N), b1.vview(0, 1, N), b2.vview(0, 1, N)
    for _ in range(4):
        many.ccfftop(vx, v1)
        once.ccfftop(vx, v2)
    graphs = int(J.lib().jvsip_fftm_graphs(many.h))
    assert int(J.lib().jvsip_fftm_graphs(once.h)) == 0
    b1.sync()
    b2.sync()
    assert np.array_equal(y1, y2)
    ref = np.fft.fft(x[0::2].astype(np.float64) + 1j * x[1::2])
    got = y1[0::2] + 1j * y1[1::2].astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-6 * np.log2(N)
    # captured from the second call on (long vectors: the two steps, into the
    # plan's scratch)
    assert graphs == 1
    for w in (vx, v1, v2):
        w.destroy()
    for b in (bx, b1, b2):
        b.destroy()


def cplx(a):
    return a[0::2].astype(np.float64) + 1j * a[1::2].astype(np.float64)


@pytest.mark.parametrize("N,dtype", [(1 << 20, np.float32), (1 << 24, np.float32), (1 << 26, np.float32),
                                     (3 << 20, np.float32), (1 << 22, np.float64), (1000000, np.float64)])
def test_fullsize_vector_roundtrip_and_parseval(N, dtype):
    g = np.random.default_rng(N % 9973)
    x = g.standard_normal(2 * N).astype(dtype)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.vview(0, 1, N), by.vview(0, 1, N)
    fwd = J.FFT(J.KIND_CCOP, N, 1.0, J.VSIP_FFT_FWD, dtype)
    inv = J.FFT(J.KIND_CCIP, N, 1.0 / N, J.VSIP_FFT_INV, dtype)
    fwd.ccfftop(vx, vy)
    by.sync()
    eps = 1e-6 if dtype == np.float32 else 1e-14
    lg = np.log2(N)
    e_x, e_y = float(np.dot(x.astype(np.float64), x)), float(np.dot(y.astype(np.float64), y))
    assert abs(e_y / (N * e_x) - 1.0) <= eps * lg
    if N <= (1 << 24):
        ref = np.fft.fft(cplx(x))
        assert np.linalg.norm(cplx(y) - ref) / np.linalg.norm(ref) <= eps * lg
    inv.ccfftip(vy)
    by.release(True)
    err = np.linalg.norm(y.astype(np.float64) - x) / np.linalg.norm(x.astype(np.float64))
    assert err <= 2 * eps * lg
    for w in (vx, vy):
        w.destroy()
    for b in (bx, by):
        b.destroy()


@pytest.mark.parametrize("N", [1 << 20, 1 << 24])
def test_fullsize_real_vector_roundtrip(N):
    g = np.random.default_rng(N % 7919)
    x = g.standard_normal(N, dtype=np.float32)
    z = np.zeros(2 * (N // 2 + 1), np.float32)
    back = np.zeros_like(x)
    bx, bz, bb = J.RBlock(x), J.CBlock(z), J.RBlock(back)
    for b in (bx, bz, bb):
        b.admit(True)
    vx, vz, vb = bx.vview(0, 1, N), bz.vview(0, 1, N // 2 + 1), bb.vview(0, 1, N)
    r2c = J.FFT(J.KIND_RCOP, N, 1.0)
    c2r = J.FFT(J.KIND_CROP, N, 1.0 / N)
    r2c.rcfftop(vx, vz)
    c2r.crfftop(vz, vb)
    bz.sync()
    bb.sync()
    lg = np.log2(N)
    if N <= (1 << 20):
        ref = np.fft.rfft(x.astype(np.float64))
        assert np.linalg.norm(cplx(z) - ref) / np.linalg.norm(ref) <= 1e-6 * lg
    assert np.linalg.norm(back.astype(np.float64) - x) / np.linalg.norm(x.astype(np.float64)) <= 2e-6 * lg
    for w in (vx, vz, vb):
        w.destroy()
    for b in (bx, bz, bb):
        b.destroy()
