"""Precision form: 1024-point rows through the tensor-core DFT products with
hi/lo-split FP16 (per-row scaled) or BF16 operands and FP32 accumulation,
against the FP64 oracle on rows whose magnitudes span 10^-3..10^3, forward and
inverse, in place and out of place; the device status stays clean."""
import numpy as np
import pytest

import jvsip_gb300 as J
import pyoracle as O

pytestmark = pytest.mark.gpu

M, N = 64, 1024


def data(seed):
    x = O.fill(2 * M * N, seed, 1, np.float32).reshape(M, 2 * N)
    u = O.fill(M, seed + 1, 0, np.float64) * 3.0
    return (x * (10.0 ** u).astype(np.float32)[:, None]).reshape(-1)


def oracle(x, d, scale):
    y = O.CView(np.zeros(2 * M * N), 0, N, M, 1, N)
    O.Plan(O.CCOP, M, N, scale, d, O.ROW, np.float64).ccfftmop(O.CView(x.astype(np.float64), 0, N, M, 1, N), y)
    return y.buf.reshape(M, 2 * N)


def worst_row_err(got, ref):
    g = got.reshape(M, 2 * N).astype(np.float64)
    return max(np.linalg.norm(g[r] - ref[r]) / np.linalg.norm(ref[r]) for r in range(M))


@pytest.mark.parametrize("form,bound", [(J.JVSIP_FORM_SPLIT_FP16, 1e-6), (J.JVSIP_FORM_SPLIT_BF16, 1e-5)],
                         ids=["fp16", "bf16"])
@pytest.mark.parametrize("d", [-1, 1], ids=["fwd", "inv"])
def test_split_form_accuracy(form, bound, d):
    L = J.lib()
    scale = 1.0 if d == -1 else 1.0 / N
    x = data(21)
    ref = oracle(x, d, scale)
    y = np.zeros_like(x)
    p = J.FFTM(J.KIND_CCOP, M, N, scale, d, J.VSIP_ROW)
    p.setform(form)
    assert L.jvsip_fftm_getform_f(p.h) == form
    bx, by = J.CBlock(x.copy(), admit=True), J.CBlock(y, admit=True, update=False)
    n0 = L.jvsip_gpu_kernel_launches()
    p.ccfftmop(bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N))
    assert L.jvsip_gpu_synchronize() == 0, J.last_error()
    assert L.jvsip_gpu_kernel_launches() - n0 == 1
    by.release(True)
    err = worst_row_err(y, ref)
    assert err <= bound, f"worst row rel-L2 {err:.3e}"


def test_split_form_in_place_and_fallback():
    L = J.lib()
    x = data(31)
    ref = oracle(x, -1, 1.0)
    p = J.FFTM(J.KIND_CCIP, M, N, 1.0, -1, J.VSIP_ROW)
    p.setform(J.JVSIP_FORM_SPLIT_FP16)
    b = J.CBlock(x, admit=True)
    p.ccfftmip(b.view(0, N, M, 1, N))
    assert L.jvsip_gpu_synchronize() == 0
    b.release(True)
    assert worst_row_err(x, ref) <= 1e-6
    # shapes the form does not take run on the plain kernels
    q = J.FFTM(J.KIND_CCOP, 8, 512, 1.0, -1, J.VSIP_ROW)
    q.setform(J.JVSIP_FORM_SPLIT_BF16)
    xs = O.fill(2 * 8 * 512, 5, 1, np.float32)
    ys = np.zeros_like(xs)
    q.ccfftmop(J.CBlock(xs).view(0, 512, 8, 1, 512), J.CBlock(ys).view(0, 512, 8, 1, 512))
    assert np.isfinite(ys).all() and np.abs(ys).max() > 0


def scaled_rows(Mr, seed):
    g = np.random.default_rng(seed)
    z = g.standard_normal((Mr, N)) + 1j * g.standard_normal((Mr, N))
    return z * (10.0 ** g.uniform(-3, 3, Mr))[:, None]


def rows_worst(got, ref):
    return float(np.max(np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)))


@pytest.mark.parametrize("form,bound", [(J.JVSIP_FORM_SPLIT_FP16, 1e-6), (J.JVSIP_FORM_SPLIT_BF16, 1e-5)],
                         ids=["fp16", "bf16"])
def test_split_form_many_groups(form, bound):
    # several waves of 4-row groups (2434 CTAs) and a last group of 2 rows,
    # forward and inverse
    Mr = 2 * 152 * 4 * 3 + 2
    z = scaled_rows(Mr, 41)
    x = np.empty(2 * Mr * N, np.float32)
    x[0::2], x[1::2] = z.real.reshape(-1), z.imag.reshape(-1)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x, admit=True), J.CBlock(y, admit=True, update=False)
    for d in (-1, 1):
        p = J.FFTM(J.KIND_CCOP, Mr, N, 1.0, d, J.VSIP_ROW)
        p.setform(form)
        p.ccfftmop(bx.view(0, N, Mr, 1, N), by.view(0, N, Mr, 1, N))
        assert J.lib().jvsip_gpu_synchronize() == 0, J.last_error()
        by.sync()
        got = (y[0::2] + 1j * y[1::2].astype(np.float64)).reshape(Mr, N)
        ref = np.fft.fft(z, axis=1) if d == -1 else np.fft.ifft(z, axis=1) * N
        assert rows_worst(got, ref) <= bound


def test_split_form_unaligned_rows():
    # rows starting 8 bytes off a 16-byte boundary (odd offset and pitch), in
    # place, with a scale
    Mr, pitch, off = 37, N + 1, 1
    z = scaled_rows(Mr, 43)
    buf = np.zeros((off + Mr * pitch), np.complex128)
    for r in range(Mr):
        buf[off + r * pitch: off + r * pitch + N] = z[r]
    x = np.empty(2 * buf.size, np.float32)
    x[0::2], x[1::2] = buf.real, buf.imag
    bx = J.CBlock(x, admit=True)
    p = J.FFTM(J.KIND_CCIP, Mr, N, 0.5, -1, J.VSIP_ROW)
    p.setform(J.JVSIP_FORM_SPLIT_FP16)
    p.ccfftmip(bx.view(off, pitch, Mr, 1, N))
    assert J.lib().jvsip_gpu_synchronize() == 0, J.last_error()
    bx.release(True)
    c = x[0::2] + 1j * x[1::2].astype(np.float64)
    got = np.stack([c[off + r * pitch: off + r * pitch + N] for r in range(Mr)])
    assert rows_worst(got, 0.5 * np.fft.fft(z, axis=1)) <= 1e-6
    # the gaps between rows keep their (zero) values
    for r in range(Mr - 1):
        assert c[off + r * pitch + N] == 0


@pytest.mark.parametrize("in_off,out_off", [(0, 1), (1, 0)], ids=["out-odd", "in-odd"])
def test_split_form_mixed_alignment(in_off, out_off):
    # one side on 16-byte row boundaries, the other 8 bytes off
    Mr = 21
    z = scaled_rows(Mr, 47)
    x = np.zeros(2 * (in_off + Mr * N), np.float32)
    c = z.reshape(-1)
    x[2 * in_off::2], x[2 * in_off + 1::2] = c.real, c.imag
    y = np.full(2 * (out_off + Mr * N), 9.0, np.float32)
    bx, by = J.CBlock(x, admit=True), J.CBlock(y, admit=True)
    p = J.FFTM(J.KIND_CCOP, Mr, N, 1.0, -1, J.VSIP_ROW)
    p.setform(J.JVSIP_FORM_SPLIT_BF16)
    p.ccfftmop(bx.view(in_off, N, Mr, 1, N), by.view(out_off, N, Mr, 1, N))
    assert J.lib().jvsip_gpu_synchronize() == 0, J.last_error()
    by.release(True)
    got = (y[2 * out_off::2] + 1j * y[2 * out_off + 1::2].astype(np.float64)).reshape(Mr, N)
    assert rows_worst(got, np.fft.fft(z, axis=1)) <= 1e-5
    assert np.all(y[:2 * out_off] == 9.0)
