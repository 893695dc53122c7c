"""The FP64 form (JVSIP_FORM_DF64): complex-double rows transformed in
double-float arithmetic on the FP32 pipes.  Against numpy's FP64 FFT, row by
row, at the double-precision acceptance tolerance (rel-L2 <= 1e-14 log2 N):
every power-of-two length 64..8192, forward and inverse with a scale, rows
whose magnitudes span 10^-150..10^150 (each row shifted by its own power of
two), all-zero rows, in place and pitched; lengths and kinds without the
form keep the plain path; setform_d's error on them."""
import numpy as np
import pytest

import jvsip_gb300 as J

pytestmark = pytest.mark.gpu


def interleave(z):
    a = np.empty(2 * z.size, np.float64)
    a[0::2] = z.real.reshape(-1)
    a[1::2] = z.imag.reshape(-1)
    return a


def cplx(a):
    return a[0::2] + 1j * a[1::2]


def row_err(got, ref):
    num = np.linalg.norm(got - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    den[den == 0] = 1.0
    return num / den


@pytest.mark.parametrize("N", [64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_df64_rows_against_numpy(N):
    M = 40
    g = np.random.default_rng(N)
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    z *= (10.0 ** g.uniform(-150, 150, M))[:, None]
    z[3] = 0.0                       # an all-zero row
    z[7, 5] *= 1e12                  # one dominant element
    pitch = N + 8
    buf = np.zeros((M, pitch), np.complex128)
    buf[:, :N] = z
    x = interleave(buf)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(True)
    vx, vy = bx.view(0, pitch, M, 1, N), by.view(0, pitch, M, 1, N)
    p = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, np.float64)
    p.setform(J.JVSIP_FORM_DF64)
    assert J.lib().jvsip_fftm_getform_d(p.h) == J.JVSIP_FORM_DF64
    p.ccfftmop(vx, vy)
    by.sync()
    Y = cplx(y).reshape(M, pitch)
    tol = 1e-14 * np.log2(N)
    assert row_err(Y[:, :N], np.fft.fft(z, axis=1)).max() <= tol
    assert not Y[:, N:].any()
    assert not Y[3].any()
    # inverse in place with scale 1/N
    q = J.FFTM(J.KIND_CCIP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW, np.float64)
    q.setform(J.JVSIP_FORM_DF64)
    q.ccfftmip(vy)
    by.release(True)
    assert row_err(cplx(y).reshape(M, pitch)[:, :N], z).max() <= 2 * tol
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


def test_df64_fullsize_against_plain():
    M, N = 16384, 4096
    g = np.random.default_rng(4)
    x = g.standard_normal(2 * M * N)
    y_plain, y_df = np.zeros_like(x), np.zeros_like(x)
    bx, bp, bd = J.CBlock(x), J.CBlock(y_plain), J.CBlock(y_df)
    bx.admit(True)
    bp.admit(False)
    bd.admit(False)
    vx, vp, vd = (b.view(0, N, M, 1, N) for b in (bx, bp, bd))
    plain = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, np.float64)
    df = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, np.float64)
    df.setform(J.JVSIP_FORM_DF64)
    plain.ccfftmop(vx, vp)
    df.ccfftmop(vx, vd)
    bp.sync()
    bd.sync()
    err = np.linalg.norm(y_df - y_plain) / np.linalg.norm(y_plain)
    assert err <= 1e-14 * 12
    for r in (0, M // 2, M - 1):
        ref = np.fft.fft(cplx(x[2 * r * N:2 * (r + 1) * N]))
        got = cplx(y_df[2 * r * N:2 * (r + 1) * N])
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-14 * 12
    for v in (vx, vp, vd):
        v.destroy()
    for b in (bx, bp, bd):
        b.destroy()


def test_df64_form_errors_and_fallback():
    L = J.lib()
    p = J.FFTM(J.KIND_CCOP, 4, 1000, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, np.float64)
    L.jvsip_gpu_clear_error()
    assert L.jvsip_fftm_setform_d(p.h, J.JVSIP_FORM_DF64) == 5
    L.jvsip_gpu_clear_error()
    assert L.jvsip_fftm_getform_d(p.h) == J.JVSIP_FORM_AUTO
    r = J.FFTM(J.KIND_RCOP, 4, 1024, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, np.float64)
    assert L.jvsip_fftm_setform_d(r.h, J.JVSIP_FORM_DF64) == 5
    L.jvsip_gpu_clear_error()
    # columns (element stride != 1) keep the plain path under the form
    M, N = 1024, 6
    g = np.random.default_rng(2)
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    x = interleave(z)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    q = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL, np.float64)
    q.setform(J.JVSIP_FORM_DF64)
    vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
    q.ccfftmop(vx, vy)
    assert np.linalg.norm(cplx(y).reshape(M, N) - np.fft.fft(z, axis=0)) / np.linalg.norm(z) <= 1e-13
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()
