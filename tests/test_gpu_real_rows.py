"""R2C and C2R rows on the register-resident kernel (vsip_rcfftmop_f /
vsip_crfftmop_f with real rows of unit stride, even offset and even pitch):
every half length it holds (64 .. 8192, 768 = 8*8*12, 1000 = 10*10*10), row
counts that leave the last CTA partly empty, pitched and offset rows, a scale
on the forward transform, against numpy's FP64 rfft / irfft at the acceptance
tolerance (rel-L2 <= 1e-6 log2 N); the same calls on the shared-memory kernel
(JVSIP_GPU_NO_FAST) and on rows the fast kernel refuses (odd offset) agree
with them within the same tolerance."""
import numpy as np
import pytest

import jvsip_gb300 as J

pytestmark = pytest.mark.gpu

HALVES = [64, 128, 256, 512, 768, 1000, 1024, 2048, 4096, 8192]


def tol(N):
    return 1e-6 * np.log2(N)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cplx(a):
    return a[0::2].astype(np.float64) + 1j * a[1::2].astype(np.float64)


def r2c_c2r(H, M, pitch_r, off_r, pitch_c, off_c, scale, seed):
    """Forward R2C of M rows (scale `scale`) then C2R of the exact spectrum
    (scale 1/N); returns (rel-L2 forward, rel-L2 back, pad untouched)."""
    N = 2 * H
    g = np.random.default_rng(seed)
    xr = g.standard_normal((M, N))
    xbuf = np.full(off_r + M * pitch_r, 7.0, np.float32)
    for r in range(M):
        xbuf[off_r + r * pitch_r: off_r + r * pitch_r + N] = xr[r]
    zbuf = np.full(2 * (off_c + M * pitch_c), 5.0, np.float32)
    bx, bz = J.RBlock(xbuf), J.CBlock(zbuf)
    bx.admit(True)
    bz.admit(True)
    vx, vz = bx.view(off_r, pitch_r, M, 1, N), bz.view(off_c, pitch_c, M, 1, H + 1)
    p = J.FFTM(J.KIND_RCOP, M, N, scale, J.VSIP_FFT_FWD, J.VSIP_ROW)
    p.rcfftmop(vx, vz)
    J.check("r2c")
    bz.sync()
    Z = cplx(zbuf)
    got = np.stack([Z[off_c + r * pitch_c: off_c + r * pitch_c + H + 1] for r in range(M)])
    ref = scale * np.fft.rfft(xr, axis=1)
    e_fwd = rel(got, ref)
    pad_ok = True
    for r in range(M):  # the gaps between rows keep their values
        a = off_c + r * pitch_c + H + 1
        b = off_c + (r + 1) * pitch_c if r + 1 < M else len(Z)
        pad_ok = pad_ok and np.all(Z[a:b] == 5.0 + 5.0j)
    # back from the exact spectrum
    spec = np.fft.rfft(xr, axis=1)
    zin = np.zeros(2 * (off_c + M * pitch_c), np.float32)
    for r in range(M):
        s = slice(2 * (off_c + r * pitch_c), 2 * (off_c + r * pitch_c + H + 1))
        zin[s][0::2] = spec[r].real
        zin[s][1::2] = spec[r].imag
    xo = np.full(off_r + M * pitch_r, 3.0, np.float32)
    cz, rx = J.CBlock(zin), J.RBlock(xo)
    cz.admit(True)
    rx.admit(True)
    wz, wx = cz.view(off_c, pitch_c, M, 1, H + 1), rx.view(off_r, pitch_r, M, 1, N)
    q = J.FFTM(J.KIND_CROP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW)
    q.crfftmop(wz, wx)
    J.check("c2r")
    rx.sync()
    back = np.stack([xo[off_r + r * pitch_r: off_r + r * pitch_r + N] for r in range(M)]).astype(np.float64)
    e_back = rel(back, xr)
    for r in range(M):
        a = off_r + r * pitch_r + N
        b = off_r + (r + 1) * pitch_r if r + 1 < M else len(xo)
        pad_ok = pad_ok and np.all(xo[a:b] == 3.0)
    for v in (vx, vz, wz, wx):
        v.destroy()
    for b in (bx, bz, cz, rx):
        b.destroy()
    return e_fwd, e_back, pad_ok


@pytest.mark.parametrize("H", HALVES)
@pytest.mark.parametrize("shape", ["dense", "pitched"])
def test_real_rows_fast(H, shape):
    N = 2 * H
    if shape == "dense":
        # 8192-point halves: enough rows that the plan does not split each
        # transform over many CTAs (fewer than half the SMs' worth of rows)
        M, pr, orr, pc, oc = (80 if H == 8192 else 37), N, 0, H + 1, 0
    else:
        M, pr, orr, pc, oc = 13, N + 6, 4, H + 4, 3
    e_fwd, e_back, pad_ok = r2c_c2r(H, M, pr, orr, pc, oc, 0.5 if shape == "pitched" else 1.0, H)
    assert e_fwd <= tol(N)
    assert e_back <= tol(N)
    assert pad_ok


@pytest.mark.parametrize("H", [768, 1000, 4096])
def test_real_rows_fast_agrees_with_general_kernel(H, monkeypatch):
    N = 2 * H
    fast = r2c_c2r(H, 9, N, 0, H + 1, 0, 1.0, 3)
    monkeypatch.setenv("JVSIP_GPU_NO_FAST", "1")
    general = r2c_c2r(H, 9, N, 0, H + 1, 0, 1.0, 3)
    for e in fast[:2] + general[:2]:
        assert e <= tol(N)
    assert fast[2] and general[2]


@pytest.mark.parametrize("H", [768, 2048])
def test_real_rows_odd_offset_falls_back(H):
    # an odd real offset: x_{2n}, x_{2n+1} are not one 8-byte element, the
    # shared-memory kernel takes the call
    N = 2 * H
    e_fwd, e_back, pad_ok = r2c_c2r(H, 5, N + 2, 1, H + 1, 0, 1.0, 11)
    assert e_fwd <= tol(N) and e_back <= tol(N) and pad_ok


def test_c2c_rows_768():
    M, N = 40, 768
    g = np.random.default_rng(768)
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    x = np.empty(2 * M * N, np.float32)
    x[0::2], x[1::2] = z.real.reshape(-1), z.imag.reshape(-1)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
    J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW).ccfftmop(vx, vy)
    by.sync()
    assert rel(cplx(y).reshape(M, N), np.fft.fft(z, axis=1)) <= tol(N)
    J.FFTM(J.KIND_CCIP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW).ccfftmip(vy)
    by.release(True)
    assert rel(cplx(y).reshape(M, N), z) <= 2 * tol(N)
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


@pytest.mark.parametrize("H", [256, 768, 2048])
def test_r2c_rows_into_column_major_spectrum(H):
    # real rows in, the spectrum stored column-major (element stride M,
    # adjacent rows' bins adjacent), as kw.c lays out its frequency matrix
    N, M = 2 * H, 24
    g = np.random.default_rng(H + 5)
    xr = g.standard_normal((M, N))
    x = xr.astype(np.float32).reshape(-1).copy()
    z = np.zeros(2 * M * (H + 1), np.float32)
    bx, bz = J.RBlock(x), J.CBlock(z)
    bx.admit(True)
    bz.admit(False)
    vx, vz = bx.view(0, N, M, 1, N), bz.view(0, 1, M, M, H + 1)
    J.FFTM(J.KIND_RCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW).rcfftmop(vx, vz)
    J.check("r2c column-major")
    bz.sync()
    got = cplx(z).reshape(H + 1, M).T
    assert rel(got, np.fft.rfft(xr, axis=1)) <= tol(N)
    for v in (vx, vz):
        v.destroy()
    bx.destroy()
    bz.destroy()
