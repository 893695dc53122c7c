"""Every radix codelet of the general kernel (16, 15, 14, 12, 10, 9, 8, 7, 6, 5,
4, 3, 2) as the first, a middle and the last pass, and as a one-pass
schedule, through the C ABI: c2c rows and columns, forward and inverse with a
scale, R2C and C2R rows, single and double precision, on device-resident
(admitted) blocks, against numpy's FP64 FFT at the acceptance tolerance
(rel-L2 <= 1e-6 log2 N for _f, <= 1e-14 log2 N for _d).

The lengths are chosen from the schedules the plans pick (fewest passes,
largest radix first): e.g. 14 * 14 = 196 puts radix 14 first and last,
9 * 7 * 6 = 378 puts 9, 7, 6 in every position."""
import numpy as np
import pytest

import jvsip_gb300 as J

pytestmark = pytest.mark.gpu

# one-pass lengths, then multi-pass ones covering each codelet in each role
LENGTHS = [2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16,
           36, 42, 49, 63, 84, 90, 98, 126, 140, 150, 180, 196, 210, 225, 270, 294, 300, 324,
           343, 378, 392, 441, 490, 504, 588, 630, 686, 729, 750, 882, 1008, 1029, 1050, 1176,
           1400, 1470, 2058, 2100, 2744, 3087, 3375, 4116, 5040, 6174, 7203, 8232, 9604, 10290,
           12348, 14406]
ROWS = 5


def tol(N, dtype):
    return (1e-6 if dtype == np.float32 else 1e-14) * max(1.0, np.log2(N))


def rng_complex(n, seed, dtype):
    g = np.random.default_rng(seed)
    return (g.standard_normal(n) + 1j * g.standard_normal(n)).astype(np.complex128)


def interleave(z, dtype):
    a = np.empty(2 * z.size, dtype=dtype)
    a[0::2] = z.real
    a[1::2] = z.imag
    return a


def deinterleave(a):
    return a[0::2].astype(np.float64) + 1j * a[1::2].astype(np.float64)


def rel_l2(got, ref):
    return float(np.linalg.norm(got - ref) / np.linalg.norm(ref))


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("N", LENGTHS)
def test_c2c_rows_and_columns(N, dtype):
    if dtype == np.float64 and N > 8192:
        pytest.skip("double precision: the shared-memory kernel takes up to 8192 points")
    M = ROWS
    z = rng_complex(M * N, N, dtype).reshape(M, N)
    # rows, forward, scale 1
    x = interleave(z.reshape(-1), dtype)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    p = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, dtype=dtype)
    vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
    p.ccfftmop(vx, vy)
    J.check("rows")
    by.sync()
    ref = np.fft.fft(z.astype(np.complex128), axis=1)
    assert rel_l2(deinterleave(y).reshape(M, N), ref) <= tol(N, dtype)
    # columns of an N x M matrix, inverse with scale 1/N (the transposed data)
    zt = np.ascontiguousarray(z.T)  # N rows x M columns
    x2 = interleave(zt.reshape(-1), dtype)
    y2 = np.zeros_like(x2)
    cx, cy = J.CBlock(x2), J.CBlock(y2)
    cx.admit(True)
    cy.admit(False)
    q = J.FFTM(J.KIND_CCOP, N, M, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_COL, dtype=dtype)
    wx, wy = cx.view(0, M, N, 1, M), cy.view(0, M, N, 1, M)
    q.ccfftmop(wx, wy)
    J.check("columns")
    cy.sync()
    ref2 = np.fft.ifft(zt.astype(np.complex128), axis=0)
    assert rel_l2(deinterleave(y2).reshape(N, M), ref2) <= tol(N, dtype)
    for v in (vx, vy, wx, wy):
        v.destroy()
    for b in (bx, by, cx, cy):
        b.destroy()


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("H", [n for n in LENGTHS if n <= 8192])
def test_real_pairs_rows(H, dtype):
    """R2C of 2H real points per row, then C2R back with scale 1/(2H)."""
    N, M = 2 * H, ROWS
    g = np.random.default_rng(H)
    xr = g.standard_normal((M, N))
    x = xr.astype(dtype).reshape(-1).copy()
    zc = np.zeros(2 * M * (H + 1), dtype=dtype)
    bx, bz = J.RBlock(x), J.CBlock(zc)
    bx.admit(True)
    bz.admit(False)
    p = J.FFTM(J.KIND_RCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, dtype=dtype)
    vx, vz = bx.view(0, N, M, 1, N), bz.view(0, H + 1, M, 1, H + 1)
    p.rcfftmop(vx, vz)
    J.check("r2c")
    bz.sync()
    ref = np.fft.rfft(xr, axis=1)
    assert rel_l2(deinterleave(zc).reshape(M, H + 1), ref) <= tol(N, dtype)
    # back: the exact spectrum in, the rows out
    zin = interleave(ref.reshape(-1), dtype)
    xo = np.zeros(M * N, dtype=dtype)
    cz, rx = J.CBlock(zin), J.RBlock(xo)
    cz.admit(True)
    rx.admit(False)
    q = J.FFTM(J.KIND_CROP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW, dtype=dtype)
    wz, wx = cz.view(0, H + 1, M, 1, H + 1), rx.view(0, N, M, 1, N)
    q.crfftmop(wz, wx)
    J.check("c2r")
    rx.sync()
    assert rel_l2(xo.astype(np.float64).reshape(M, N), xr) <= tol(N, dtype)
    for v in (vx, vz, wz, wx):
        v.destroy()
    for b in (bx, bz, cz, rx):
        b.destroy()


@pytest.mark.parametrize("tma", ["auto", "on"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("N,M", [(1000, 4096), (1000, 130), (64, 6), (300, 10), (729, 66), (4096, 34),
                                 (6174, 18), (16, 8), (17, 12)])
def test_columns_even_pitch(N, M, dtype, tma, monkeypatch):
    """Column transforms of an N x M matrix with an even row pitch: the tiles of
    adjacent columns are staged in shared memory by TMA boxes when the layout
    allows it (automatically for transforms of 1536 points or more, at every
    length when JVSIP_GPU_TMA_COLUMNS=1), by the first pass's own loads
    otherwise; inverse with scale 1/N, and a column count that leaves a
    partial last tile."""
    if dtype == np.float64 and N > 8192:
        pytest.skip("double precision: the shared-memory kernel takes up to 8192 points")
    if tma == "on":
        monkeypatch.setenv("JVSIP_GPU_TMA_COLUMNS", "1")
    else:
        monkeypatch.delenv("JVSIP_GPU_TMA_COLUMNS", raising=False)
    z = rng_complex(M * N, N + M, dtype).reshape(N, M)
    x = interleave(z.reshape(-1), dtype)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    for d, scale in ((J.VSIP_FFT_FWD, 1.0), (J.VSIP_FFT_INV, 1.0 / N)):
        p = J.FFTM(J.KIND_CCOP, N, M, scale, d, J.VSIP_COL, dtype=dtype)
        vx, vy = bx.view(0, M, N, 1, M), by.view(0, M, N, 1, M)
        p.ccfftmop(vx, vy)
        J.check("columns")
        by.sync()
        zz = z.astype(np.complex128)
        ref = np.fft.fft(zz, axis=0) if d == J.VSIP_FFT_FWD else np.fft.ifft(zz, axis=0)
        assert rel_l2(deinterleave(y).reshape(N, M), ref) <= tol(N, dtype)
        vx.destroy()
        vy.destroy()
    bx.destroy()
    by.destroy()
