"""Split complex blocks (real and imaginary parts in separate arrays, cstride
1) as a first-class path: power-of-two rows through the register-resident
kernel's split instance, every other length and double precision through the
shared-memory kernel's split instance, columns, in place, forward and inverse
with a scale, against numpy's FP64 FFT at the acceptance tolerance; mixed
split / interleaved calls still run (through the view walkers)."""
import numpy as np
import pytest

import jvsip_gb300 as J

pytestmark = pytest.mark.gpu


def tol(N, dtype):
    return (1e-6 if dtype == np.float32 else 1e-14) * max(1.0, np.log2(N))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("N", [64, 256, 1024, 4096, 8192, 1000, 1536, 6000, 12, 7])
@pytest.mark.parametrize("major", ["row", "col"])
def test_split_rows_and_columns(N, major, dtype):
    if dtype == np.float64 and N > 8192:
        pytest.skip("double precision: the shared-memory kernel takes up to 8192 points")
    M = 24
    g = np.random.default_rng(N + (major == "col"))
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    if major == "row":
        zz = z
        mj = J.VSIP_ROW
        PM, PN = M, N
    else:
        zz = np.ascontiguousarray(z.T)  # N x M matrix, transforms down the columns
        mj = J.VSIP_COL
        PM, PN = N, M
    xr, xi = zz.real.astype(dtype).reshape(-1).copy(), zz.imag.astype(dtype).reshape(-1).copy()
    yr, yi = np.zeros_like(xr), np.zeros_like(xi)
    bx, by = J.CBlock(xr, xi), J.CBlock(yr, yi)
    bx.admit(True)
    by.admit(False)
    cols = zz.shape[1]
    vx, vy = bx.view(0, cols, zz.shape[0], 1, cols), by.view(0, cols, zz.shape[0], 1, cols)
    J.FFTM(J.KIND_CCOP, PM, PN, 1.0, J.VSIP_FFT_FWD, mj, dtype).ccfftmop(vx, vy)
    by.sync()
    axis = 1 if major == "row" else 0
    ref = np.fft.fft(zz, axis=axis)
    assert rel((yr + 1j * yi).reshape(zz.shape), ref) <= tol(N, dtype)
    # inverse in place with scale 1/N
    J.FFTM(J.KIND_CCIP, PM, PN, 1.0 / N, J.VSIP_FFT_INV, mj, dtype).ccfftmip(vy)
    by.release(True)
    assert rel((yr + 1j * yi).reshape(zz.shape), zz) <= 2 * tol(N, dtype)
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


def test_split_input_interleaved_output():
    M, N = 8, 1024
    g = np.random.default_rng(5)
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    xr, xi = z.real.astype(np.float32).reshape(-1).copy(), z.imag.astype(np.float32).reshape(-1).copy()
    y = np.zeros(2 * M * N, np.float32)
    bx, by = J.CBlock(xr, xi), J.CBlock(y)
    vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
    J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW).ccfftmop(vx, vy)
    got = (y[0::2] + 1j * y[1::2].astype(np.float64)).reshape(M, N)
    assert rel(got, np.fft.fft(z, axis=1)) <= tol(N, np.float32)
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


def test_split_fullsize_rows_roundtrip():
    M, N = 16384, 4096
    g = np.random.default_rng(9)
    xr = g.standard_normal(M * N, dtype=np.float32)
    xi = g.standard_normal(M * N, dtype=np.float32)
    x0r, x0i = xr.copy(), xi.copy()
    bx = J.CBlock(xr, xi)
    bx.admit(True)
    vx = bx.view(0, N, M, 1, N)
    J.FFTM(J.KIND_CCIP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW).ccfftmip(vx)
    bx.sync()
    for r in (0, M // 2, M - 1):
        ref = np.fft.fft(x0r[r * N:(r + 1) * N].astype(np.float64) + 1j * x0i[r * N:(r + 1) * N])
        assert rel(xr[r * N:(r + 1) * N] + 1j * xi[r * N:(r + 1) * N].astype(np.float64), ref) <= tol(N, np.float32)
    J.FFTM(J.KIND_CCIP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW).ccfftmip(vx)
    bx.release(True)
    err = np.sqrt(np.sum((xr - x0r).astype(np.float64) ** 2 + (xi - x0i).astype(np.float64) ** 2) /
                  np.sum(x0r.astype(np.float64) ** 2 + x0i.astype(np.float64) ** 2))
    assert err <= 2 * tol(N, np.float32)
    vx.destroy()
    bx.destroy()
