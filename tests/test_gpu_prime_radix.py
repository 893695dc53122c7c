"""Lengths with odd prime factors 11-23 run on the global passes with the
odd-prime codelet (one thread per butterfly, the symmetric O(R^2) DFT of
VI_dftm_f), larger primes as direct sums: rows and columns, forward and
inverse with a scale, single and double precision, in place, against numpy's
FP64 FFT at the acceptance tolerance (rel-L2 <= 1e-6 log2 N for _f, 1e-14
log2 N for _d)."""
import numpy as np
import pytest

import jvsip_gb300 as J

pytestmark = pytest.mark.gpu


def tol(N, dtype):
    return (1e-6 if dtype == np.float32 else 1e-14) * np.log2(N)


def interleave(z, dtype):
    a = np.empty(2 * z.size, dtype)
    a[0::2] = z.real.reshape(-1)
    a[1::2] = z.imag.reshape(-1)
    return a


def cplx(a):
    return a[0::2].astype(np.float64) + 1j * a[1::2].astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# 11 * 64, 13 * 32, 17 * 16, 19 * 8, 23 * 4, 11 * 13, 23 * 23, 5632 = 8^3 * 11,
# 29 * 4 (a direct sum), 11 and 23 alone
LENGTHS = [704, 416, 272, 152, 92, 143, 529, 5632, 116, 11, 23]


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("N", LENGTHS)
@pytest.mark.parametrize("major", [J.VSIP_ROW, J.VSIP_COL], ids=["row", "col"])
def test_prime_radix_lengths(N, major, dtype):
    M = 37
    g = np.random.default_rng(N + 7 * major)
    for d, scale in ((J.VSIP_FFT_FWD, 1.0), (J.VSIP_FFT_INV, 1.0 / N)):
        if major == J.VSIP_ROW:
            z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
            ref = np.fft.fft(z, axis=1) if d == J.VSIP_FFT_FWD else np.fft.ifft(z, axis=1)
        else:
            z = g.standard_normal((N, M)) + 1j * g.standard_normal((N, M))
            ref = np.fft.fft(z, axis=0) if d == J.VSIP_FFT_FWD else np.fft.ifft(z, axis=0)
        x = interleave(z, dtype)
        y = np.zeros_like(x)
        bx, by = J.CBlock(x), J.CBlock(y)
        if major == J.VSIP_ROW:
            p = J.FFTM(J.KIND_CCOP, M, N, scale, d, major, dtype)
            vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
        else:
            p = J.FFTM(J.KIND_CCOP, N, M, scale, d, major, dtype)
            vx, vy = bx.view(0, M, N, 1, M), by.view(0, M, N, 1, M)
        p.ccfftmop(vx, vy)
        assert J.lib().jvsip_gpu_synchronize() == 0, J.last_error()
        assert rel(cplx(y).reshape(ref.shape), ref) <= tol(N, dtype), (N, major, d)
        for v in (vx, vy):
            v.destroy()
        bx.destroy()
        by.destroy()


@pytest.mark.parametrize("N", [143, 5632])
def test_prime_radix_in_place_with_scale(N):
    M = 9
    g = np.random.default_rng(N)
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    x = interleave(z, np.float32)
    b = J.CBlock(x)
    b.admit(True)
    p = J.FFTM(J.KIND_CCIP, M, N, 0.25, J.VSIP_FFT_FWD, J.VSIP_ROW)
    v = b.view(0, N, M, 1, N)
    p.ccfftmip(v)
    b.release(True)
    assert rel(cplx(x).reshape(M, N), 0.25 * np.fft.fft(z, axis=1)) <= tol(N, np.float32)
    v.destroy()
    b.destroy()
