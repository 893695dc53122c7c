"""The large-radix Stockham decomposition the single-vector path runs on the
GPU (jv_exec.cu sp_passes, one register-resident launch per pass), restated
in numpy and checked against numpy's FFT: pass p of radix R (Ns = product of
the earlier radices) reads element n of transform j at j + n*N/R, multiplies
it by W_N^((n*m*N/(Ns*R)) mod N) with m = j mod Ns, transforms R points and
writes output k at (j - m)*R + m + k*Ns; the inverse conjugates on each
pass's load and store.  Also the plan's rule for the radices (jv_plan.cu:
two passes up to 2^23 points, ceil(n/9) beyond, each 2^6..2^12)."""
import numpy as np
import pytest


def radices(bits, k=None):
    if k is None:
        k = 2 if bits <= 23 else (bits + 8) // 9
    return [1 << (bits // k + (1 if i < bits % k else 0)) for i in range(k)]


def passes(x, rad, inverse=False):
    N = x.size
    Ns = 1
    for R in rad:
        src = np.conj(x) if inverse else x
        X = src.reshape(R, N // R)                 # X[n, j] = x[j + n*N/R]
        j = np.arange(N // R)
        m = j % Ns
        n = np.arange(R)[:, None]
        e = (n * m[None, :] * (N // (Ns * R))) % N
        X = X * np.exp(-2j * np.pi * e / N)
        Y = np.fft.fft(X, axis=0)                  # Y[k, j]
        out = np.empty(N, np.complex128)
        k = np.arange(R)[:, None]
        out[((j - m) * R + m)[None, :] + k * Ns] = Y
        x = np.conj(out) if inverse else out
        Ns *= R
    return x


@pytest.mark.parametrize("bits", [13, 16, 20, 23, 24, 26, 27, 31])
def test_plan_radices(bits):
    rad = radices(bits)
    assert int(np.prod(rad)) == 1 << bits
    assert all(64 <= r <= 4096 for r in rad)
    assert len(rad) == (2 if bits <= 23 else -(-bits // 9))
    assert rad == sorted(rad, reverse=True)


@pytest.mark.parametrize("bits,k", [(13, 2), (16, 2), (20, 2), (15, 3), (18, 3), (21, 3), (16, 4)])
def test_passes_compute_the_dft(bits, k):
    N = 1 << bits
    g = np.random.default_rng(bits * 10 + k)
    x = g.standard_normal(N) + 1j * g.standard_normal(N)
    rad = radices(bits, k)
    ref = np.fft.fft(x)
    assert np.linalg.norm(passes(x, rad) - ref) / np.linalg.norm(ref) < 1e-12
    back = passes(ref, rad, inverse=True) / N
    assert np.linalg.norm(back - x) / np.linalg.norm(x) < 1e-12
