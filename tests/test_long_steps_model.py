"""The two-step decomposition of long transforms (jv_exec.cu two_steps; the
plan's split N = N1 x N2 in jv_plan.cu build_long), restated in numpy and
checked against numpy's FFT: with n = n1 + N1*n2 and k = k2 + N2*k1, step A
transforms x down n2 (N2 points) for each n1 and multiplies output k2 by
W_N^(n1*k2); step B transforms down n1 (N1 points) and lands X in natural
order.  The inverse conjugates on each step's load and store.  R2C: the real
vector read as N/2 complex pairs, the steps on them, then the Hermitian split
by pairs (k, N/2-k) with the reference's formulas (VI_rcfftmop_f_def.h:79-118,
k_r2c_split_pairs)."""
import numpy as np
import pytest


def steps(x, N1, N2, inverse=False):
    N = N1 * N2
    src = np.conj(x) if inverse else x
    A = src.reshape(N2, N1)                       # A[n2, n1] = x[n1 + N1*n2]
    Z = np.fft.fft(A, axis=0)                     # Z[k2, n1]
    k2 = np.arange(N2)[:, None]
    n1 = np.arange(N1)[None, :]
    Z = Z * np.exp(-2j * np.pi * ((n1 * k2) % N) / N)
    # (inverse: step A stores conj Z and step B loads conj of that -- they cancel)
    Y = np.fft.fft(Z, axis=1)                     # Y[k2, k1]
    X = Y.T.reshape(-1)                           # X[k2 + N2*k1]
    return np.conj(X) if inverse else X


@pytest.mark.parametrize("N1,N2", [(64, 64), (64, 128), (128, 128), (125, 128), (96, 100), (1000, 1024)])
def test_steps_compute_the_dft(N1, N2):
    N = N1 * N2
    g = np.random.default_rng(N)
    x = g.standard_normal(N) + 1j * g.standard_normal(N)
    ref = np.fft.fft(x)
    assert np.linalg.norm(steps(x, N1, N2) - ref) / np.linalg.norm(ref) < 1e-12
    back = steps(ref, N1, N2, inverse=True) / N
    assert np.linalg.norm(back - x) / np.linalg.norm(x) < 1e-12


@pytest.mark.parametrize("N1,N2", [(64, 64), (64, 128), (96, 100)])
def test_r2c_through_the_steps(N1, N2):
    H = N1 * N2            # complex pairs; real length 2H
    g = np.random.default_rng(H + 1)
    xr = g.standard_normal(2 * H)
    Z = steps(xr[0::2] + 1j * xr[1::2], N1, N2)
    k = np.arange(H + 1)
    f = Z[np.where(k == H, 0, k)]
    b = Z[np.where(k == 0, 0, H - k)]
    w = np.exp(-1j * np.pi * k / H)                 # the R2C half-angle table
    X = 0.5 * ((b.real + f.real + w.real * (b.imag + f.imag) + w.imag * (f.real - b.real)) +
               1j * (f.imag - b.imag + w.real * (b.real - f.real) + w.imag * (b.imag + f.imag)))
    ref = np.fft.rfft(xr)
    assert np.linalg.norm(X - ref) / np.linalg.norm(ref) < 1e-12
