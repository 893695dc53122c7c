"""Full-size configurations, checked through properties that hold at any size:
forward -> inverse (scale 1/N) round trips, Parseval's identity
sum |X|^2 = N sum |x|^2, linearity F(a x + b y) = a F(x) + b F(y), and
sampled rows against numpy's FP64 FFT.  Blocks are admitted (device
resident); the calls go through the C ABI.

Sizes: 65536 x 4096 c64 rows (2 GiB per buffer), 16384 x 4096 c128 rows,
1000-point columns x 4096, R2C/C2R 4096 x 1536, 32768 x 1024 rows scaled by
10^U(-3,3) in the plain and both split-precision forms."""
import numpy as np
import pytest

import jvsip_gb300 as J

pytestmark = pytest.mark.gpu


def normal_interleaved(n_complex, seed, dtype):
    g = np.random.default_rng(seed)
    return g.standard_normal(2 * n_complex, dtype=np.float64 if dtype == np.float64 else np.float32).astype(dtype)


def cplx(a):
    return a[0::2].astype(np.float64) + 1j * a[1::2].astype(np.float64)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def energy(a):
    a64 = a.astype(np.float64)
    return float(np.dot(a64, a64))


def roundtrip_rows(M, N, dtype, tol_scale, seed):
    x = normal_interleaved(M * N, seed, dtype)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
    fwd = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, dtype=dtype)
    inv = J.FFTM(J.KIND_CCIP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW, dtype=dtype)
    fwd.ccfftmop(vx, vy)
    J.check("forward")
    by.sync()
    # Parseval on the whole matrix, sampled rows against numpy
    assert abs(energy(y) / (N * energy(x)) - 1.0) <= tol_scale
    for r in (0, 1, M // 2, M - 1):
        got = cplx(y[2 * r * N:2 * (r + 1) * N])
        ref = np.fft.fft(cplx(x[2 * r * N:2 * (r + 1) * N]))
        assert rel(got, ref) <= tol_scale
    inv.ccfftmip(vy)
    J.check("inverse")
    by.release(True)
    bx.release(False)
    err = rel(y.astype(np.float64), x.astype(np.float64))
    for v in (vx, vy):
        v.destroy()
    for b in (bx, by):
        b.destroy()
    return err


def test_rows_65536x4096_f32():
    err = roundtrip_rows(65536, 4096, np.float32, 1e-6 * 12, 41)
    assert err <= 2e-6 * 12


def test_rows_16384x4096_f64():
    err = roundtrip_rows(16384, 4096, np.float64, 1e-14 * 12, 43)
    assert err <= 2e-14 * 12


def test_columns_1000x4096_roundtrip():
    M, N = 1000, 4096  # 4096 transforms of 1000 points down the columns
    x = normal_interleaved(M * N, 47, np.float32)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
    fwd = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL)
    inv = J.FFTM(J.KIND_CCIP, M, N, 1.0 / M, J.VSIP_FFT_INV, J.VSIP_COL)
    fwd.ccfftmop(vx, vy)
    J.check("forward")
    by.sync()
    assert abs(energy(y) / (M * energy(x)) - 1.0) <= 1e-6 * 10
    X = cplx(x).reshape(M, N)
    Y = cplx(y).reshape(M, N)
    for c in (0, 1, N // 2, N - 1):
        assert rel(Y[:, c], np.fft.fft(X[:, c])) <= 1e-6 * 10
    inv.ccfftmip(vy)
    J.check("inverse")
    by.release(True)
    assert rel(y.astype(np.float64), x.astype(np.float64)) <= 2e-6 * 10
    for v in (vx, vy):
        v.destroy()
    for b in (bx, by):
        b.destroy()


def test_real_pairs_4096x1536_roundtrip():
    M, N, H = 4096, 1536, 769
    g = np.random.default_rng(53)
    x = g.standard_normal(M * N, dtype=np.float32)
    z = np.zeros(2 * M * H, np.float32)
    back = np.zeros_like(x)
    bx, bz, bb = J.RBlock(x), J.CBlock(z), J.RBlock(back)
    for b in (bx, bz, bb):
        b.admit(True)
    vx, vz, vb = bx.view(0, N, M, 1, N), bz.view(0, H, M, 1, H), bb.view(0, N, M, 1, N)
    r2c = J.FFTM(J.KIND_RCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW)
    c2r = J.FFTM(J.KIND_CROP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW)
    r2c.rcfftmop(vx, vz)
    c2r.crfftmop(vz, vb)
    J.check("r2c -> c2r")
    bz.sync()
    bb.sync()
    Z = cplx(z).reshape(M, H)
    X = x.reshape(M, N).astype(np.float64)
    for r in (0, M // 3, M - 1):
        assert rel(Z[r], np.fft.rfft(X[r])) <= 1e-6 * 11
    assert rel(back.astype(np.float64), x.astype(np.float64)) <= 2e-6 * 11
    for v in (vx, vz, vb):
        v.destroy()
    for b in (bx, bz, bb):
        b.destroy()


@pytest.mark.parametrize("form", ["plain", "fp16", "bf16"])
def test_precision_config_linearity_and_roundtrip(form):
    M, N = 32768, 1024
    g = np.random.default_rng(59)
    scale_rows = (10.0 ** g.uniform(-3, 3, M)).astype(np.float32)
    x = (normal_interleaved(M * N, 61, np.float32).reshape(M, 2 * N) * scale_rows[:, None]).reshape(-1)
    u = (normal_interleaved(M * N, 67, np.float32).reshape(M, 2 * N) * scale_rows[:, None]).reshape(-1)
    a, b = np.float32(0.75), np.float32(-1.5)
    w = (a * x + b * u).astype(np.float32)
    tol = {"plain": 1e-6, "fp16": 1e-6, "bf16": 1e-5}[form] * 10
    f = {"plain": J.JVSIP_FORM_PLAIN, "fp16": J.JVSIP_FORM_SPLIT_FP16, "bf16": J.JVSIP_FORM_SPLIT_BF16}[form]
    outs = []
    for src in (x, u, w):
        y = np.zeros_like(src)
        bs, by = J.CBlock(src), J.CBlock(y)
        bs.admit(True)
        by.admit(False)
        vs, vy = bs.view(0, N, M, 1, N), by.view(0, N, M, 1, N)
        p = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW)
        p.setform(f)
        p.ccfftmop(vs, vy)
        assert J.lib().jvsip_gpu_synchronize() == 0, J.last_error()
        by.sync()
        outs.append(cplx(y).reshape(M, N))
        for v in (vs, vy):
            v.destroy()
        for blk in (bs, by):
            blk.destroy()
    Fx, Fu, Fw = outs
    # linearity, row by row (rows span six decades)
    lin = a * Fx.astype(np.complex128) + b * Fu.astype(np.complex128)
    row_err = np.linalg.norm(Fw - lin, axis=1) / np.linalg.norm(lin, axis=1)
    assert float(row_err.max()) <= 2 * tol
    # the round trip of x through the same form
    X = Fx
    xi = np.zeros(2 * M * N, np.float32)
    xi[0::2] = X.real.reshape(-1)
    xi[1::2] = X.imag.reshape(-1)
    bi = J.CBlock(xi)
    bi.admit(True)
    vi = bi.view(0, N, M, 1, N)
    q = J.FFTM(J.KIND_CCIP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW)
    q.setform(f)
    q.ccfftmip(vi)
    assert J.lib().jvsip_gpu_synchronize() == 0, J.last_error()
    bi.release(True)
    back = cplx(xi).reshape(M, N)
    ref = cplx(x).reshape(M, N)
    rt = np.linalg.norm(back - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert float(rt.max()) <= 2 * tol
    vi.destroy()
    bi.destroy()
