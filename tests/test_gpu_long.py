"""Transforms longer than one CTA takes (N above the shared-memory kernel's
limit, 2^a 3^b 5^c 7^d lengths) run as two steps of N = N1 * N2 points:
single FFTs and fftm rows and columns, unit and non-unit strides, in place,
inverse with a scale, single and double precision, against numpy's FP64 FFT
at the acceptance tolerance (rel-L2 <= 1e-6 log2 N for _f, 1e-14 log2 N for
_d); plans with ntimes == 0 capture the two steps as a CUDA graph and replay
them with identical results."""
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


def rnd(n, seed):
    g = np.random.default_rng(seed)
    return g.standard_normal(n) + 1j * g.standard_normal(n)


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("N", [16807 * 2, 32768, 40000, 65536, 3 ** 10, 2 ** 17, 5 ** 7, 7 ** 6, 1 << 20, 1 << 23])
def test_long_single_fft(N, dtype):
    z = rnd(N, N)
    x = interleave(z, dtype)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.vview(0, 1, N), by.vview(0, 1, N)
    p = J.FFT(J.KIND_CCOP, N, 1.0, J.VSIP_FFT_FWD, dtype)
    p.ccfftop(vx, vy)
    by.sync()
    assert rel(cplx(y), np.fft.fft(z)) <= tol(N, dtype)
    q = J.FFT(J.KIND_CCIP, N, 1.0 / N, J.VSIP_FFT_INV, dtype)
    q.ccfftip(vy)
    by.release(True)
    assert rel(cplx(y), z) <= 2 * tol(N, dtype)
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("M,N", [(3, 65536), (8, 40000), (2, 1 << 18)])
def test_long_fftm_rows_pitched(M, N, dtype):
    """Rows with a pitch larger than the row, forward out of place and the
    inverse with scale 1/N in place."""
    pitch = N + 24
    z = rnd(M * N, M + N).reshape(M, N)
    buf = np.zeros((M, pitch), np.complex128)
    buf[:, :N] = z
    x = interleave(buf, dtype)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(True)
    vx, vy = bx.view(0, pitch, M, 1, N), by.view(0, pitch, M, 1, N)
    J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, dtype).ccfftmop(vx, vy)
    by.sync()
    Y = cplx(y).reshape(M, pitch)
    assert rel(Y[:, :N], np.fft.fft(z, axis=1)) <= tol(N, dtype)
    assert not Y[:, N:].any()
    J.FFTM(J.KIND_CCIP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW, dtype).ccfftmip(vy)
    by.release(True)
    assert rel(cplx(y).reshape(M, pitch)[:, :N], z) <= 2 * tol(N, dtype)
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("N,M", [(65536, 16), (40000, 5), (32768, 64)])
def test_long_fftm_columns(N, M, dtype):
    """N-point transforms down the M columns of a row-major N x M matrix:
    adjacent transforms are adjacent in memory."""
    z = rnd(N * M, N * 7 + M).reshape(N, M)
    x = interleave(z, dtype)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.view(0, M, N, 1, M), by.view(0, M, N, 1, M)
    J.FFTM(J.KIND_CCOP, N, M, 1.0, J.VSIP_FFT_INV, J.VSIP_COL, dtype).ccfftmop(vx, vy)
    by.sync()
    assert rel(cplx(y).reshape(N, M), np.fft.ifft(z, axis=0) * N) <= tol(N, dtype)
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


@pytest.mark.parametrize("stride", [2, -3])
def test_long_single_fft_strided(stride):
    N = 65536
    z = rnd(N, 11)
    span = abs(stride) * (N - 1) + 1
    off = 0 if stride > 0 else span - 1
    buf = np.zeros(span + 4, np.complex128)
    buf[off + stride * np.arange(N)] = z
    x = interleave(buf, np.float32)
    y = np.zeros(2 * N, np.float32)
    bx, by = J.CBlock(x), J.CBlock(y)
    vx, vy = bx.vview(off, stride, N), by.vview(0, 1, N)
    J.FFT(J.KIND_CCOP, N, 0.5, J.VSIP_FFT_FWD).ccfftop(vx, vy)
    assert rel(cplx(y), 0.5 * np.fft.fft(z)) <= tol(N, np.float32)
    for v in (vx, vy):
        v.destroy()
    bx.destroy()
    by.destroy()


@pytest.mark.parametrize("N", [65536, 1 << 22])
def test_long_plan_graph_replay(N):
    z = rnd(N, 5)
    x = interleave(z, np.float32)
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
    assert int(J.lib().jvsip_fftm_graphs(many.h)) == 1
    assert int(J.lib().jvsip_fftm_graphs(once.h)) == 0
    b1.sync()
    b2.sync()
    assert np.array_equal(y1, y2)
    assert rel(cplx(y1), np.fft.fft(z)) <= tol(N, np.float32)
    for v in (vx, v1, v2):
        v.destroy()
    for b in (bx, b1, b2):
        b.destroy()


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f", "d"])
@pytest.mark.parametrize("M,N,pitch", [(3, 1 << 17, 1 << 17), (2, 80000, 80010), (1, 1 << 20, 1 << 20)])
def test_long_real_rows(M, N, pitch, dtype):
    """R2C rows of N real points (half length N/2 beyond one CTA) into pitched
    spectra, then C2R back with scale 1/N; the real rows have a pitch."""
    H = N // 2 + 1
    g = np.random.default_rng(N + M)
    xr = g.standard_normal((M, N))
    xb = np.zeros((M, pitch), dtype)
    xb[:, :N] = xr
    x = xb.reshape(-1).copy()
    zp = H + 6
    z = np.zeros(2 * M * zp, dtype)
    back = np.zeros(M * pitch, dtype)
    bx, bz, bb = J.RBlock(x), J.CBlock(z), J.RBlock(back)
    for b in (bx, bz, bb):
        b.admit(True)
    vx, vz, vb = bx.view(0, pitch, M, 1, N), bz.view(0, zp, M, 1, H), bb.view(0, pitch, M, 1, N)
    J.FFTM(J.KIND_RCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, dtype).rcfftmop(vx, vz)
    J.FFTM(J.KIND_CROP, M, N, 1.0 / N, J.VSIP_FFT_INV, J.VSIP_ROW, dtype).crfftmop(vz, vb)
    bz.sync()
    bb.sync()
    Z = cplx(z).reshape(M, zp)
    assert rel(Z[:, :H], np.fft.rfft(xr, axis=1)) <= tol(N // 2, dtype)
    assert not Z[:, H:].any()
    B = back.reshape(M, pitch).astype(np.float64)
    assert rel(B[:, :N], xr) <= 2 * tol(N // 2, dtype)
    assert not B[:, N:].any()
    for v in (vx, vz, vb):
        v.destroy()
    for b in (bx, bz, bb):
        b.destroy()


@pytest.mark.parametrize("stride", [2, -1])
def test_long_real_vector_strided(stride):
    """Real vectors of non-unit stride take the multi-pass path for R2C and
    the two steps plus the final store for C2R."""
    N = 1 << 16
    g = np.random.default_rng(3 + stride)
    xr = g.standard_normal(N)
    span = abs(stride) * (N - 1) + 1
    off = 0 if stride > 0 else span - 1
    x = np.zeros(span, np.float32)
    x[off + stride * np.arange(N)] = xr
    z = np.zeros(2 * (N // 2 + 1), np.float32)
    back = np.zeros(span, np.float32)
    bx, bz, bb = J.RBlock(x), J.CBlock(z), J.RBlock(back)
    vx, vz, vb = bx.vview(off, stride, N), bz.vview(0, 1, N // 2 + 1), bb.vview(off, stride, N)
    J.FFT(J.KIND_RCOP, N, 1.0).rcfftop(vx, vz)
    J.FFT(J.KIND_CROP, N, 1.0 / N).crfftop(vz, vb)
    assert rel(cplx(z), np.fft.rfft(xr)) <= tol(N // 2, np.float32)
    assert rel(back[off + stride * np.arange(N)].astype(np.float64), xr) <= 2 * tol(N // 2, np.float32)
    for v in (vx, vz, vb):
        v.destroy()
    for b in (bx, bz, bb):
        b.destroy()


@pytest.mark.parametrize("N", [1 << 25])
def test_long_real_vector_stockham_passes(N):
    """Real vectors whose half length takes three Stockham passes (2^24
    complex points): R2C through the passes and the in-place split, C2R back
    through the two steps, against numpy's rfft."""
    g = np.random.default_rng(17)
    x = g.standard_normal(N, dtype=np.float32)
    z = np.zeros(2 * (N // 2 + 1), np.float32)
    back = np.zeros_like(x)
    bx, bz, bb = J.RBlock(x), J.CBlock(z), J.RBlock(back)
    for b in (bx, bz, bb):
        b.admit(True)
    vx, vz, vb = bx.vview(0, 1, N), bz.vview(0, 1, N // 2 + 1), bb.vview(0, 1, N)
    J.FFT(J.KIND_RCOP, N, 0.5).rcfftop(vx, vz)
    J.FFT(J.KIND_CROP, N, 2.0 / N).crfftop(vz, vb)
    bz.sync()
    bb.sync()
    ref = 0.5 * np.fft.rfft(x.astype(np.float64))
    assert rel(cplx(z), ref) <= tol(N // 2, np.float32)
    assert rel(back.astype(np.float64), x.astype(np.float64)) <= 2 * tol(N // 2, np.float32)
    for v in (vx, vz, vb):
        v.destroy()
    for b in (bx, bz, bb):
        b.destroy()


def test_long_plan_scratch_stays_put_across_paths():
    """A plan created with ntimes == 0 captures its strided calls (two steps)
    and its unit-stride calls (Stockham passes) as graphs over one scratch; the
    strided call's graph replayed after the unit-stride calls is still right."""
    N = 65536
    z = rnd(N, 23)
    x2 = interleave(np.repeat(z, 2), np.float32)        # element n at 2n (stride 2)
    x1 = interleave(z, np.float32)
    y2, y1 = np.zeros(2 * N, np.float32), np.zeros(2 * N, np.float32)
    b2, b1, c2, c1 = J.CBlock(x2), J.CBlock(x1), J.CBlock(y2), J.CBlock(y1)
    for b in (b2, b1, c2, c1):
        b.admit(True)
    p = J.FFT(J.KIND_CCOP, N, 1.0, J.VSIP_FFT_FWD, ntimes=0)
    v2, v1, w2, w1 = b2.vview(0, 2, N), b1.vview(0, 1, N), c2.vview(0, 1, N), c1.vview(0, 1, N)
    ref = np.fft.fft(z)
    for _ in range(3):
        p.ccfftop(v2, w2)
    for _ in range(3):
        p.ccfftop(v1, w1)
    c2.sync()
    y2[:] = 0
    c2.release(False)
    c2.admit(True)
    p.ccfftop(v2, w2)
    c1.sync()
    c2.sync()
    assert int(J.lib().jvsip_fftm_graphs(p.h)) == 2
    assert rel(cplx(y1), ref) <= tol(N, np.float32)
    assert rel(cplx(y2), ref) <= tol(N, np.float32)
    for v in (v2, v1, w2, w1):
        v.destroy()
    for b in (b2, b1, c2, c1):
        b.destroy()


@pytest.mark.parametrize("N,M,d,inplace", [(8192, 200, J.VSIP_FFT_FWD, False), (10000, 160, J.VSIP_FFT_INV, True),
                                           (16384, 96, J.VSIP_FFT_FWD, True), (13824, 77, J.VSIP_FFT_INV, False),
                                           (3000, 200, J.VSIP_FFT_FWD, False), (6000, 90, J.VSIP_FFT_INV, True),
                                           (3125, 130, J.VSIP_FFT_INV, False)])
def test_long_columns_many(N, M, d, inplace):
    """Single-precision c2c columns from 3000 points that one CTA takes and the
    register-resident column tiles do not run as the two steps whatever their
    count (two launches, the plan's scratch): forward and inverse with scale
    1/N, in place and out of place; the same plan on a column-major matrix
    (vectors not adjacent) runs the column kernel (one launch)."""
    L = J.lib()
    z = rnd(N * M, N + M).reshape(N, M)
    scale = 1.0 if d == J.VSIP_FFT_FWD else 1.0 / N
    ref = np.fft.fft(z, axis=0) if d == J.VSIP_FFT_FWD else np.fft.ifft(z, axis=0)
    x = interleave(z, np.float32)
    y = x if inplace else np.zeros_like(x)
    bx = J.CBlock(x)
    bx.admit(True)
    by = bx if inplace else J.CBlock(y)
    if not inplace:
        by.admit(False)
    vx, vy = bx.view(0, M, N, 1, M), by.view(0, M, N, 1, M)
    p = J.FFTM(J.KIND_CCIP if inplace else J.KIND_CCOP, N, M, scale, d, J.VSIP_COL, ntimes=1)
    n0 = L.jvsip_gpu_kernel_launches()
    if inplace:
        p.ccfftmip(vx)
    else:
        p.ccfftmop(vx, vy)
    assert L.jvsip_gpu_synchronize() == 0, J.last_error()
    assert L.jvsip_gpu_kernel_launches() - n0 == 2
    by.sync()
    assert rel(cplx(y).reshape(N, M), ref) <= tol(N, np.float32)
    # column-major storage: vector v at v * N, element n at n (not adjacent)
    xc = interleave(z.T.copy(), np.float32)
    yc = np.zeros_like(xc)
    cx, cy = J.CBlock(xc), J.CBlock(yc)
    cx.admit(True)
    cy.admit(False)
    ux, uy = cx.view(0, 1, N, N, M), cy.view(0, 1, N, N, M)
    q = J.FFTM(J.KIND_CCOP, N, M, scale, d, J.VSIP_COL, ntimes=1)
    n0 = L.jvsip_gpu_kernel_launches()
    q.ccfftmop(ux, uy)
    assert L.jvsip_gpu_synchronize() == 0, J.last_error()
    assert L.jvsip_gpu_kernel_launches() - n0 == 1
    cy.sync()
    assert rel(cplx(yc).reshape(M, N).T, ref) <= tol(N, np.float32)
    for v in (vx, vy, ux, uy) if not inplace else (vx, ux, uy):
        v.destroy()
    for b in (bx, by, cx, cy) if not inplace else (bx, cx, cy):
        b.destroy()


def test_long_columns_many_graph_replay():
    """A column plan created with ntimes == 0 captures the two steps once its
    scratch exists and replays them with the direct call's results."""
    N, M = 16384, 128
    z = rnd(N * M, 29).reshape(N, M)
    x = interleave(z, np.float32)
    y1, y2 = np.zeros_like(x), np.zeros_like(x)
    bx, b1, b2 = J.CBlock(x), J.CBlock(y1), J.CBlock(y2)
    for b in (bx, b1, b2):
        b.admit(True)
    many = J.FFTM(J.KIND_CCOP, N, M, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL, ntimes=0)
    once = J.FFTM(J.KIND_CCOP, N, M, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL, ntimes=1)
    vx, v1, v2 = bx.view(0, M, N, 1, M), b1.view(0, M, N, 1, M), b2.view(0, M, N, 1, M)
    for _ in range(4):
        many.ccfftmop(vx, v1)
        once.ccfftmop(vx, v2)
    assert int(J.lib().jvsip_fftm_graphs(many.h)) == 1
    b1.sync()
    b2.sync()
    assert np.array_equal(y1, y2)
    assert rel(cplx(y1).reshape(N, M), np.fft.fft(z, axis=0)) <= tol(N, np.float32)
    for v in (vx, v1, v2):
        v.destroy()
    for b in (bx, b1, b2):
        b.destroy()


@pytest.mark.parametrize("N", [2048, 2400, 4096])
def test_columns_of_register_resident_lengths_stay_one_launch(N):
    """Column lengths the register-resident column tiles take, and lengths
    below 3000 points, keep one column-tile launch whatever the column count."""
    L = J.lib()
    M = 200
    z = rnd(N * M, N).reshape(N, M)
    x = interleave(z, np.float32)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    vx, vy = bx.view(0, M, N, 1, M), by.view(0, M, N, 1, M)
    p = J.FFTM(J.KIND_CCOP, N, M, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL, ntimes=1)
    n0 = L.jvsip_gpu_kernel_launches()
    p.ccfftmop(vx, vy)
    assert L.jvsip_gpu_synchronize() == 0, J.last_error()
    assert L.jvsip_gpu_kernel_launches() - n0 == 1
    by.sync()
    assert rel(cplx(y).reshape(N, M), np.fft.fft(z, axis=0)) <= tol(N, np.float32)
    for v in (vx, vy):
        v.destroy()
    for b in (bx, by):
        b.destroy()
