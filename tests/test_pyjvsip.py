"""The pyJvsip-style interface (jvsip_gb300.pyjvsip): the FFT class with the
reference's type names, creation arguments and dft() calls, blocks and views
with the signal-processing properties; host-side checks run anywhere, the
transforms on a GPU against the FP64 oracle and numpy."""
import numpy as np
import pytest

import jvsip_gb300 as J
import pyoracle as O
from jvsip_gb300 import pyjvsip as P

# the sixteen type names of python/pyJvsip/pyJvsip.py:3703-3705, in that order
REFERENCE_TYPES = ['ccfftip_f', 'ccfftop_f', 'rcfftop_f', 'crfftop_f', 'ccfftip_d', 'ccfftop_d', 'rcfftop_d',
                   'crfftop_d', 'ccfftmip_f', 'ccfftmop_f', 'rcfftmop_f', 'crfftmop_f', 'ccfftmip_d', 'ccfftmop_d',
                   'rcfftmop_d', 'crfftmop_d']


def test_type_names_and_symbols():
    assert P.FFT.tFft == REFERENCE_TYPES
    L = J.lib()
    for t in P.FFT.tFft:
        kind, prec = t.rsplit("_", 1)
        assert hasattr(L, "vsip_%s_create_%s" % (kind, prec))
        assert hasattr(L, "vsip_%s_%s" % (kind, prec))


def test_host_side_errors_and_views():
    with pytest.raises(ValueError):
        P.FFT("ccfftmop_q", 4, 8, 1.0, -1, 0, 0, 0)
    with pytest.raises(ValueError):
        P.FFT("ccfftmop_f", 4, 8, 1.0)             # creation arguments missing
    with pytest.raises(ValueError):
        P.Block("cblock_x", 4)
    v = P.create("cmview_d", 3, 4)
    z = np.arange(12).reshape(3, 4) * (1 + 2j)
    v.set(z)
    assert v.type == "cmview_d" and v.major == "ROW" and v.COL.major == "COL"
    assert np.array_equal(v.values, z)
    w = P.Block("block_f", 10).bind(1, 2, 4)
    w.set([1, 2, 3, 4])
    assert w.type == "vview_f" and np.array_equal(w.block.array, [0, 1, 0, 2, 0, 3, 0, 4, 0, 0])
    if not J.gpu_available():
        with pytest.raises(RuntimeError, match="device"):
            P.FFT("ccfftmop_f", 4, 8, 1.0, -1, J.VSIP_ROW, 0, 0)


def oracle_rows(z, d, scale, major):
    M, N = z.shape
    buf = np.zeros(2 * M * N)
    buf[0::2], buf[1::2] = z.real.ravel(), z.imag.ravel()
    y = O.CView(np.zeros(2 * M * N), 0, N, M, 1, N)
    O.Plan(O.CCOP, M, N, scale, d, O.COL if major == J.VSIP_COL else O.ROW, np.float64).ccfftmop(
        O.CView(buf, 0, N, M, 1, N), y)
    return y.get()


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("f", 1e-6), ("d", 1e-14)])
def test_fft_class_multiple(prec, tol):
    M, N = 6, 120
    g = np.random.default_rng(3)
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    x = P.create("cmview_" + prec, M, N).set(z)
    y = P.create("cmview_" + prec, M, N)
    f = P.FFT("ccfftmop_" + prec, M, N, 1.0, -1, J.VSIP_ROW, 0, 0)
    assert f.type == "ccfftmop_" + prec and f.arg == (M, N, 1.0, -1, J.VSIP_ROW, 0, 0) and f.vsip
    assert f.dft(x, y) is y
    assert rel(y.values, oracle_rows(z, -1, 1.0, J.VSIP_ROW)) <= tol * np.log2(N)
    # in place, by columns, inverse with scale
    c = P.FFT("ccfftmip_" + prec, (M, N, 0.5, 1, J.VSIP_COL, 0, 0))
    c.dft(x)
    assert rel(x.values, oracle_rows(z, 1, 0.5, J.VSIP_COL)) <= tol * np.log2(M) * 4
    with pytest.raises(ValueError):
        f.dft(x)                                     # out-of-place type needs two views


@pytest.mark.gpu
def test_view_properties_round_trip():
    M, N = 8, 64
    g = np.random.default_rng(5)
    z = g.standard_normal((M, N)) + 1j * g.standard_normal((M, N))
    x = P.create("cmview_f", M, N).set(z)
    X = x.fftop
    assert rel(X.values, np.fft.fft(z, axis=1)) < 1e-6 * 6
    Xc = x.COL.fftop
    assert rel(Xc.values, np.fft.fft(z, axis=0)) < 1e-6 * 3
    back = X.ifftop                                   # unscaled inverse, as in pyJvsip
    assert rel(back.values / N, z) < 1e-6 * 6
    v = P.create("cvview_d", 256).set(z.ravel()[:256])
    assert rel(v.fftop.values, np.fft.fft(z.ravel()[:256])) < 1e-14 * 8
    r = P.create("mview_f", M, N).set(z.real)
    R = r.rcfft
    assert R.type == "cmview_f" and (R.collength, R.rowlength) == (M, N // 2 + 1)
    assert rel(R.values, np.fft.rfft(z.real, axis=1)) < 1e-6 * 6
    back = R.crfft
    assert (back.collength, back.rowlength) == (M, N)
    assert rel(back.values / N, z.real) < 1e-6 * 6
    rc = r.COL.rcfft
    assert (rc.collength, rc.rowlength) == (M // 2 + 1, N)
    assert rel(rc.values, np.fft.rfft(z.real, axis=0)) < 1e-6 * 3
    rv = P.create("vview_d", 128).set(z.real.ravel()[:128])
    assert rel(rv.rcfft.values, np.fft.rfft(z.real.ravel()[:128])) < 1e-14 * 7
