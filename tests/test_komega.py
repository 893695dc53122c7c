"""The k-omega pipeline (jvsip_komega_f) against the reference's kw.c
komega() sequence (examples/komegaExamples/kw_c/kw.c:8-26): the CPU oracle
bit for bit on every fixture case; on the GPU the tapered data bit for bit
(the tapers are single float32 products in the reference's order), the
spectrum's power and imaginary parts and the accumulated gram within the
fftm tolerance (power: twice the transform's), and the calls' error paths."""
import numpy as np
import pytest

import golden_cases as G
import jvsip_gb300 as J
import pyoracle as O


def sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("c", G.komega_cases(), ids=lambda c: c["id"])
def test_oracle_matches_reference_komega(c):
    assert c["oracle_bit_exact"]
    A = G.komega_arrays()
    data, freq, gram, scale = G.komega_views(c)
    O.komega_f(A[c["id"] + "__ts"], A[c["id"] + "__arr"], data, freq, gram, scale)
    for name, buf in (("data_out", data.buf), ("freq_out", freq.buf), ("gram_out", gram.buf)):
        idx, ref = G.komega_reference(c, name)
        assert np.array_equal(buf[idx], ref)
        assert sha(buf) == c[name + "_sha256"]


def tol(c):
    return 1e-6 * np.log2((c["Nts"] // 2) * c["Nsens"])


@pytest.mark.gpu
@pytest.mark.parametrize("c", G.komega_cases(), ids=lambda c: c["id"])
def test_gpu_komega_matches_reference(c):
    A = G.komega_arrays()
    data, freq, gram, scale = G.komega_views(c)
    ts, arr = A[c["id"] + "__ts"].copy(), A[c["id"] + "__arr"].copy()
    Ns, Nt = c["Nsens"], c["Nts"]
    Nf = Nt // 2 + 1
    L = J.lib()
    bx, bf, bg = J.RBlock(data.buf), J.CBlock(freq.buf), J.RBlock(gram.buf)
    bt, ba = J.RBlock(ts), J.RBlock(arr)
    for b in (bx, bf, bg, bt, ba):
        b.admit(True)
    vx = bx.view(data.off, data.col_stride, Ns, 1, Nt)
    vf = bf.view(freq.off, freq.col_stride, Ns, freq.row_stride, Nf)
    vg = bg.view(gram.off, gram.col_stride, Ns, gram.row_stride, Nf)
    vt, va = bt.vview(0, 1, Nt), ba.vview(0, 1, Ns)
    rc = J.FFTM(J.KIND_RCOP, Ns, Nt, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, ntimes=1)
    cc = J.FFTM(J.KIND_CCIP, Ns, Nf, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL, ntimes=1)
    rc_ = L.jvsip_komega_f(rc.h, cc.h, vt.h, va.h, vx.h, vf.h, float(scale), vg.h)
    assert rc_ == 0, J.last_error()
    for b in (bx, bf, bg):
        b.release(True)
    idx, ref = G.komega_reference(c, "data_out")
    assert np.array_equal(data.buf[idx], ref)
    idx, ref = G.komega_reference(c, "freq_out")
    got = freq.buf[idx]
    # power (even indices) and imaginary parts (odd indices) separately
    pe, po = idx % 2 == 0, idx % 2 == 1
    assert G.rel_l2(got[pe], ref[pe]) <= 2 * tol(c)
    assert G.rel_l2(got[po], ref[po]) <= tol(c)
    idx, ref = G.komega_reference(c, "gram_out")
    assert G.rel_l2(gram.buf[idx], ref) <= 2 * tol(c)
    for v in (vx, vf, vg, vt, va):
        v.destroy()
    for b in (bx, bf, bg, bt, ba):
        b.destroy()


@pytest.mark.gpu
def test_gpu_komega_errors():
    Ns, Nt = 8, 32
    Nf = Nt // 2 + 1
    L = J.lib()
    x = np.ones(Ns * Nt, np.float32)
    f = np.zeros(2 * Ns * Nf, np.float32)
    g = np.zeros(Ns * Nf, np.float32)
    ts, arr = np.ones(Nt, np.float32), np.ones(Ns, np.float32)
    bx, bf, bg, bt, ba = J.RBlock(x), J.CBlock(f), J.RBlock(g), J.RBlock(ts), J.RBlock(arr)
    vx, vf, vg = bx.view(0, Nt, Ns, 1, Nt), bf.view(0, 1, Ns, Ns, Nf), bg.view(0, 1, Ns, Ns, Nf)
    vt, va = bt.vview(0, 1, Nt), ba.vview(0, 1, Ns)
    rc = J.FFTM(J.KIND_RCOP, Ns, Nt, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, ntimes=1)
    cc = J.FFTM(J.KIND_CCIP, Ns, Nf, 1.0, J.VSIP_FFT_FWD, J.VSIP_COL, ntimes=1)
    bad = J.FFTM(J.KIND_CCIP, Ns, Nf, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, ntimes=1)
    L.jvsip_gpu_clear_error()
    assert L.jvsip_komega_f(rc.h, cc.h, vt.h, va.h, vx.h, vf.h, 1.0, vg.h) == 5   # blocks not admitted
    L.jvsip_gpu_clear_error()
    for b in (bx, bf, bg, bt, ba):
        b.admit(True)
    assert L.jvsip_komega_f(rc.h, bad.h, vt.h, va.h, vx.h, vf.h, 1.0, vg.h) == 3  # ccfftm not VSIP_COL
    L.jvsip_gpu_clear_error()
    assert L.jvsip_komega_f(rc.h, cc.h, vt.h, va.h, vx.h, vf.h, 1.0, vg.h) == 0
    for b in (bx, bf, bg):
        b.release(True)
    # all-ones data and tapers: only the DC bin is nonzero, |X_00|^2 = (Ns*Nt)^2
    assert abs(g[0] - (Ns * Nt) ** 2) <= 1e-3 * (Ns * Nt) ** 2
    assert np.abs(g[1:]).max() <= 1e-3 * (Ns * Nt) ** 2
    for v in (vx, vf, vg, vt, va):
        v.destroy()
    for b in (bx, bf, bg, bt, ba):
        b.destroy()
