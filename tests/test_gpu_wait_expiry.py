"""Bounded device waits: a TMA-staged column tile whose barrier wait runs out
(the test hook makes the kernel wait, after every box has landed, on a phase
that nothing completes) records the device status word; the next
jvsip_gpu_synchronize returns E_DEVICE with a message, the context stays
usable, and after clearing the error a normal call matches the FP64 oracle."""
import numpy as np
import pytest

import jvsip_gb300 as J
import pyoracle as O

pytestmark = pytest.mark.gpu

E_DEVICE = 6


def oracle_cols(x, N, cols):
    ref = O.CView(np.zeros(2 * N * cols), 0, cols, N, 1, cols)
    O.Plan(O.CCOP, N, cols, 1.0, O.FWD, O.COL, np.float64).ccfftmop(
        O.CView(x.astype(np.float64), 0, cols, N, 1, cols), ref)
    return ref.buf


def test_tma_column_wait_expiry_reports_e_device(monkeypatch):
    monkeypatch.setenv("JVSIP_GPU_TMA_COLUMNS", "1")
    L = J.lib()
    N, cols = 1536, 64
    x = O.fill(2 * N * cols, 17, 1, np.float32)
    y = np.zeros_like(x)
    p = J.FFTM(J.KIND_CCOP, N, cols, 1.0, -1, J.VSIP_COL, ntimes=1)
    bx, by = J.CBlock(x, admit=True), J.CBlock(y, admit=True, update=False)
    vx, vy = bx.view(0, cols, N, 1, cols), by.view(0, cols, N, 1, cols)
    assert L.jvsip_gpu_synchronize() == 0
    L.jvsip_gpu_clear_error()
    L.jvsip_gpu_test_wait_expiry(1)
    try:
        L.vsip_ccfftmop_f(p.h, vx.h, vy.h)
    finally:
        L.jvsip_gpu_test_wait_expiry(0)
    assert L.jvsip_gpu_synchronize() == E_DEVICE
    code, msg = J.last_error()
    assert code == E_DEVICE and "wait" in msg
    L.jvsip_gpu_clear_error()
    # the status word was cleared by the synchronisation; the context works
    assert L.jvsip_gpu_synchronize() == 0
    p.ccfftmop(vx, vy)
    assert L.jvsip_gpu_synchronize() == 0
    by.release(True)
    ref = oracle_cols(x, N, cols)
    err = np.linalg.norm(y.astype(np.float64) - ref) / np.linalg.norm(ref)
    assert err <= 1e-6 * np.log2(N)
