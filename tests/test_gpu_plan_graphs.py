"""Plans created with ntimes == 0 ("used many times") hold their repeated
device-resident calls as captured CUDA graphs: the first call with given views
runs directly, the second is captured, later ones replay; results are
identical to a plan that launches directly (ntimes = 1); at most 8 calls are
held per plan; staged calls and the multi-pass global path never capture."""
import numpy as np
import pytest

import jvsip_gb300 as J

pytestmark = pytest.mark.gpu


def graphs(plan):
    return int(J.lib().jvsip_fftm_graphs(plan.h))


def run(plan, bx, by, M, N, off=0):
    vx, vy = bx.view(off, N, M, 1, N), by.view(off, N, M, 1, N)
    plan.ccfftmop(vx, vy)
    J.check("call")
    vx.destroy()
    vy.destroy()


@pytest.mark.parametrize("N", [1024, 1000, 12000])
def test_capture_on_second_call_and_identical_results(N):
    M = 12
    g = np.random.default_rng(N)
    x = g.standard_normal(2 * M * N).astype(np.float32)
    y_many, y_once = np.zeros_like(x), np.zeros_like(x)
    bx, bm, bo = J.CBlock(x), J.CBlock(y_many), J.CBlock(y_once)
    for b in (bx, bm, bo):
        b.admit(True)
    many = J.FFTM(J.KIND_CCOP, M, N, 0.5, J.VSIP_FFT_INV, J.VSIP_ROW, ntimes=0)
    once = J.FFTM(J.KIND_CCOP, M, N, 0.5, J.VSIP_FFT_INV, J.VSIP_ROW, ntimes=1)
    run(many, bx, bm, M, N)
    assert graphs(many) == 0
    run(many, bx, bm, M, N)
    assert graphs(many) == 1
    for _ in range(3):
        run(many, bx, bm, M, N)
    assert graphs(many) == 1
    run(once, bx, bo, M, N)
    run(once, bx, bo, M, N)
    assert graphs(once) == 0
    bm.sync()
    bo.sync()
    assert np.array_equal(y_many, y_once)
    for b in (bx, bm, bo):
        b.destroy()


def test_at_most_eight_calls_per_plan():
    M, N = 4, 256
    x = np.random.default_rng(1).standard_normal(2 * 10 * M * N).astype(np.float32)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    p = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, ntimes=0)
    for k in range(10):   # ten different views, each called twice
        run(p, bx, by, M, N, off=k * M * N)
        run(p, bx, by, M, N, off=k * M * N)
    assert graphs(p) == 8
    by.sync()
    ref = np.fft.fft((x[0::2] + 1j * x[1::2]).astype(np.complex128).reshape(10 * M, N), axis=1)
    got = (y[0::2] + 1j * y[1::2]).reshape(10 * M, N)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-6 * 8
    bx.destroy()
    by.destroy()


def test_staged_and_global_calls_do_not_capture():
    M, N = 4, 1024
    x = np.random.default_rng(2).standard_normal(2 * M * N).astype(np.float32)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)  # not admitted: staged inside each call
    p = J.FFTM(J.KIND_CCOP, M, N, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, ntimes=0)
    for _ in range(3):
        run(p, bx, by, M, N)
    assert graphs(p) == 0
    # a prime length runs the multi-pass global path
    P = 1009
    x2 = np.random.default_rng(3).standard_normal(2 * M * P).astype(np.float32)
    y2 = np.zeros_like(x2)
    cx, cy = J.CBlock(x2), J.CBlock(y2)
    cx.admit(True)
    cy.admit(False)
    q = J.FFTM(J.KIND_CCOP, M, P, 1.0, J.VSIP_FFT_FWD, J.VSIP_ROW, ntimes=0)
    for _ in range(3):
        run(q, cx, cy, M, P)
    assert graphs(q) == 0
    for b in (bx, by, cx, cy):
        b.destroy()
