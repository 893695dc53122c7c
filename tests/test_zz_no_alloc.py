"""The no-allocation transform (jvsip_ccfftm_noalloc_f) through the C ABI.

Callers that cannot allocate device memory when they transform (real-time
threads, applications whose device memory is reserved up front) use this entry
point; its intermediate buffers come from a
fixed array inside the library.  Its output must match the regular
vsip_ccfftmop_f entry point on the same plan and data, on two calls in a row,
within the parity tolerance rel-L2 <= 1e-6*log2(N).  This file is collected
last so a failure here leaves every other test already run.
"""
import numpy as np
import pytest

import jvsip_gb300 as J
import pyoracle as O

pytestmark = pytest.mark.gpu


def regular_result(plan, x, M, N):
    y = np.zeros_like(x)
    bx, by = J.CBlock(x.copy()), J.CBlock(y)
    plan.ccfftmop(bx.view(0, N, M, 1, N), by.view(0, N, M, 1, N))
    return y


@pytest.mark.parametrize("M,N,d", [(64, 1000, -1), (33, 11 * 64, 1), (16, 4096, -1)])
def test_noalloc_matches_regular_entry_point_twice(M, N, d):
    import torch
    L = J.lib()
    scale = 1.0 if d == -1 else 1.0 / N
    plan = J.FFTM(J.KIND_CCOP, M, N, scale, d, J.VSIP_ROW)
    for call, seed in enumerate((5, 6)):
        x = O.fill(2 * M * N, seed, 1, np.float32)
        want = regular_result(plan, x, M, N)
        xd = torch.from_numpy(x).cuda()
        yd = torch.full_like(xd, 3.0)
        torch.cuda.synchronize()
        rc = L.jvsip_ccfftm_noalloc_f(plan.h, xd.data_ptr(), N, yd.data_ptr(), N)
        assert rc == 0, J.last_error()
        assert L.jvsip_gpu_synchronize() == 0
        got = yd.cpu().numpy()
        err = np.linalg.norm(got.astype(np.float64) - want) / np.linalg.norm(want)
        assert err <= 1e-6 * np.log2(N), f"call {call}: rel-L2 {err:.3e}"


def test_noalloc_in_place_and_limit():
    import torch
    L = J.lib()
    M, N = 8, 1536
    plan = J.FFTM(J.KIND_CCIP, M, N, 1.0, -1, J.VSIP_ROW)
    x = O.fill(2 * M * N, 9, 1, np.float32)
    want = regular_result(J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_ROW), x, M, N)
    xd = torch.from_numpy(x).cuda()
    assert L.jvsip_ccfftm_noalloc_f(plan.h, xd.data_ptr(), N, xd.data_ptr(), N) == 0
    L.jvsip_gpu_synchronize()
    got = xd.cpu().numpy()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) <= 1e-6 * np.log2(N)
    # beyond the fixed scratch: rejected with an error, nothing launched
    big = J.FFTM(J.KIND_CCOP, 2048, 1024, 1.0, -1, J.VSIP_ROW)
    n0 = L.jvsip_gpu_kernel_launches()
    rc = L.jvsip_ccfftm_noalloc_f(big.h, xd.data_ptr(), 1024, xd.data_ptr(), 1024)
    assert rc != 0
    code, msg = J.last_error()
    assert "scratch" in msg
    L.jvsip_gpu_clear_error()
    assert L.jvsip_gpu_kernel_launches() == n0


def test_noalloc_column_plan_with_padded_rows():
    # VSIP_COL: the mN = 24 transforms of MN = 640 points run down the columns
    # of a row-major matrix whose rows are 27 complex elements apart
    import torch
    L = J.lib()
    M, N, P = 640, 24, 27
    plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_COL)
    for seed in (11, 12):
        x = O.fill(2 * M * P, seed, 1, np.float32)
        y = np.zeros_like(x)
        bx, by = J.CBlock(x.copy()), J.CBlock(y)
        plan.ccfftmop(bx.view(0, P, M, 1, N), by.view(0, P, M, 1, N))
        want = y.reshape(M, P, 2)[:, :N]
        xd = torch.from_numpy(x).cuda()
        yd = torch.full_like(xd, 3.0)
        rc = L.jvsip_ccfftm_noalloc_f(plan.h, xd.data_ptr(), P, yd.data_ptr(), P)
        assert rc == 0, J.last_error()
        assert L.jvsip_gpu_synchronize() == 0
        got = yd.cpu().numpy().reshape(M, P, 2)
        assert np.all(got[:, N:] == 3.0), "padding columns were written"
        err = np.linalg.norm(got[:, :N].astype(np.float64) - want) / np.linalg.norm(want)
        assert err <= 1e-6 * np.log2(M), f"rel-L2 {err:.3e}"


def test_noalloc_refuses_partly_overlapping_buffers():
    import torch
    L = J.lib()
    M, N = 4, 256
    plan = J.FFTM(J.KIND_CCOP, M, N, 1.0, -1, J.VSIP_ROW)
    buf = torch.zeros(2 * (M * N + 64), dtype=torch.float32, device="cuda")
    n0 = L.jvsip_gpu_kernel_launches()
    rc = L.jvsip_ccfftm_noalloc_f(plan.h, buf.data_ptr(), N, buf.data_ptr() + 8 * 16, N)
    assert rc != 0
    code, msg = J.last_error()
    assert "overlap" in msg
    L.jvsip_gpu_clear_error()
    assert L.jvsip_gpu_kernel_launches() == n0
