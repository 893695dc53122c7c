"""The no-allocation transform (jvsip_ccfftm_noalloc_f) through the C ABI.

Callers that cannot allocate device memory when they transform (code running
during stream capture, real-time threads, applications whose device memory is
reserved up front) use this entry point; its intermediate buffers come from a
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
