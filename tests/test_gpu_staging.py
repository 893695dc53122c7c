"""Host-resident (staged) calls large enough for the pipelined copy path:
dense and pitched rows, out of place and in place, forward and inverse,
checked against the device-resident result and the FP64 oracle on sampled rows."""
import numpy as np
import pytest

import golden_cases as G
import jvsip_gb300 as J
import pyoracle as O

pytestmark = pytest.mark.gpu


def oracle_rows(x, rows, N, pitch, d, scale):
    out = []
    for r in rows:
        xr = x[2 * r * pitch: 2 * (r * pitch + N)].astype(np.float64)
        yo = O.CView(np.zeros(2 * N), 0, N, 1, 1, N)
        O.Plan(O.CCOP, 1, N, scale, d, O.ROW, np.float64).ccfftmop(O.CView(xr, 0, N, 1, 1, N), yo)
        out.append(yo.buf)
    return out


@pytest.mark.parametrize("N,rows,pitch,d,inplace", [
    (4096, 2048, 4096, -1, False),
    (4096, 3000, 4100, 1, False),
    (1024, 9000, 1024, -1, True),
    (1000, 9000, 1000, -1, False),
])
def test_pipelined_staging(N, rows, pitch, d, inplace):
    x = O.fill(2 * rows * pitch, 77, 1, np.float32)
    x0 = x.copy()
    scale = 1.0 if d == -1 else 1.0 / N
    kind = J.KIND_CCIP if inplace else J.KIND_CCOP
    p = J.FFTM(kind, rows, N, scale, d, J.VSIP_ROW)
    bx = J.CBlock(x)
    vx = bx.view(0, pitch, rows, 1, N)
    if inplace:
        p.ccfftmip(vx)
        y = x
    else:
        y = np.full(2 * rows * pitch, 7.0, np.float32)
        by = J.CBlock(y)
        p.ccfftmop(vx, by.view(0, pitch, rows, 1, N))
    sample = [0, 1, rows // 3, rows - 1]
    ref = oracle_rows(x0, sample, N, pitch, d, scale)
    for r, yo in zip(sample, ref):
        got = y[2 * r * pitch: 2 * (r * pitch + N)].astype(np.float64)
        assert np.linalg.norm(got - yo) / np.linalg.norm(yo) <= 1e-6 * np.log2(N)
    if pitch > N and not inplace:
        # the gaps between rows are not touched
        gaps = y.reshape(rows, 2 * pitch)[:, 2 * N:]
        assert np.all(gaps == 7.0)
    if not inplace:
        assert np.array_equal(x, x0)
