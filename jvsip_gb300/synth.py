"""Seeded synthetic inputs for benchmarks and tools (numpy only).

The stream is a counter-based SplitMix64 of (seed, index): 53-bit uniforms,
mapped to U[-1,1) (exact in double) or to N(0,1) by Box-Muller in double, then
rounded to the requested type.  It is the same stream the test fixtures use,
so the U[-1,1) draws agree bit for bit.

`batch_sequence` draws the batching configuration's instances: length N
log-uniform over the 2^a 3^b 5^c values in [64, 16384] (v = exp(U(ln 64,
ln 16384)), the smallest member >= v), rows uniform in {1..256}, 50/50
forward/inverse and VSIP_ROW/VSIP_COL.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = (1 << 64) - 1


def _mix(seed: int, idx: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = np.uint64((seed * 0xD1342543DE82EF95) & _M64) + (idx.astype(np.uint64) + np.uint64(1)) * np.uint64(
            0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def unit(seed: int, n: int, start: int = 0) -> np.ndarray:
    """n uniforms in [0, 1) (53-bit)."""
    idx = np.arange(start, start + n, dtype=np.uint64)
    return (_mix(seed, idx) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def fill(n: int, seed: int, dist: int = 0, dtype=np.float32, chunk: int = 1 << 24) -> np.ndarray:
    """n scalars: dist 0 = U[-1,1), dist 1 = N(0,1)."""
    out = np.empty(n, dtype=dtype)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        if dist == 0:
            out[s:s + m] = 2.0 * unit(seed, m, s) - 1.0
        else:
            p0 = (s // 2) * 2
            pairs = (s + m - p0 + 1) // 2
            u = unit(seed, 2 * pairs, p0).reshape(pairs, 2)
            r = np.sqrt(-2.0 * np.log(1.0 - u[:, 0]))
            t = 6.283185307179586476925286766559 * u[:, 1]
            z = np.empty(2 * pairs)
            z[0::2] = r * np.cos(t)
            z[1::2] = r * np.sin(t)
            out[s:s + m] = z[s - p0:s - p0 + m]
    return out


def smooth_lengths(lo: int = 64, hi: int = 16384):
    vals = set()
    a = 1
    while a <= hi:
        b = a
        while b <= hi:
            c = b
            while c <= hi:
                if c >= lo:
                    vals.add(c)
                c *= 5
            b *= 3
        a *= 2
    return sorted(vals)


def batch_sequence(count: int, seed: int = 6, max_bytes: float | None = None):
    """[(N, rows, dir, major)] of the batching configuration; truncated when the
    cumulative c64 bytes of one buffer would exceed max_bytes."""
    lens = smooth_lengths()
    u = unit(seed, 4 * count).reshape(count, 4)
    seq, total = [], 0.0
    lo, hi = math.log(64.0), math.log(16384.0)
    for k in range(count):
        v = math.exp(lo + (hi - lo) * u[k, 0])
        N = next(x for x in lens if x >= v - 1e-9)
        rows = 1 + min(255, int(u[k, 1] * 256))
        d = -1 if u[k, 2] < 0.5 else 1
        major = 0 if u[k, 3] < 0.5 else 1
        b = 8.0 * N * rows
        if max_bytes is not None and total + b > max_bytes:
            break
        total += b
        seq.append((N, rows, d, major))
    return seq
