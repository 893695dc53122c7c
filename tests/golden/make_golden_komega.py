"""Generate the k-omega golden fixtures (tests/golden/komega_cases.json and
.npz) from the jvsip reference: kw.c's komega() sequence
(examples/komegaExamples/kw_c/kw.c:8-26 -- vsip_vmmul_f ROW and COL,
vsip_rcfftmop_f ROW, vsip_ccfftmip_f COL, vsip_mcmagsq_f, vsip_smmul_f,
vsip_madd_f) run by the reference library (oracle/_ref/libvsip_ref.so) on
seeded data with the reference's own Hanning tapers
(vsip_vcreate_hanning_f), in the layouts kw.c creates (freq and gram
column-major) and others.  Each case records whether the oracle
(pyoracle.komega_f) reproduced every output bit for bit.  Inputs come from the
host-exact U[-1,1) stream (regenerated by the readers); outputs up to 64 KB are
stored whole, larger ones as a SHA-256 and a sample of 4096 elements.

    python tests/golden/make_golden_komega.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import pyoracle as O  # noqa: E402
import pyref as R  # noqa: E402
from golden_cases import komega_views as views  # noqa: E402

# (id, Nsens, Nts, data pitch, data offset, freq layout, gram layout, gram offset, scale, seed)
CASES = [
    ("kw_8x16", 8, 16, 16, 0, "col", "col", 0, 0.25, 1),
    ("kw_16x64_pitched", 16, 64, 70, 2, "col", "row", 3, 1.0 / 3.0, 2),
    ("kw_128x512", 128, 512, 512, 0, "col", "col", 0, 0.125, 3),
    ("kw_128x1024", 128, 1024, 1024, 0, "col", "col", 0, 0.1, 4),
    ("kw_96x1536_rowfreq", 96, 1536, 1540, 4, "row", "col", 5, 0.5, 5),
    ("kw_12x250", 12, 250, 250, 0, "col", "row", 0, 1.0, 6),
    ("kw_60x2048", 60, 2048, 2048, 0, "row", "row", 0, 0.0625, 7),
    ("kw_64x256_rowfreq", 64, 256, 258, 2, "row", "row", 1, 0.2, 8),
]


def main():
    R.build()
    cases, arrays = [], {}
    for case in CASES:
        cid, Ns, Nt = case[0], case[1], case[2]
        case = dict(zip(("id", "Nsens", "Nts", "pitch", "doff", "freq", "gram", "goff", "scale", "seed"), case))
        ts, arr = R.hanning_f(Nt), R.hanning_f(Ns)
        d1, f1, g1, sc = views(case)
        R.komega_f(ts, arr, d1, f1, g1, float(sc))
        d2, f2, g2, _ = views(case)
        O.komega_f(ts, arr, d2, f2, g2, sc)
        exact = bool(np.array_equal(d1.buf, d2.buf) and np.array_equal(f1.buf, f2.buf) and
                     np.array_equal(g1.buf, g2.buf))
        c = dict(case)
        c["oracle_bit_exact"] = exact
        cases.append(c)
        arrays[cid + "__ts"] = ts
        arrays[cid + "__arr"] = arr
        for k, v in (("data_out", d1.buf), ("freq_out", f1.buf), ("gram_out", g1.buf)):
            c[k + "_sha256"] = hashlib.sha256(v.tobytes()).hexdigest()
            if v.nbytes <= 64 * 1024:
                arrays[cid + "__" + k] = v
            else:
                idx = np.unique(np.linspace(0, v.size - 1, 4096).astype(np.int64))
                arrays[cid + "__" + k + "__idx"] = idx
                arrays[cid + "__" + k + "__val"] = v[idx]
    with open(os.path.join(HERE, "komega_cases.json"), "w") as f:
        json.dump(dict(cases=cases, source="jvsip reference kw.c komega() sequence, oracle/Makefile.ref"), f,
                  indent=1)
    np.savez_compressed(os.path.join(HERE, "komega_cases.npz"), **arrays)
    print(f"{len(cases)} k-omega cases, oracle bit-exact on {sum(c['oracle_bit_exact'] for c in cases)}")


if __name__ == "__main__":
    main()
