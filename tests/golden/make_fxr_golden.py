"""Generate tests/golden/fxr.json from the reference library itself.

For the deterministic fields of ``fields.py`` (float and double), records what
the reference's fixed-rate machinery returns:

* the sampled value range and one ratio estimate with its integer sums
  (computeRadiusBuffer / estimateCRbasedonErrorBound_buffered,
  szx/src/szx.cc:475-498), at three bounds;
* the bound its search settles on for several target ratios and tolerances
  (szx/src/szx_float.cc:921-949, szx/src/szx_double.cc:918-940);
* length and sha256 of the stream ``SZx_fast_compress_args`` produces in the
  fixed-rate mode (szx/src/szx.cc:240-243, 291-294).  The reference writes it
  into a buffer of sizeof(T)*n/ratio*(1+2*tolerance) bytes; cases whose stream
  (computed first with the oracle) would not fit are not run through it.

Usage:  python tests/golden/make_fxr_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)
import fields as F  # noqa: E402
import oracle as O  # noqa: E402

FXR = 2
N = {np.float32: 1 << 18, np.float64: 1 << 17}


def bits(v) -> int:
    return int(np.float32(v).view(np.uint32))


def main():
    if O.reference() is None:
        O.build(reference=True, reference_src=os.environ.get("SZX_REFERENCE_SRC"))
    assert O.reference() is not None, "reference library not built: set SZX_REFERENCE_SRC to the reference source tree"
    out = []
    for dt in (np.float32, np.float64):
        for name in F.FIELDS:
            x = F.make(name, N[dt], dt)
            ptp = float(np.float32(x.max() - x.min()))
            est = []
            for scale in (1e-5, 1e-3, 3e-2):
                eb = float(np.float32(scale * ptp))
                cr, req, lead, rng = O.ref_fxr_estimate(x, eb)
                est.append(dict(eb=eb, cr_bits=bits(cr), sum_req=req, sum_lead=lead))
            searches = []
            for ratio in (4.0, 8.0, 16.0, 32.0):
                for tol in (0.05, 0.1):
                    eb = O.ref_fxr_bound(x, ratio, tol)
                    rec = dict(ratio=ratio, tolerance=tol, eb_bits=bits(eb))
                    s2 = O.compress(2, x, eb, 128)
                    room = int(x.itemsize * x.size / np.float32(ratio) * (1 + np.float32(tol) * 2))
                    if len(s2) + 64 < room:
                        s = O.ref_compress_args(2, x, FXR, 0.0, 0.0, ratio=ratio, tolerance=tol)
                        assert s == s2, (name, dt, ratio, tol)
                        rec.update(stream_len=len(s), stream_sha256=hashlib.sha256(s).hexdigest())
                    searches.append(rec)
            out.append(dict(field=name, dtype=np.dtype(dt).name, n=int(x.size), range_bits=bits(rng),
                            estimates=est, searches=searches))
            print(name, np.dtype(dt).name, x.size, "range", np.uint32(bits(rng)).view(np.float32),
                  "bounds", [np.uint32(s["eb_bits"]).view(np.float32) for s in searches])
    with open(os.path.join(HERE, "fxr.json"), "w") as f:
        json.dump(dict(generator="tests/golden/make_fxr_golden.py",
                       reference="szcompressor/SZx compiled from source by oracle/Makefile", fields=out), f, indent=1)


if __name__ == "__main__":
    main()
