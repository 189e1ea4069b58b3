"""Oracle MP2 and converged RCCD energies of the nbf=200 synthetic system (FP64 numpy).

The MO blocks are built from the B factors (oracle/df_blocks.py), the same numbers as
get_eri's up to rounding, at O(naux n^3) instead of the n^5 transform; the CCD sweeps are the
mRCCD.jl GEMM form with FP64 DIIS from the MP2 guess.  Writes the "S200" entry of
synthetic_golden.json.  Takes ~25 min on 8 cores.  Test infrastructure only.
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "jues.jl_gb300")]

import numpy as np  # noqa: E402

from oracle import ccd  # noqa: E402
from oracle.df_blocks import rccd_blocks_from_B  # noqa: E402
from oracle.mp2 import rmp2_energy  # noqa: E402
from juesgpu.synthetic import make_named  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "synthetic_golden.json")


def main():
    t0 = time.time()
    s = make_named("S200")
    ints = rccd_blocks_from_B(s.B, s.C, s.nocc)
    class W:   # the sweeps only read nalpha, epsa and the blocks
        nalpha, epsa = s.nocc, s.eps
    w = W()
    rec = {"mp2": rmp2_energy(ints[0], s.eps, s.nocc)}
    print("mp2", rec["mp2"], flush=True)
    log = []
    e = ccd.do_rccd(w, maxit=40, r_conv=1e-9, guess="mp2", integrals=ints, log=log)
    rec["ccd_mp2guess_diis"] = {"energy": e, "niter": len(log), "log": log, "r_conv": 1e-9}
    rec["seconds"] = time.time() - t0
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    data["S200"] = rec
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1)
    print("S200", e, len(log), rec["seconds"], flush=True)


if __name__ == "__main__":
    main()
