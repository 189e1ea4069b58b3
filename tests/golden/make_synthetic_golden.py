"""Oracle energies of the seeded synthetic systems, committed as synthetic_golden.json.

The GPU parity tests compare against these numbers (the oracle is too slow to rerun at
nbf=100 inside a test).  Run: ``python tests/golden/make_synthetic_golden.py [S25 S100 ...]``;
``--ccsd-m S25 S100`` adds only the mRCCSD.jl-variant CCSD records.
Test infrastructure only.
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "jues.jl_gb300")]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from oracle import ccd, ccsd  # noqa: E402
from juesgpu.synthetic import make_named  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "synthetic_golden.json")


def run(name):
    t0 = time.time()
    w = make_named(name).wfn()
    rec = {}
    ints = ccd.make_rccd_integrals(w)
    rec["mp2"] = oracle.rmp2_energy(ints[0], w.epsa, w.nalpha)
    log = []
    e, T, nit = ccd.do_rccd(w, maxit=60, r_conv=1e-11, guess="mp2", integrals=ints, log=log,
                            return_T2=True)
    rec["ccd_mp2guess_diis"] = {"energy": e, "niter": nit, "log": log}
    log = []
    ccd.do_rccd(w, maxit=8, r_conv=None, guess="zero", integrals=ints, log=log)
    rec["ccd_zero_diis_8"] = log
    rec["ccd_t2_norm"] = float(np.linalg.norm(T))
    blocks = ccsd.make_rccsd_integrals(w)
    log = []
    e = ccsd.do_rccsd(w, form="m", fae_variant="jl", maxit=60, diis=True, r_conv=1e-11, log=log,
                      blocks=blocks)
    rec["ccsd_diis"] = {"energy": e, "niter": len(log), "log": log}
    log = []
    ccsd.do_rccsd(w, form="m", fae_variant="jl", maxit=6, log=log, blocks=blocks)
    rec["ccsd_plain_6"] = log
    rec.update(run_ccsd_m(name, w, blocks))
    rec["seconds"] = time.time() - t0
    return rec


def run_ccsd_m(name, w=None, blocks=None):
    """mRCCSD.jl's own Fae t1 term (<me|af>, mRCCSD.jl:140): converged DIIS energy and log, and
    six plain sweeps."""
    w = w if w is not None else make_named(name).wfn()
    blocks = blocks if blocks is not None else ccsd.make_rccsd_integrals(w)
    rec = {}
    log = []
    e = ccsd.do_rccsd(w, form="m", fae_variant="m", maxit=60, diis=True, r_conv=1e-11, log=log,
                      blocks=blocks)
    rec["ccsd_m_diis"] = {"energy": e, "niter": len(log), "log": log}
    log = []
    ccsd.do_rccsd(w, form="m", fae_variant="m", maxit=6, log=log, blocks=blocks)
    rec["ccsd_m_plain_6"] = log
    return rec


def main(names):
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    if names and names[0] == "--ccsd-m":
        # add only the mRCCSD.jl-variant records to existing entries
        for n in names[1:]:
            data[n].update(run_ccsd_m(n))
            with open(OUT, "w") as f:
                json.dump(data, f, indent=1)
            print(n, data[n]["ccsd_m_diis"]["energy"], flush=True)
        return
    for n in names:
        data[n] = run(n)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1)
        print(n, data[n]["ccd_mp2guess_diis"]["energy"], data[n]["ccsd_diis"]["energy"],
              data[n]["seconds"], flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or ["S25", "S100"])
