"""Mirror of ``JuES.CoupledCluster.mRCCD`` (src/CoupledCluster/mRCCD.jl:38-118).

Defaults follow the reference: T2 = 0 initial amplitudes, DIIS with 6 vectors, stop when
||T2_new - T2_old|| < 1e-7 or after ``maxit`` sweeps.  The DIIS runs in FP64 (the
reference keeps its vectors in Float32).
"""
from ._solve import solve


def do_rccd(refWfn, maxit=40, doprint=False, return_T2=False, *, precision="fp64", guess="zero",
            r_conv=1e-7, e_conv=0.0, diis=True, diis_size=6, refine=2, transform_precision=None, device=0, return_log=False):
    e, _, T2, nit, log = solve(0, refWfn, device=device, maxit=maxit, e_conv=e_conv, r_conv=r_conv,
                               diis=diis, diis_size=diis_size, precision=precision, guess=guess,
                               refine=refine, transform_precision=transform_precision)
    if doprint:
        for it, en, rn, ms, _p in log:
            print(f"@CCD {en:20.17f}")
        print(f"CCD iterations computed in {sum(r[3] for r in log) / 1e3} s")
    out = (e, T2) if return_T2 else e
    return (out, log) if return_log else out
