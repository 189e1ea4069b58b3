"""Mirror of ``JuES.CoupledCluster.RCCD`` (src/CoupledCluster/RCCD.jl:33-83).

The reference runs exactly 40 Jacobi sweeps from T2 = (ij|ab)/D with no DIIS and no
convergence test; those are the defaults here.
"""
from ._solve import solve


def do_rccd(refWfn, maxit=40, doprint=False, return_T2=False, *, precision="fp64", guess="ovov",
            diis=False, r_conv=0.0, e_conv=0.0, diis_size=6, refine=0, transform_precision=None, device=0, **kwargs):
    e, _, T2, nit, log = solve(0, refWfn, device=device, maxit=maxit, e_conv=e_conv, r_conv=r_conv,
                               diis=diis, diis_size=diis_size, precision=precision, guess=guess,
                               refine=refine, transform_precision=transform_precision)
    if doprint:
        for it, en, rn, ms, _p in log:
            print(f"{it - 1} @CCD {en}")
    return (e, T2) if return_T2 else e
