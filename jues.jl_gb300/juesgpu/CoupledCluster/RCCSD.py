"""Mirror of ``JuES.CoupledCluster.RCCSD`` (src/CoupledCluster/RCCSD.jl:33-116).

40 Jacobi sweeps from T1 = 0, T2 = <ij|ab>/D, no DIIS, as the reference; returns E or
(E, T2) with ``return_T``.  ``return_T1=True`` also returns t1 (an addition).
"""
from ._solve import solve


def do_rccsd(refWfn, maxit=40, return_T=False, *, precision="fp64", diis=False, r_conv=0.0,
             e_conv=0.0, diis_size=6, refine=0, transform_precision=None, return_T1=False, device=0,
             return_log=False, ccsd_fae="rccsd", **kwargs):
    e, t1, T2, nit, log = solve(1, refWfn, device=device, maxit=maxit, e_conv=e_conv, r_conv=r_conv,
                                diis=diis, diis_size=diis_size, precision=precision, guess="mp2",
                                refine=refine, transform_precision=transform_precision, ccsd_fae=ccsd_fae)
    if return_log:
        return e, log
    if return_T1:
        return e, t1, T2
    return (e, T2) if return_T else e
