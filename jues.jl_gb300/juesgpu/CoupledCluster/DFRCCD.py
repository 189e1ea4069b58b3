"""Mirror of ``JuES.CoupledCluster.DFRCCD`` (src/CoupledCluster/DF-RCCD.jl:11-54).

The reference takes its fitted integrals from ``DF.make_bmunu`` (psi4's three-index
integrals (pq|P) and J^-1/2, src/Backend/DF.jl:30-58); this library does not wrap psi4, so the
caller passes ``pqP`` and ``Jpqh`` (or the fitted b[mu,nu,Q] with ``Jpqh=None``).  The
defaults are the reference's: T2 = (ia|jb)/D, 40 Jacobi sweeps, no DIIS, no convergence
test, and WmBeJ exactly as DF-RCCD.jl:239-242 writes it (``variant="reference"``;
``variant="rccd"`` uses RCCD.jl's index order in that term).
"""
from ._solve import solve_df


def do_df_rccd(refWfn, pqP, Jpqh=None, maxit=40, doprint=False, return_T2=False, *, variant="reference",
               precision="fp64", guess="mp2", diis=False, r_conv=0.0, e_conv=0.0, diis_size=6, refine=0,
               transform_precision=None, device=0, **kwargs):
    e, T2, nit, log = solve_df(refWfn, pqP, Jpqh, variant=variant, device=device, maxit=maxit, e_conv=e_conv,
                               r_conv=r_conv, diis=diis, diis_size=diis_size, precision=precision, guess=guess,
                               refine=refine, transform_precision=transform_precision)
    if doprint:
        for it, en, rn, ms, _p in log:
            print(f"{it - 1} @CCD {en}")
    return (e, T2) if return_T2 else e
