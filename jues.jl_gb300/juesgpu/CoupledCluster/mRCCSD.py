"""Mirror of ``JuES.CoupledCluster.mRCCSD`` (src/CoupledCluster/mRCCSD.jl:35-101), the 6-block
form.  The same solve as RCCSD.do_rccsd except for the t1 term of Fae, which contracts <me|af>
as mRCCSD.jl:140 does (RCCSD.jl:190 and the textbook closed-shell equations use <ma|ef>); the two
converge to energies ~1e-12 Eh apart on the test systems.
"""
from . import RCCSD


def do_rccsd(refWfn, maxit=40, return_T=False, **kwargs):
    """mRCCSD.do_rccsd: 40 Jacobi sweeps from T1 = 0, T2 = <ij|ab>/D, no DIIS (mRCCSD.jl:55-101)."""
    kwargs.setdefault("ccsd_fae", "mrccsd")
    return RCCSD.do_rccsd(refWfn, maxit=maxit, return_T=return_T, **kwargs)
