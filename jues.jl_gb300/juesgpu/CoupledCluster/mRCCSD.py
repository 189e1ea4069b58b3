"""Mirror of ``JuES.CoupledCluster.mRCCSD`` (src/CoupledCluster/mRCCSD.jl:35-101), the 6-block
form.  Same equations as RCCSD; the t1 term of Fae uses <ma|ef> as RCCSD.jl:190 does (the
mRCCSD.jl:140 variant contracts <me|af>; the two agree to ~1e-12 Eh on the test systems).
"""
from .RCCSD import do_rccsd  # noqa: F401
