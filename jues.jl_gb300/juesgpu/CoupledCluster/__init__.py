"""Mirror of ``JuES.CoupledCluster`` (src/CoupledCluster/CoupledCluster.jl).

``defaults`` are the module defaults of CoupledCluster.jl:36-43.
"""
defaults = {"cc_max_iter": 50, "cc_max_rms": 1e-10, "cc_e_conv": 1e-10, "diis": False,
            "do_pT": False, "fcn": 0}

from . import AutoRCCSD, DFRCCD, PerturbativeTriples, RCCD, RCCSD, mRCCD, mRCCSD  # noqa: F401,E402
from ._solve import CCSession, solve, solve_df  # noqa: F401,E402
