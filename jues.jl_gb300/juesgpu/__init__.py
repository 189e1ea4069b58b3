"""juesgpu: GB300 implementation of the JuES correlated-method hot path.

The modules mirror JuES's own (``JuES.Transformation``, ``JuES.IntegralTransformation``,
``JuES.MollerPlesset``, ``JuES.CoupledCluster.{RCCD,mRCCD,RCCSD,mRCCSD}``) and call
``libjuesgpu.so`` through its C ABI.  Arrays use Julia's column-major layout.
"""
from . import Wavefunction, synthetic  # noqa: F401
from ._lib import JuESError, NotConverged, context, load  # noqa: F401

__all__ = ["Wavefunction", "synthetic", "Transformation", "IntegralTransformation",
           "MollerPlesset", "CoupledCluster", "context", "load", "JuESError", "NotConverged"]


def __getattr__(name):
    import importlib
    if name in ("Transformation", "IntegralTransformation", "MollerPlesset", "CoupledCluster"):
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
