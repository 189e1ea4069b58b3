"""CPU oracle for the JuES correlated-method hot path.

TEST INFRASTRUCTURE ONLY.  This package is a plain numpy (FP64) restatement of
the reference Julia code, function by function, each citing the reference
``file:line`` it follows.  It is imported only by ``tests/``,
``__graft_entry__.smoke()`` (as the checker) and ``bench.py``'s CPU-baseline
leg.  The product (``libjuesgpu.so`` and the ``juesgpu`` host package) never
imports or calls it, and has no CPU fallback.

Parity pin: the reference cannot run here (it is Julia; its arithmetic lives in
TensorOperations.jl 2.2.0 / Strided.jl 0.3.5 / OpenBLAS 0.3.9, none vendored).
The restatement is pinned against the reference's own known answers for
H2O/STO-3G (``test/TestMollerPlesset.jl:35``, ``test/TestCoupledCluster.jl:41-46``)
and H2/STO-3G AO integrals (``test/TestWavefunction.jl:33-35``), reproduced from
integrals computed by ``tests/golden/make_sto3g_fixtures.py`` and committed as
``tests/golden/*.npz``; and by cross-checking the two independent CC forms of
the reference (``RCCD.jl`` einsum vs ``mRCCD.jl`` GEMM, ``RCCSD.jl`` vs
``mRCCSD.jl``).
"""
from .transform import tei_transform, get_eri  # noqa: F401
from .mp2 import do_rmp2, rmp2_energy, df_rmp2  # noqa: F401
