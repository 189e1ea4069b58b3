"""Reference-determinant container, mirroring ``JuES.Wavefunction.Wfn``.

Reference: ``src/Backend/Wavefunction.jl:67-88`` (struct fields) and
``src/Backend/Wavefunction.jl:94-141`` (the RHF constructor: ``nocc = fld(nelec,2)``,
``Cao = C[:,1:nocc]``, ``Cav = C[:,nocc+1:end]``, beta blocks equal to alpha).

Arrays follow Julia's memory order: every matrix and 4-index tensor is stored
column-major (numpy ``order='F'``) so that element ``X[i,j,a,b]`` sits at the same
byte offset as in the Julia array.  The C ABI reads these buffers directly.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Optional

import numpy as np


@dataclass
class Wfn:
    """Closed-shell (or unrestricted-shaped) reference wavefunction.

    Only ``nalpha``, ``nvira``, ``epsa``, ``Cao``, ``Cav``, ``Cbo``, ``Cbv`` and
    ``ao_eri`` are read by the transform / MP2 / CC entry points, exactly as in
    the reference (``src/MollerPlesset/RMP2.jl:14-22``,
    ``src/CoupledCluster/mRCCD.jl:42-46``).
    """

    energy: float
    vnuc: float
    nalpha: int
    nbeta: int
    nvira: int
    nvirb: int
    nmo: int
    unrestricted: bool
    basis: Any
    molecule: Any
    Ca: np.ndarray
    Cb: np.ndarray
    Cao: np.ndarray
    Cav: np.ndarray
    Cbo: np.ndarray
    Cbv: np.ndarray
    hao: np.ndarray
    epsa: np.ndarray
    epsb: np.ndarray
    ao_eri: np.ndarray

    @property
    def nbf(self) -> int:
        return int(self.Ca.shape[0])


def wfn_from_rhf(C: np.ndarray, eps: np.ndarray, ao_eri: np.ndarray, nocc: int,
                 hao: Optional[np.ndarray] = None, energy: float = 0.0,
                 vnuc: float = 0.0, dtype=np.float64) -> Wfn:
    """Build a ``Wfn`` the way ``Wfn{T}(::RHFWfn)`` does (Wavefunction.jl:94-141).

    ``C`` is the n x n MO coefficient matrix (AO rows, MO columns), ``eps`` the
    n orbital energies (occupied first), ``ao_eri`` the n^4 AO integrals
    (mu nu|lambda sigma) indexed ``[mu,nu,lambda,sigma]``.
    """
    C = np.asfortranarray(np.asarray(C, dtype=dtype))
    n = C.shape[0]
    if C.shape != (n, n):
        raise ValueError("C must be square (nbf x nmo)")
    eps = np.asarray(eps, dtype=dtype).copy()
    if ao_eri is None:
        g = None   # density-fitted paths read C and eps only
    else:
        g = np.asfortranarray(np.asarray(ao_eri, dtype=dtype))
        if g.shape != (n, n, n, n):
            raise ValueError("ao_eri must be nbf^4")
    if hao is None:
        hao = np.zeros((n, n), dtype=dtype, order="F")
    nv = n - nocc
    Cao = np.asfortranarray(C[:, :nocc])
    Cav = np.asfortranarray(C[:, nocc:])
    return Wfn(energy=energy, vnuc=vnuc, nalpha=nocc, nbeta=nocc, nvira=nv,
               nvirb=nv, nmo=n, unrestricted=False, basis=None, molecule=None,
               Ca=C, Cb=C, Cao=Cao, Cav=Cav, Cbo=Cao, Cbv=Cav,
               hao=np.asfortranarray(np.asarray(hao, dtype=dtype)),
               epsa=eps, epsb=eps.copy(), ao_eri=g)
