"""AO->MO four-index transformation (oracle; test infrastructure).

``tei_transform`` follows ``src/Backend/Transformation.jl:39-93``: four quarter
transforms in the order sigma->b with C4 (:71-73), lambda->j with C3 (:77-79),
nu->a with C2 (:83-85), mu->i with C1 (:89-91); result (C1 C2|C3 C4) indexed
``[i,a,j,b]`` (chemists' notation).

``get_eri`` follows ``src/Backend/IntegralTransformation.jl:38-101``.
"""
import numpy as np


def tei_transform(gao, C1, C2=None, C3=None, C4=None, name="default"):
    if C2 is None:                      # 2-argument form, Transformation.jl:15-20
        C2 = C3 = C4 = C1
    t = np.tensordot(gao, C4, axes=([3], [0]))          # [mu,nu,lam,b]
    t = np.tensordot(t, C3, axes=([2], [0]))            # [mu,nu,b,j]
    t = np.transpose(t, (0, 1, 3, 2))                   # [mu,nu,j,b]
    t = np.tensordot(t, C2, axes=([1], [0]))            # [mu,j,b,a]
    t = np.transpose(t, (0, 3, 1, 2))                   # [mu,a,j,b]
    t = np.tensordot(C1, t, axes=([0], [0]))            # [i,a,j,b]
    return t


def eri_coefficients(wfn, eri_string, notation="phys", fcn=0):
    """The (C1,C2,C3,C4) selection of IntegralTransformation.jl:41-70."""
    if len(eri_string.encode()) != 4:
        raise ValueError(f"Invalid string given to get_eri: {eri_string}")
    s = eri_string
    if notation == "phys":
        s = s[0] + s[2] + s[1] + s[3]
    Cs = []
    for ch in s:
        if ch == "o":
            Cs.append(wfn.Cbo[:, fcn:])
        elif ch == "O":
            Cs.append(wfn.Cao[:, fcn:])
        elif ch == "v":
            Cs.append(wfn.Cbv)
        elif ch == "V":
            Cs.append(wfn.Cav)
        else:
            # the reference pushes nothing and fails on the 4-way unpack (:70)
            raise ValueError(f"Invalid string given to get_eri: {eri_string}")
    return Cs


def get_eri(wfn, eri_string, notation="phys", fcn=0):
    C1, C2, C3, C4 = eri_coefficients(wfn, eri_string, notation, fcn)
    V = tei_transform(wfn.ao_eri, C1, C2, C3, C4)          # :94, chem [i,a,j,b]
    if notation == "phys":
        V = np.transpose(V, (0, 2, 1, 3))                  # :96-98, [i,j,a,b]
    return np.ascontiguousarray(V)
