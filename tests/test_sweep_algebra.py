"""The device CCD sweep's contraction sequence, restated in numpy, against the reference's
equations (no GPU).

`ccd_sweep` (csrc/cc.cu) does not evaluate RCCD.jl's T2 update term by term: Wabef is never
formed, the (i,a)<->(j,b) image terms go through one Z array that the finalisation
symmetrises, the two Fmi terms ride in the hole-hole ladder, and the energy is one dot product
with precomputed weights.  Each GETT below is one device contraction, written with the same
operands and index roles; the result must equal RCCD.jl's einsum form (oracle.ccd.jl_cciter)
and the reference energy to rounding.
"""
import numpy as np

from oracle import ccd
from oracle.mp2 import denominators
from juesgpu.synthetic import make_named

E = lambda s, *ops: np.einsum(s, *ops, optimize=True)  # noqa: E731


def device_form_sweep(T, oovv, vvvv, oooo, ovov, ovvo, D):
    o = T.shape[0]
    Tt = 2.0 * T - T.transpose(1, 0, 2, 3)                       # t_tilde
    Fae = -E("mnaf,mnef->ae", Tt, oovv)                           # ccd_fae
    Fmi = E("mnef,inef->mi", oovv, Tt)                            # ccd_fmi
    Wp = oooo + E("mnef,ijef->mnij", oovv, T)                     # ccd_x: W' = oooo + X
    d = np.eye(o)
    Wp = Wp - E("mi,nj->mnij", d, Fmi) - E("nj,mi->mnij", d, Fmi)  # wp_fmi: the two Fmi terms
    L = oovv + E("mnij,mnab->ijab", Wp, T) + E("ijef,abef->ijab", T, vvvv)   # hh and pp ladders
    WJ = ovvo + 0.5 * E("mnef,njfb->mbej", oovv, Tt) - 0.5 * E("nmef,njfb->mbej", oovv, T)   # ccd_wj
    WK = -ovov.transpose(0, 1, 3, 2) + 0.5 * E("jnfb,nmef->mbej", T, oovv)                 # ccd_wk
    W12 = 2.0 * WJ + WK                                           # axpby
    Z = (E("ijae,be->ijab", T, Fae)                               # ccd_z_fae
         + E("imae,mbej->ijab", T, W12)                           # ccd_ring x3
         - E("miae,mbej->ijab", T, WJ)
         + E("mibe,maej->ijab", T, WK))
    return (L + Z + Z.transpose(1, 0, 3, 2)) / D                  # t2_finalize


def energy_device_form(T, oovv):
    return float(np.sum(T * (2.0 * oovv - oovv.transpose(1, 0, 2, 3))))


def test_device_sweep_equals_reference_update():
    s = make_named("S25")
    w = s.wfn()
    oovv, ovov, ovvo, oooo, vvvv = ccd.make_rccd_integrals(w)
    D = denominators(w.epsa, w.nalpha)
    # MP2 amplitudes, then one reference sweep: a pair-symmetric T that is not a fixed point
    T0 = oovv / D
    T = ccd.jl_cciter(T0, oovv, vvvv, oooo, ovov, ovvo, D)
    assert np.abs(T - T.transpose(1, 0, 3, 2)).max() < 1e-14
    ref = ccd.jl_cciter(T, oovv, vvvv, oooo, ovov, ovvo, D)
    dev = device_form_sweep(T, oovv, vvvv, oooo, ovov, ovvo, D)
    assert np.abs(dev - ref).max() < 1e-12 * np.abs(ref).max()
    assert abs(energy_device_form(T, oovv) - ccd.ccenergy(T, oovv)) < 1e-13 * abs(ccd.ccenergy(T, oovv))


def test_ccsd_wabef_t1_terms_through_y():
    # ccsd_sweep never forms Wabef: its t1 parts, sum_ef Ttau[ij,ef] (-t1[m,b] <am|ef> - t1[m,a]
    # <mb|ef>), become -sum_m t1[m,b] Y[ij,a,m] with Y = Ttau . <am|ef>, plus its (i,a)<->(j,b)
    # image, which the finalisation adds (Z[i,j,a,b] + Z[j,i,b,a]).  On real integrals and a
    # pair-symmetric Ttau the two agree to rounding.
    from oracle import ccsd
    w = make_named("S25").wfn()
    oooo, ooov, oovv, ovov, ovvv, vvvv = ccsd.make_rccsd_integrals(w)
    o, v = w.nalpha, oovv.shape[2]
    rng = np.random.default_rng(3)
    t1 = 0.05 * rng.normal(size=(o, v))
    T2 = 0.05 * rng.normal(size=(o, o, v, v))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))                       # pair symmetry
    Ttau = T2 + E("ia,jb->ijab", t1, t1)
    # the reference's form: Wabef's t1 parts (<am|ef> = ovvv[m,a,f,e], <mb|ef> = ovvv[m,b,e,f])
    W1 = -E("mb,mafe->abef", t1, ovvv) - E("ma,mbef->abef", t1, ovvv)
    ref = E("ijef,abef->ijab", Ttau, W1)
    # the device form: ccsd_y then ccsd_y_t1 into Z, symmetrised by t2_finalize
    Y = E("ijef,mafe->ijam", Ttau, ovvv)
    Z = -E("ijam,mb->ijab", Y, t1)
    dev = Z + Z.transpose(1, 0, 3, 2)
    assert np.abs(dev - ref).max() < 1e-14 * max(1.0, np.abs(ref).max())
