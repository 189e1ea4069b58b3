"""The folded ladders of the split sweeps (csrc/cc.cu pair_x / pair_l / pair_y, csrc/kernels.cu
pair_fold_kernel / pair_unfold_kernel / t2_finalize_smem_kernel<*, true>), restated in numpy on
the same flat column-major indices, against the plain contractions (no GPU).

With the pair symmetry T[i,j,a,b] = T[j,i,b,a], the ladders' output L, X and CCSD's Y are
evaluated over occupied pairs p = (i <= j) and virtual pairs q = (a <= b) in a symmetric (+) and
an antisymmetric (-) part; the unfolded results must equal oovv + W'^T.T + T.vvvv^T,
oovv.T^T and ooovQ + T.<am|ef> to rounding, on the S25 system's integrals and amplitudes.
"""
import numpy as np
import pytest

from oracle import ccd, ccsd
from oracle.mp2 import denominators
from juesgpu.synthetic import make_named

fl = lambda a: np.asarray(a).reshape(-1, order="F")  # noqa: E731


def pair_decode(p):
    """kernels.cu pair_ab: p = b(b+1)/2 + a, a <= b."""
    p = np.asarray(p, dtype=np.int64)
    b = ((np.sqrt(8.0 * p + 1.0) - 1.0) * 0.5).astype(np.int64)
    b = np.where(b * (b + 1) // 2 > p, b - 1, b)
    b = np.where((b + 1) * (b + 2) // 2 <= p, b + 1, b)
    return p - b * (b + 1) // 2, b


def pair_fold(src, R, rowpair, rd, rs0, rs1, d, ke, kf, scale, diag_half):
    """pair_fold_kernel: [out+ | out-], out_s[r + R q] for the K pair q = (e <= f)."""
    nk = d * (d + 1) // 2
    e, f = pair_decode(np.arange(nk))
    r = np.arange(R)
    if rowpair:
        a, b = pair_decode(r)
        ro = a * rs0 + b * rs1
    else:
        ro = (r % rd) * rs0 + (r // rd) * rs1
    i1 = ro[:, None] + (e * ke + f * kf)[None, :]
    i2 = ro[:, None] + (f * ke + e * kf)[None, :]
    assert min(i1.min(), i2.min()) >= 0 and max(i1.max(), i2.max()) < src.size
    c = np.where(diag_half & (e == f), 0.5 * scale, scale)[None, :]
    x, y = src[i1], src[i2]
    return np.concatenate([fl(c * (x + y)), fl(c * (x - y))])


def pair_unfold(P, npc, base, o, C, sij, sc, tp, tc, size):
    """pair_unfold_kernel: out[(i + o j) sij + c sc] = base + P+ + sgn P- (no P- for i = j)."""
    ij = np.arange(o * o)
    i, j = ij % o, ij // o
    i0, j0 = np.minimum(i, j), np.maximum(i, j)
    p = j0 * (j0 + 1) // 2 + i0
    c = np.arange(C)
    pi = p[:, None] * tp + c[None, :] * tc
    assert pi.min() >= 0 and (npc + pi).max() < P.size
    sgn = np.where(i == j, 0.0, np.where(i < j, 1.0, -1.0))[:, None]
    oi = ij[:, None] * sij + c[None, :] * sc
    out = np.zeros(size)
    out[oi] = (base[oi] if base is not None else 0.0) + P[pi] + sgn * P[npc + pi]
    return out


def unfold_ladder(Lpm, o, v):
    """t2_finalize_smem_kernel's L[i,j,a,b] from [L+ | L-] (block q = (a <= b), column q)."""
    np_, nq = o * (o + 1) // 2, v * (v + 1) // 2
    Lp = Lpm[: np_ * nq].reshape(np_, nq, order="F")
    Lm = Lpm[np_ * nq:].reshape(np_, nq, order="F")
    L = np.zeros((o, o, v, v))
    for q in range(nq):
        a, b = (int(x) for x in pair_decode(q))
        for i in range(o):
            for j in range(o):
                i0, j0 = min(i, j), max(i, j)
                pij = j0 * (j0 + 1) // 2 + i0
                lm = 0.0 if (i == j or a == b) else (Lm[pij, q] if i < j else -Lm[pij, q])
                L[i, j, a, b] = Lp[pij, q] + lm
                L[i, j, b, a] = Lp[pij, q] - lm
    return L


def gemm_rows(A, B):
    """C[m, n] = sum_k A[m, k] B[n, k]: gett_tc_views with A and B as row-major-K packs."""
    return A @ B.T


def folded(T, oovv, vvvv, oooo, Wp_extra=None, ovvv=None, ooovQ=None):
    """pair_begin + pair_x + pair_l (+ pair_y): W', L and Y through the folded contractions."""
    o, v = T.shape[0], T.shape[2]
    oo, vv, ov = o * o, v * v, o * v
    np_, nq = o * (o + 1) // 2, v * (v + 1) // 2
    blk = lambda a, k, r, c: a[k * r * c:(k + 1) * r * c].reshape(r, c, order="F")  # noqa: E731
    Bpm = pair_fold(fl(vvvv), nq, True, 0, 1, v, v, vv, vv * v, 0.5, True)
    Xw = pair_fold(fl(oovv), oo, False, oo, 1, 0, v, oo, oo * v, 0.5, True)
    Opm = pair_fold(fl(oovv), np_, True, 0, 1, o, v, oo, oo * v, 0.5, False)
    Apm = pair_fold(fl(T), np_, True, 0, 1, o, v, oo, oo * v, 1.0, False)
    Xpm = np.concatenate([fl(gemm_rows(blk(Xw, k, oo, nq), blk(Apm, k, np_, nq))) for k in range(2)])
    Wp = pair_unfold(Xpm, oo * np_, fl(oooo), o, oo, oo, 1, oo, 1, oo * oo).reshape(o, o, o, o, order="F")
    if Wp_extra is not None:
        Wp = Wp + Wp_extra
    Cpm = pair_fold(fl(Wp), np_, True, 0, oo, oo * o, o, 1, o, 0.5, True)
    Lpm = []
    for k in range(2):
        A, C, B = blk(Apm, k, np_, nq), blk(Cpm, k, np_, np_), blk(Bpm, k, nq, nq)
        Lpm.append(fl(blk(Opm, k, np_, nq) + gemm_rows(np.hstack([C, A]), np.hstack([A.T, B]))))
    L = unfold_ladder(np.concatenate(Lpm), o, v)
    Y = None
    if ovvv is not None:
        Yw = pair_fold(fl(ovvv), ov, False, v, o, 1, v, ov * v, ov, 0.5, True)
        Ypm = np.concatenate([fl(gemm_rows(blk(Apm, k, np_, nq), blk(Yw, k, ov, nq))) for k in range(2)])
        Y = pair_unfold(Ypm, np_ * ov, fl(ooovQ), o, ov, 1, oo, 1, np_, oo * ov).reshape(o, o, v, o, order="F")
    return Wp, L, Y


def test_pair_decode_order():
    a, b = pair_decode(np.arange(66))
    want = [(x, y) for y in range(11) for x in range(y + 1)]
    assert list(zip(a.tolist(), b.tolist())) == want


def test_folded_ladders_equal_plain_ccd():
    s = make_named("S25")
    w = s.wfn()
    oovv, ovov, ovvo, oooo, vvvv = ccd.make_rccd_integrals(w)
    D = denominators(w.epsa, w.nalpha)
    T = ccd.jl_cciter(oovv / D, oovv, vvvv, oooo, ovov, ovvo, D)   # pair-symmetric, not a fixed point
    assert np.abs(T - T.transpose(1, 0, 3, 2)).max() < 1e-14
    o = T.shape[0]
    # any pair-symmetric addition to W' (the Fmi terms of wp_fmi are one)
    rng = np.random.default_rng(3)
    S = 1e-2 * rng.standard_normal((o, o, o, o))
    Sx = S + S.transpose(1, 0, 3, 2)
    Wp, L, _ = folded(T, oovv, vvvv, oooo, Wp_extra=Sx)
    X = np.einsum("mnef,ijef->mnij", oovv, T)
    assert np.abs(Wp - (oooo + X + Sx)).max() < 1e-13 * max(1.0, np.abs(Wp).max())
    Lp = oovv + np.einsum("mnij,mnab->ijab", oooo + X + Sx, T) + np.einsum("ijef,abef->ijab", T, vvvv)
    assert np.abs(L - Lp).max() < 1e-13 * max(1.0, np.abs(Lp).max())


def test_folded_y_equals_plain_ccsd():
    s = make_named("S25")
    w = s.wfn()
    oooo, _, oovv, _, ovvv, vvvv = ccsd.make_rccsd_integrals(w)
    o, v = oovv.shape[0], oovv.shape[2]
    rng = np.random.default_rng(5)
    R = 1e-2 * rng.standard_normal((o, o, v, v))
    t1 = 1e-2 * rng.standard_normal((o, v))
    Ttau = R + R.transpose(1, 0, 3, 2) + np.einsum("ia,jb->ijab", t1, t1)   # T2 + tau: pair-symmetric
    ooovQ = rng.standard_normal((o, o, v, o))
    _, L, Y = folded(Ttau, oovv, vvvv, oooo, ovvv=ovvv, ooovQ=ooovQ)
    Yp = ooovQ + np.einsum("ijef,mafe->ijam", Ttau, ovvv)
    assert np.abs(Y - Yp).max() < 1e-13 * max(1.0, np.abs(Yp).max())
    X = np.einsum("mnef,ijef->mnij", oovv, Ttau)
    Lp = oovv + np.einsum("mnij,mnab->ijab", oooo + X, Ttau) + np.einsum("ijef,abef->ijab", Ttau, vvvv)
    assert np.abs(L - Lp).max() < 1e-13 * max(1.0, np.abs(Lp).max())


def pair_decode32(p):
    """kernels.cu pair_ab32: the FP32 square root, then the integer correction."""
    p = np.asarray(p, dtype=np.int64)
    b = ((np.sqrt(np.float32(8.0) * p.astype(np.float32) + np.float32(1.0)) - np.float32(1.0))
         * np.float32(0.5)).astype(np.int64)
    for _ in range(2):
        b = np.where(b * (b + 1) // 2 > p, b - 1, b)
        b = np.where((b + 1) * (b + 2) // 2 <= p, b + 1, b)
    return p - b * (b + 1) // 2, b


def test_pair_decode32_exact():
    p = np.arange(1 << 20)
    a, b = pair_decode32(p)
    assert np.all((a >= 0) & (a <= b) & (b * (b + 1) // 2 + a == p))
    a2, b2 = pair_decode(p)
    assert np.array_equal(a, a2) and np.array_equal(b, b2)


def inv_folded(e, o, v):
    """inv_denominators_folded_kernel: 1/D[i0,j0,a,b] at p + np q, sums in the same order."""
    np_, nq = o * (o + 1) // 2, v * (v + 1) // 2
    x = np.arange(np_ * nq)
    i, j = pair_decode32(x % np_)
    a, b = pair_decode32(x // np_)
    return 1.0 / (e[i] + e[j] - e[o + a] - e[o + b])


def finalize_fold(Lpm, Z, invF, o, v):
    """t2_finalize_fold_kernel: per block (a <= b), Z_ab and Z_ba staged, each pair (i0 <= j0)
    forms u/D and w/D over its four Z elements, then Tn = the staged values."""
    np_, nq = o * (o + 1) // 2, v * (v + 1) // 2
    Zf = fl(Z)
    Tn = np.zeros(o * o * v * v)
    oo = o * o
    for q in range(nq):
        a, b = (int(x) for x in pair_decode(q))
        ab, ba = oo * (a + v * b), oo * (b + v * a)
        za = Zf[ab:ab + oo].reshape(o, o, order="F").copy()   # za[i, j] = Z[i,j,a,b]
        zb = Zf[ba:ba + oo].reshape(o, o, order="F").copy()
        lp, lm = Lpm[np_ * q:np_ * q + np_], Lpm[np_ * nq + np_ * q:np_ * nq + np_ * q + np_]
        for p in range(np_):
            i0, j0 = (int(x) for x in pair_decode32(p))
            lpv, lmv = lp[p], (0.0 if (i0 == j0 or a == b) else lm[p])
            inv = invF[p + np_ * q]
            u = ((lpv + lmv) + (za[i0, j0] + zb[j0, i0])) * inv
            w = ((lpv - lmv) + (za[j0, i0] + zb[i0, j0])) * inv
            za[i0, j0] = u
            zb[j0, i0] = u
            za[j0, i0] = w
            zb[i0, j0] = w
        Tn[ab:ab + oo] = fl(za)
        if a != b:
            Tn[ba:ba + oo] = fl(zb)
    return Tn.reshape(o, o, v, v, order="F")


def test_folded_finalisation_equals_plain():
    rng = np.random.default_rng(7)
    o, v = 4, 6
    R = rng.standard_normal((o, o, v, v))
    L = R + R.transpose(1, 0, 3, 2)                       # a pair-symmetric ladder output
    Z = rng.standard_normal((o, o, v, v))                 # any Z
    e = np.sort(rng.standard_normal(o + v))
    D = e[:o, None, None, None] + e[None, :o, None, None] - e[None, None, o:, None] - e[None, None, None, o:]
    invD = 1.0 / D
    invF = inv_folded(e, o, v)
    i, j = np.triu_indices(o)
    assert np.array_equal(np.sort(invF[:o * (o + 1) // 2]), np.sort(invD[i, j, 0, 0]))
    np_, nq = o * (o + 1) // 2, v * (v + 1) // 2
    # [L+ | L-]: L_s[p, q] = 1/2 (L[i,j,a,b] + s L[i,j,b,a])
    Lpm = pair_fold(fl(L), np_, True, 0, 1, o, v, o * o, o * o * v, 0.5, False)
    Tn = finalize_fold(Lpm, Z, invF, o, v)
    want = (L + Z + Z.transpose(1, 0, 3, 2)) * invD
    assert np.abs(Tn - want).max() < 1e-13 * np.abs(want).max()
    assert np.array_equal(Tn, Tn.transpose(1, 0, 3, 2))   # pair-symmetric to the bit


def _symmetric_blocks(o, v, rng, nq=5):
    """Physicists' <pq|rs> with the full 8-fold symmetry, from a factorised (pr|qs)."""
    n = o + v
    B = rng.standard_normal((n, n, nq))
    B = B + B.transpose(1, 0, 2)
    phys = np.einsum("prQ,qsQ->pqrs", B, B)   # <pq|rs> = (pr|qs)
    O, V = slice(0, o), slice(o, n)
    return (np.asfortranarray(phys[O, O, V, V]), np.asfortranarray(phys[V, V, V, V]),
            np.asfortranarray(phys[O, O, O, O]), np.asfortranarray(phys[O, V, V, V]))


@pytest.mark.parametrize("o,v", [(1, 1), (1, 3), (2, 1), (3, 4), (5, 7), (8, 3)])
def test_folded_chain_edge_sizes(o, v):
    rng = np.random.default_rng(100 * o + v)
    oovv, vvvv, oooo, ovvv = _symmetric_blocks(o, v, rng)
    R = rng.standard_normal((o, o, v, v))
    T = R + R.transpose(1, 0, 3, 2)
    ooovQ = rng.standard_normal((o, o, v, o))
    Wp, L, Y = folded(T, oovv, vvvv, oooo, ovvv=ovvv, ooovQ=ooovQ)
    X = np.einsum("mnef,ijef->mnij", oovv, T)
    Lp = oovv + np.einsum("mnij,mnab->ijab", oooo + X, T) + np.einsum("ijef,abef->ijab", T, vvvv)
    Yp = ooovQ + np.einsum("ijef,mafe->ijam", T, ovvv)
    scale = lambda a: max(1.0, np.abs(a).max())  # noqa: E731
    assert np.abs(Wp - (oooo + X)).max() < 1e-12 * scale(Wp)
    assert np.abs(L - Lp).max() < 1e-12 * scale(Lp)
    assert np.abs(Y - Yp).max() < 1e-12 * scale(Yp)
    # the finalisation from the folded ladders
    e = np.sort(rng.standard_normal(o + v)) + np.r_[np.full(o, -5.0), np.full(v, 5.0)]
    D = e[:o, None, None, None] + e[None, :o, None, None] - e[None, None, o:, None] - e[None, None, None, o:]
    Z = rng.standard_normal((o, o, v, v))
    np_, nq = o * (o + 1) // 2, v * (v + 1) // 2
    Lpm = pair_fold(fl(Lp), np_, True, 0, 1, o, v, o * o, o * o * v, 0.5, False)
    Tn = finalize_fold(Lpm, Z, inv_folded(e, o, v), o, v)
    want = (Lp + Z + Z.transpose(1, 0, 3, 2)) / D
    assert np.abs(Tn - want).max() < 1e-12 * scale(want)
    assert np.array_equal(Tn, Tn.transpose(1, 0, 3, 2))


BIG = 1 << 60


def mode_offsets(mode, n):
    """common.cuh Mode{d0, d1, s0, s1, s2}: offset (r % d0) s0 + ((r / d0) % d1) s1 + (r / (d0 d1)) s2."""
    d0, d1, s0, s1, s2 = mode
    r = np.arange(n, dtype=np.int64)
    return (r % d0) * s0 + ((r // d0) % d1) * s1 + (r // (d0 * d1 if d0 * d1 < BIG else BIG)) * s2


def mode2(d0, s0, s1):
    return (d0, BIG, s0, s1, 0)


def plain(s):
    return (BIG, 1, s, 0, 0)


def test_t1_fme_terms_as_one_gemm_on_the_ring_packs():
    """ccsd_sweep (split): sum_me (2 T2[i,m,a,e] - T2[m,i,a,e]) Fme[m,e] = [R1 | R23] . [2 Fme ; -Fme]
    with R1 = T2 packed as rows (i,a) mode2(o,1,oo), K (m,e) mode2(o,o,oov) and R23 as rows
    mode2(o,o,oo), K mode2(o,1,oov) (ring_stacks_begin), and Fme packed along K with plain(1)."""
    rng = np.random.default_rng(11)
    o, v = 3, 5
    oo, ov, oov = o * o, o * v, o * o * v
    T = rng.standard_normal((o, o, v, v))
    T = T + T.transpose(1, 0, 3, 2)
    Fme = rng.standard_normal((o, v))
    Tf, Ff = fl(T), fl(Fme)
    rows1, k1 = mode_offsets(mode2(o, 1, oo), ov), mode_offsets(mode2(o, o, oov), ov)
    rows2, k2 = mode_offsets(mode2(o, o, oo), ov), mode_offsets(mode2(o, 1, oov), ov)
    R1 = Tf[rows1[:, None] + k1[None, :]]
    R23 = Tf[rows2[:, None] + k2[None, :]]
    B = np.concatenate([2.0 * Ff[mode_offsets(plain(1), ov)], -Ff[mode_offsets(plain(1), ov)]])
    got = np.hstack([R1, R23]) @ B                      # rows r = i + o a: t1's layout
    want = np.einsum("imae,me->ia", 2.0 * T - T.transpose(1, 0, 2, 3), Fme)
    assert np.abs(got - fl(want)).max() < 1e-13
