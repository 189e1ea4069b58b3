"""MP2 energy adjoint (oracle; test infrastructure).

E(g, C) = sum_{iajb} K_iajb (2 K_iajb - K_ibja) / D_ijab with K = (C_o C_v | C_o C_v) the
(ia|jb) block of ``tei_transform`` and D_ijab = e_i + e_j - e_a - e_b (RMP2.jl:24-41).

dE/dK_iajb = Gamma_iajb = 2 (2 K_iajb - K_ibja) / D_ijab.  Then
  dE/dg[mu,nu,lam,sig] = sum Gamma_iajb C_mu,i C_nu,a C_lam,j C_sig,b    (back-transform)
  dE/dC[mu,i] = sum_{ajb} Gamma_iajb (mu a|j b) + sum_{iab} Gamma_jaib (j a|mu b)
  dE/dC[mu,a] = sum_{ijb} Gamma_iajb (i mu|j b) + sum_{ija} Gamma_ibja (i b|j mu)
which for 8-fold symmetric g reduce to twice the first term each.  ``mp2_energy_torch`` gives
an independent autograd gradient (torch, CPU, FP64).
"""
import numpy as np

from .transform import tei_transform


def gamma(K, eps, o):
    """Gamma[i,a,j,b] for K[i,a,j,b] in chemists' order."""
    v = K.shape[1]
    eo, ev = eps[:o], eps[o:o + v]
    D = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    Kx = np.transpose(K, (0, 3, 2, 1))             # K[i,b,j,a] at [i,a,j,b]
    return 2.0 * (2.0 * K - Kx) / D


def mp2_energy(g, C, o, eps):
    Co, Cv = C[:, :o], C[:, o:]
    K = tei_transform(g, Co, Cv, Co, Cv)
    v = Cv.shape[1]
    eo, ev = eps[:o], eps[o:o + v]
    D = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    return float(np.sum(K * (2 * K - np.transpose(K, (0, 3, 2, 1))) / D))


def mp2_adjoint(g, C, o, eps, e_bar=1.0):
    """(E, dE/dg * e_bar, dE/dC * e_bar) for symmetric g."""
    Co, Cv = C[:, :o], C[:, o:]
    K = tei_transform(g, Co, Cv, Co, Cv)
    G = gamma(K, eps, o) * e_bar
    E = float(np.sum(K * (2 * K - np.transpose(K, (0, 3, 2, 1))) / (
        eps[:o, None, None, None] - eps[None, o:, None, None] + eps[None, None, :o, None]
        - eps[None, None, None, o:])))
    g_bar = np.einsum("iajb,mi,na,lj,sb->mnls", G, Co, Cv, Co, Cv, optimize=True)
    H = np.einsum("mnls,na,lj,sb->majb", g, Cv, Co, Cv, optimize=True)     # (mu a|j b)
    Hp = np.einsum("mnls,mi,lj,sb->injb", g, Co, Co, Cv, optimize=True)    # (i nu|j b)
    C_bar = np.zeros_like(C)
    C_bar[:, :o] = 2.0 * np.einsum("iajb,majb->mi", G, H, optimize=True)
    C_bar[:, o:] = 2.0 * np.einsum("iajb,injb->na", G, Hp, optimize=True)
    return E, g_bar, C_bar


def mp2_energy_torch(g, C, o, eps):
    """E and autograd dE/dg, dE/dC (torch CPU FP64) -- an independent check."""
    import torch
    gt = torch.tensor(np.asarray(g), dtype=torch.float64, requires_grad=True)
    Ct = torch.tensor(np.asarray(C), dtype=torch.float64, requires_grad=True)
    e = torch.tensor(np.asarray(eps), dtype=torch.float64)
    Co, Cv = Ct[:, :o], Ct[:, o:]
    K = torch.einsum("mnls,mi,na,lj,sb->iajb", gt, Co, Cv, Co, Cv)
    v = Cv.shape[1]
    D = (e[:o, None, None, None] - e[None, o:o + v, None, None] + e[None, None, :o, None]
         - e[None, None, None, o:o + v])
    E = torch.sum(K * (2 * K - K.permute(0, 3, 2, 1)) / D)
    E.backward()
    return float(E), gt.grad.numpy(), Ct.grad.numpy()
