"""ORACLE (test infrastructure only): the XCHF RHF SCF of NEO-RXCHF restated
in numpy over the C oracle's integrals.

Follows xchf1_independent/xcscf.f:2-658 (xcscf, the plain Roothaan branch
without SOSCF), xchf1_fock.f:2-361 (Fock and energy assembly, in-core
gam_2/gam_3 contractions, GAM4_DSCF) with E_from_GAM_ecore/pcore/ee/ep/1 and
S_from_GAM_1s (:786-1150), XCfock_correction (:728-783), ROOTHAN
(xcscf.f:766-953), guess_prot (:683-716) and DENDIF (:719-740).  Matrices are
numpy arrays indexed [i, j] = F(i, j); the C oracle takes them column-major.
Only the tests load this module.
"""
from __future__ import annotations

import numpy as np

try:   # imported as part of the oracle directory package
    from . import oracle as O
except ImportError:   # imported with the oracle directory on sys.path (tests)
    import oracle as O


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


def _m(v, n):
    return np.asarray(v).reshape(n, n, order="F")


class XchfIntegrals:
    """All integral tensors one XCHF SCF needs, from the C oracle."""

    def __init__(self, s):
        self.s = s
        L, h = O.lib(), O.SystemHandle(s)
        self.h = h
        ne, np_ = s.nebf, s.npbf
        self.Se, self.Sp = np.zeros(ne * ne), np.zeros(np_ * np_)
        L.orc_overlaps(h.ref, O.ptr(self.Se), O.ptr(self.Sp))
        self.Gecore, self.Gpcore = np.zeros(ne * ne), np.zeros(np_ * np_)
        L.orc_gam_epcore(h.ref, O.ptr(self.Gecore), O.ptr(self.Gpcore))
        self.Gep = np.zeros(ne * ne * np_ * np_)
        L.orc_gam_ep(h.ref, O.ptr(self.Gep))
        self.G1, self.G1s = np.zeros(ne * ne * np_ * np_), np.zeros(ne * ne * np_ * np_)
        L.orc_gam1(h.ref, O.ptr(self.G1), O.ptr(self.G1s))
        self.Gee = np.zeros(ne ** 4)
        L.orc_calc_gam_ee(h.ref, O.ptr(self.Gee))
        self.G2, self.G2s = np.zeros(s.ng2), np.zeros(s.ng2)
        self.G3 = np.zeros(s.ng3) if s.nelec > 2 else None
        if s.nelec > 1:
            L.orc_gam2_ic1(h.ref, O.ptr(self.G2), O.ptr(self.G2s))
        if s.nelec > 2:
            L.orc_gam3_ic1(h.ref, O.ptr(self.G3))
        self.E_nuc = float(L.orc_nuc_rep(h.ref))

    # pack_2D(n, j, i) = j + n (i-1): C-order [i][j]
    def ecore(self):
        n = self.s.nebf
        return self.Gecore.reshape(n, n)

    def pcore(self):
        n = self.s.npbf
        return self.Gpcore.reshape(n, n)

    def S_e(self):
        n = self.s.nebf
        return self.Se.reshape(n, n)

    def S_p(self):
        n = self.s.npbf
        return self.Sp.reshape(n, n)


def xchf1_fock(ints: XchfIntegrals, DE, DP):
    """xchf1_fock.f:2-361 with in-core gam_2/gam_3 and direct gam_4."""
    s = ints.s
    ne, np_ = s.nebf, s.npbf
    L = O.lib()
    # E_from_GAM_ecore / pcore: the Fock matrices start as the core matrices
    focke = ints.ecore().copy()
    fockp = ints.pcore().copy()
    E_ecore = float((DE * focke).sum())
    E_pcore = float((DP * fockp).sum())
    # E_from_GAM_ep: GAM_ep[ip][jp][ie][je]
    gep = ints.Gep.reshape(np_, np_, ne, ne)
    focke = focke + np.einsum("pq,pqij->ij", DP, gep)
    fockp = fockp + np.einsum("ij,pqij->pq", DE, gep)
    E_ep = float(np.einsum("ij,pq,pqij->", DE, DP, gep))
    # E_from_GAM_ee: val = (J - K/2)/2 with J = (ie1 je1|ie2 je2), K = (ie1 je2|ie2 je1)
    E_ee = 0.0
    if s.nelec > 1:
        g = ints.Gee.reshape(ne, ne, ne, ne)
        val = 0.5 * (g - 0.5 * g.transpose(0, 3, 2, 1))
        focke = focke + 2.0 * np.einsum("kl,ijkl->ij", DE, val)
        E_ee = float(np.einsum("ij,kl,ijkl->", DE, DE, val))
    # S_from_GAM_1s, E_from_GAM_1: same layout as GAM_ep
    g1 = ints.G1.reshape(np_, np_, ne, ne)
    g1s = ints.G1s.reshape(np_, np_, ne, ne)
    se1 = np.einsum("pq,pqij->ij", DP, g1s)
    sp1 = np.einsum("ij,pqij->pq", DE, g1s)
    S_gam1 = float(np.einsum("ij,pq,pqij->", DE, DP, g1s))
    focke = focke + np.einsum("pq,pqij->ij", DP, g1)
    fockp = fockp + np.einsum("ij,pqij->pq", DE, g1)
    E_gam1 = float(np.einsum("ij,pq,pqij->", DE, DP, g1))
    E_gam2 = E_gam3 = E_gam4 = S_gam2 = 0.0
    se2 = np.zeros((ne, ne))
    sp2 = np.zeros((np_, np_))
    fe, fp = _f(focke), _f(fockp)
    de, dp = _f(DE), _f(DP)
    if s.nelec > 1:
        SE, SP, E, S = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1), np.zeros(1)
        L.orc_eg2ic1(ne, np_, O.ptr(de), O.ptr(dp), O.ptr(ints.G2), O.ptr(ints.G2s),
                     O.ptr(fe), O.ptr(SE), O.ptr(fp), O.ptr(SP), O.ptr(E), O.ptr(S))
        se2, sp2 = _m(SE, ne), _m(SP, np_)
        E_gam2, S_gam2 = float(E[0]), float(S[0])
        if s.nelec > 2:
            E = np.zeros(1)
            L.orc_eg3ic1(ne, np_, O.ptr(de), O.ptr(dp), O.ptr(ints.G3), O.ptr(fe),
                         O.ptr(fp), O.ptr(E))
            E_gam3 = float(E[0])
            E = np.zeros(1)
            L.orc_gam4_dscf(ne, np_, O.ptr(ints.Gee), O.ptr(ints.G2s), O.ptr(de),
                            O.ptr(dp), O.ptr(fe), O.ptr(fp), O.ptr(E))
            E_gam4 = float(E[0])
    S_total = 1.0 + S_gam1 + S_gam2
    psiHpsi = (E_ecore + E_pcore + E_ep + E_ee + E_gam1 + E_gam2 + E_gam3 + E_gam4) / S_total
    E_total = psiHpsi + ints.E_nuc
    H_expect = psiHpsi / S_total
    L.orc_xcfock_correction(ne, np_, S_total, H_expect, O.ptr(_f(se1)), O.ptr(_f(sp1)),
                            O.ptr(_f(se2)), O.ptr(_f(sp2)), O.ptr(fe), O.ptr(fp))
    return {"focke": _m(fe, ne), "fockp": _m(fp, np_), "E_total": E_total,
            "E_nuc": ints.E_nuc, "E_ecore": E_ecore, "E_pcore": E_pcore, "E_ep": E_ep,
            "E_ee": E_ee, "E_gam1": E_gam1, "E_gam2": E_gam2, "E_gam3": E_gam3,
            "E_gam4": E_gam4, "S_total": S_total, "S_gam1": S_gam1, "S_gam2": S_gam2}


def roothan(F, S, nocc, prefac, first=0):
    """xcscf.f:766-953 ROOTHAN: symmetric orthogonalisation X = S^-1/2,
    diagonalise X F X, density prefac sum_k C_k C_k^T over the orbitals
    first..first+nocc-1 (eigenvalues ascending)."""
    w, U = np.linalg.eigh(S)
    X = U @ np.diag(1.0 / np.sqrt(w)) @ U.T
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    C = X @ Cp
    occ = C[:, first:first + nocc]
    return prefac * occ @ occ.T, C, e


def xchf_scf(ints: XchfIntegrals, DE, DP=None, nucst=1, maxit=100, tole=1.0e-6,
             tolp=1.0e-4, orbitals=None):
    """xcscf.f:2-658 (plain Roothaan): returns (history, last Fock result, DE, DP).
    With a list as `orbitals`, each iteration appends (it, EE, EP, CE, CP):
    ROOTHAN's eigenvalues and MO coefficients of that iteration."""
    s = ints.s
    noccE, prefE = (s.nelec // 2, 2.0) if s.nelec > 1 else (1, 1.0)
    if DP is None:   # guess_prot: diagonalise the nuclear core Hamiltonian
        DP, _, _ = roothan(ints.pcore(), ints.S_p(), 1, 1.0, nucst - 1)
    DE0 = np.zeros_like(DE)
    DP0 = np.zeros_like(DP)
    hist = []
    r = None
    for it in range(1, maxit + 1):
        r = xchf1_fock(ints, DE, DP)
        if it == 1:
            hist.append(("initial", dict(r)))
        DP, CP, eP = roothan(r["fockp"], ints.S_p(), 1, 1.0, nucst - 1)
        r = xchf1_fock(ints, DE, DP)
        DE, CE, eE = roothan(r["focke"], ints.S_e(), noccE, prefE, 0)
        if orbitals is not None:
            orbitals.append((it, eE, eP, CE, CP))
        diffE = float(np.abs(DE0 - DE).max())
        diffP = float(np.abs(DP0 - DP).max())
        DE0, DP0 = DE.copy(), DP.copy()
        hist.append((it, r["E_total"], diffE, diffP))
        done = (diffE < tole and diffP < tolp) if s.npbf > 1 else diffE < tole
        if done:
            return hist, r, DE, DP, True
    return hist, r, DE, DP, False
