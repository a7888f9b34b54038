"""ORACLE (test infrastructure only): the XCUHF (open-shell XC-NEO) energy
expression of NEO-RXCHF restated in numpy over the C oracle.

Follows xcuhf/xcuhf_fock.f:2-427 UHF_FOCK with IC_construct_FAE / FP
(:782-1041), the HF terms of xcuhf/xcuhf_hfterms.f (FAE_ecore, FP_pcore,
FAE_GAMep, FP_GAMep, FAE_GAMee), the core-Hamiltonian guesses guess_A_elec
/ guess_prot2 (xcuhf/xcuhf_scf.f:585-640, UROOTHAN :642) and the spin
contractions of ``spin.c``.  The in-core integral tensors may come from
elsewhere (the tests pass device-built GM2ICR / GM3ICR for large cases);
the one-body terms, GAM_1 and GAM_ee come from the C oracle.  Only the
tests load this module.
"""
from __future__ import annotations

import numpy as np

try:   # imported as part of the oracle directory package
    from . import oracle as O
    from .xchf_scf import roothan
except ImportError:   # imported with the oracle directory on sys.path (tests)
    import oracle as O
    from xchf_scf import roothan


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


class XcuhfIntegrals:
    """One-body integrals, GAM_ep, GAM_1/GAM_1s and GAM_ee from the C oracle;
    GM2ICR / GM2sICR / GM3ICR given or built by the oracle; the OMG4 terms
    are evaluated from GAM_2s and GAM_ee on the fly (orc_*_omg4_direct)."""

    def __init__(self, s, G2=None, G2s=None, G3=None):
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
        if G2 is None and s.nelec > 1:
            G2, G2s = np.zeros(s.ng2), np.zeros(s.ng2)
            L.orc_gam2_ic1(h.ref, O.ptr(G2), O.ptr(G2s))
        if G3 is None and s.nelec > 2:
            G3 = np.zeros(s.ng3)
            L.orc_gam3_ic1(h.ref, O.ptr(G3))
        self.G2, self.G2s, self.G3 = G2, G2s, G3
        self.E_nuc = float(L.orc_nuc_rep(h.ref))

    def ecore(self):
        n = self.s.nebf
        return self.Gecore.reshape(n, n)   # pack_2D(n, j, i): [i][j]

    def pcore(self):
        n = self.s.npbf
        return self.Gpcore.reshape(n, n)

    def S_e(self):
        n = self.s.nebf
        return self.Se.reshape(n, n)

    def S_p(self):
        n = self.s.npbf
        return self.Sp.reshape(n, n)


def guess(ints: XcuhfIntegrals, nae: int, nbe: int, nucst: int = 1):
    """guess_A_elec for alpha and beta (lowest NAE / NBE core-Hamiltonian
    orbitals, prefac 1) and guess_prot2 (orbital NUCST of the nuclear core
    Hamiltonian)."""
    DAE, _, _ = roothan(ints.ecore(), ints.S_e(), nae, 1.0, 0)
    DBE, _, _ = roothan(ints.ecore(), ints.S_e(), nbe, 1.0, 0)
    DP, _, _ = roothan(ints.pcore(), ints.S_p(), 1, 1.0, nucst - 1)
    return DAE, DBE, DP


def uhf_energetics(ints: XcuhfIntegrals, nae: int, nbe: int, DAE, DBE, DP) -> dict:
    """UHF_FOCK energy components (the 'NEOXCHF ENERGETIC COMPONENTS'
    block of an XCUHF log): every term divided by S_total, as printed."""
    s = ints.s
    L = O.lib()
    ne, np_ = s.nebf, s.npbf
    DETOT = DAE + DBE
    da, db, dt, dp = _f(DAE), _f(DBE), _f(DETOT), _f(DP)
    ecore, pcore = ints.ecore(), ints.pcore()
    E_ecore = float((DAE * ecore).sum() + (DBE * ecore).sum())
    E_pcore = float((DP * pcore).sum())
    gep = ints.Gep.reshape(np_, np_, ne, ne)
    E_ep = float(np.einsum("ij,pq,pqij->", DETOT, DP, gep))
    # FAE_GAMee: 1/2 sum D(1) [DETOT(2) (11|22) - D(2) (12|21)] per spin
    g = ints.Gee.reshape(ne, ne, ne, ne)
    E_ee = 0.0
    for D in (DAE, DBE):
        E_ee += 0.5 * float(np.einsum("ij,kl,ijkl->", D, DETOT, g) -
                            np.einsum("ij,kl,ilkj->", D, D, g))
    r = {}
    F, S = np.zeros(np_ * np_), np.zeros(np_ * np_)
    E, Sv = np.zeros(1), np.zeros(1)
    L.orc_ufp_omg1(ne, np_, O.ptr(dt), O.ptr(dp), O.ptr(ints.G1), O.ptr(ints.G1s), O.ptr(F),
                   O.ptr(S), O.ptr(E), O.ptr(Sv))
    r["E_P_OMG1"], r["S_P_OMG1"] = float(E[0]), float(Sv[0])
    r["E_P_OMG2"] = r["S_P_OMG2"] = r["E_P_OMG3"] = r["E_P_OMG4"] = 0.0
    if s.nelec > 1:
        L.orc_ufp_omg2(ne, np_, nae, nbe, O.ptr(da), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                       O.ptr(ints.G2s), O.ptr(F), O.ptr(S), O.ptr(E), O.ptr(Sv))
        r["E_P_OMG2"], r["S_P_OMG2"] = float(E[0]), float(Sv[0])
    if s.nelec > 2:
        L.orc_ufp_omg3(ne, np_, nae, nbe, O.ptr(da), O.ptr(db), O.ptr(dp), O.ptr(ints.G3),
                       O.ptr(F), O.ptr(E))
        r["E_P_OMG3"] = float(E[0])
    if s.nelec > 3:
        g2s = _f(ints.G2s)
        L.orc_ufp_omg4_direct(ne, np_, nae, nbe, O.ptr(da), O.ptr(db), O.ptr(dp),
                              O.ptr(g2s), O.ptr(ints.Gee), O.ptr(F), O.ptr(E))
        r["E_P_OMG4"] = float(E[0])
    S_total = 1.0 + r["S_P_OMG1"] + r["S_P_OMG2"]
    out = {"E_NUC": ints.E_nuc, "E_ECORE": E_ecore / S_total, "E_PCORE": E_pcore / S_total,
           "E_EP": E_ep / S_total, "E_EE": E_ee / S_total,
           "E_OMG1": r["E_P_OMG1"] / S_total, "E_OMG2": r["E_P_OMG2"] / S_total,
           "E_OMG3": r["E_P_OMG3"] / S_total, "E_OMG4": r["E_P_OMG4"] / S_total,
           "S_TOTAL": S_total}
    out["E_TOTAL"] = sum(out[k] for k in ("E_NUC", "E_ECORE", "E_PCORE", "E_EP", "E_EE",
                                          "E_OMG1", "E_OMG2", "E_OMG3", "E_OMG4"))
    return out
