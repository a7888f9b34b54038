"""ORACLE (test infrastructure only): the one-special-electron RXCHF Fock
build and SCF of NEO-RXCHF restated in numpy over the C oracle's integrals,
for the two variants whose gam_2 is RXCHFne_GAM2_IC1's:

* RXCHF-ne, closed-shell regular electrons: rxchfne/rxchfne_fock.f:2-250
  RXCHFne_FOCK (RXCHFne_IC_construct_FAE/FP/FBE, RXCHFne_Fock_correction1/2),
  rxchfne/rxchfne_hfterms.f:2-50 RXCHFne_FAE_GAMee;
* RXCUHF-ne / RXCUHF-ae (EXCHLEV 0 / 1), open-shell regular electrons:
  rxchfne/rxcuhfne_fock.f RXCUHFne_FOCK with xcuhf/xcuhf_hfterms.f FAE_ecore
  and FAE_GAMee, LADDEXCH = (EXCHLEV == 1) selecting the RXCUHFne_*_OMG2
  exchange routines.

GAM_1 / GAM_1s come from rxchf/rxchf_gam_1_OMP.f RXCHF_GAM1_OMP_MD (the
geminal-pair terms only).  Initial guesses: rxchf/rxchf_scf.f:785-844
RXCHF_guess_elec, rxchf/rxcuhf_scf.f:863-934 RXCUHF_guess_elec,
xcuhf/xcuhf_scf.f:611-640 guess_prot2.  The SCF follows the LOCBSE2 branch
of rxchfne/rxchfne_scf.f and rxcuhfne_scf.f (proton UROOTHAN per
iteration, then micro-iterations of regular-electron UROOTHAN and
RXCHF_OCBSE2 / RXCUHF_OCBSE2 for the special electron, rxchf/rxchf_scf.f:
1124-1330) without the second-order SCF steps (SOSCF only changes the path
to the converged densities).  Matrices are numpy arrays indexed
[i, j] = F(i, j); the C oracle takes them column-major.  Only the tests load
this module.
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


def _m(v, n):
    return np.asarray(v).reshape(n, n, order="F")


class RxIntegrals:
    """Tables of one RXCHF-ne / RXCUHF-ne(ae) run from the C oracle."""

    def __init__(self, s, G2=None, G2ex=None):
        self.s = s
        L, h = O.lib(), O.SystemHandle(s)
        self.h = h
        ne, np_ = s.nebf, s.npbf
        self.Se, self.Sp = np.zeros(ne * ne), np.zeros(np_ * np_)
        L.orc_overlaps(h.ref, O.ptr(self.Se), O.ptr(self.Sp))
        self.Gecore, self.Gpcore = np.zeros(ne * ne), np.zeros(np_ * np_)
        L.orc_gam_epcore(h.ref, O.ptr(self.Gecore), O.ptr(self.Gpcore))
        self.G1, self.G1s = np.zeros(ne * ne * np_ * np_), np.zeros(ne * ne * np_ * np_)
        L.orc_rxchf_gam1(h.ref, O.ptr(self.G1), O.ptr(self.G1s))
        self.Gee = np.zeros(ne ** 4)
        L.orc_calc_gam_ee(h.ref, O.ptr(self.Gee))
        if G2 is None:
            G2, G2ex = np.zeros(s.ng2), np.zeros(s.ng2)
            L.orc_rxchfne_gam2_ic1(h.ref, O.ptr(G2), O.ptr(G2ex))
        self.G2, self.G2ex = G2, G2ex
        self.E_nuc = float(L.orc_nuc_rep(h.ref))

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


def _omg1(ints, DBE, DP):
    """RXCHF_FP_OMG1 / RXCHF_FBE_OMG1 (rxchf/rxchf_omg1.f:2-165): UFP_OMG1 /
    FAE_OMG1 of xcuhf_omg1.f with the special electron's density."""
    s, L = ints.s, O.lib()
    ne, np_ = s.nebf, s.npbf
    db, dp = _f(DBE), _f(DP)
    XFP, XSP, E, S = np.zeros(np_ * np_), np.zeros(np_ * np_), np.zeros(1), np.zeros(1)
    L.orc_ufp_omg1(ne, np_, O.ptr(db), O.ptr(dp), O.ptr(ints.G1), O.ptr(ints.G1s),
                   O.ptr(XFP), O.ptr(XSP), O.ptr(E), O.ptr(S))
    XFB, XSB, Eb, Sb = np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(1), np.zeros(1)
    L.orc_fae_omg1(ne, np_, O.ptr(db), O.ptr(dp), O.ptr(ints.G1), O.ptr(ints.G1s),
                   O.ptr(XFB), O.ptr(XSB), O.ptr(Eb), O.ptr(Sb))
    return (_m(XFP, np_), _m(XSP, np_), float(E[0]), float(S[0]),
            _m(XFB, ne), _m(XSB, ne), float(Eb[0]), float(Sb[0]))


def _gee(ints):
    n = ints.s.nebf
    return ints.Gee.reshape(n, n, n, n)


def _corrections(ints, XFP, XSP, XFB, XSB, E_P1, E_P2, S_total):
    """RXCHFne_Fock_correction2 (rxchfne_fock.f) for the proton and the
    special electron."""
    psi = E_P1 + E_P2
    c1, c2 = 1.0 / S_total, psi / (S_total * S_total)
    return c1 * XFP - c2 * XSP, c1 * XFB - c2 * XSB


def rxchfne_fock(ints: RxIntegrals, NAE, DAE, DBE, DP) -> dict:
    """RXCHFne_FOCK: FAE, FP, FBE and the printed energy components
    (E_total without E_nuc, as the routine returns it)."""
    s, L = ints.s, O.lib()
    ne, np_ = s.nebf, s.npbf
    ecore = ints.ecore()
    XFAE1 = ecore.copy()                      # FAE_ecore
    E_ecore = float((DAE * ecore).sum())
    E_ee = 0.0
    if NAE > 1:                               # RXCHFne_FAE_GAMee
        g = _gee(ints)
        val = g - 0.5 * g.transpose(0, 3, 2, 1)
        XFAE1 = XFAE1 + np.einsum("kl,ijkl->ij", DAE, val)
        E_ee = 0.5 * float(np.einsum("ij,kl,ijkl->", DAE, DAE, val))
    da, db, dp = _f(DAE), _f(DBE), _f(DP)
    XFAE2, E2a = np.zeros(ne * ne), np.zeros(1)
    L.orc_rxchfne_fae_omg2(ne, np_, O.ptr(da), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                           O.ptr(XFAE2), O.ptr(E2a))
    XFP, XSP, E_P1, S_P1, XFB, XSB, E_B1, S_B1 = _omg1(ints, DBE, DP)
    fp2, E_P2 = np.zeros(np_ * np_), np.zeros(1)
    L.orc_rxchfne_fp_omg2(ne, np_, O.ptr(da), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                          O.ptr(fp2), O.ptr(E_P2))
    fb2, E_B2 = np.zeros(ne * ne), np.zeros(1)
    L.orc_rxchfne_fbe_omg2(ne, np_, O.ptr(da), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                           O.ptr(fb2), O.ptr(E_B2))
    XFP = XFP + _m(fp2, np_)
    XFB = XFB + _m(fb2, ne)
    return _assemble(XFAE1, [_m(XFAE2, ne)], XFP, XSP, XFB, XSB, E_ecore, E_ee,
                     E_P1, float(E_P2[0]), S_P1, float(E2a[0]), E_B1, float(E_B2[0]))


def _assemble(XF1, XF2s, XFP, XSP, XFB, XSB, E_ecore, E_ee, E_P1, E_P2, S_P1,
              E_AE2, E_B1, E_B2, XF1b=None):
    S_total = S_P1
    FP, FBE = _corrections(None, XFP, XSP, XFB, XSB, E_P1, E_P2, S_total)
    c1 = 1.0 / S_total
    r = {"FAE": XF1 + c1 * XF2s[0], "FP": FP, "FBE": FBE}
    if XF1b is not None:
        r["FAbetE"] = XF1b + c1 * XF2s[1]
    E_OMG1, E_OMG2 = E_P1 / S_total, E_P2 / S_total
    r.update({"E_ecore": E_ecore, "E_ee": E_ee, "E_OMG1": E_OMG1, "E_OMG2": E_OMG2,
              "S_total": S_total, "E_total": E_ecore + E_ee + E_OMG1 + E_OMG2,
              "E_P_OMG1": E_P1, "E_P_OMG2": E_P2, "E_AE_OMG2": E_AE2,
              "E_BE_OMG1": E_B1, "E_BE_OMG2": E_B2})
    return r


def rxcuhfne_fock(ints: RxIntegrals, NAalpE, NAbetE, DAalpE, DAbetE, DBE, DP,
                  addexch: bool) -> dict:
    """RXCUHFne_FOCK (rxchfne/rxcuhfne_fock.f): FAE (alpha), FAbetE, FP, FBE
    and the energy components."""
    s, L = ints.s, O.lib()
    ne, np_ = s.nebf, s.npbf
    DAtot = DAalpE + DAbetE
    ecore = ints.ecore()
    XFa, XFb = ecore.copy(), ecore.copy()     # FAE_ecore per spin
    E_ecore = float((DAalpE * ecore).sum()) + float((DAbetE * ecore).sum())
    E_ee = 0.0
    if NAalpE + NAbetE > 1:                   # FAE_GAMee per spin
        g = _gee(ints)
        Ea = Eb = 0.0
        for D, tag in ((DAalpE, "a"), (DAbetE, "b")):
            x = np.einsum("kl,ijkl->ij", DAtot, g) - np.einsum("kl,ilkj->ij", D, g)
            e = 0.5 * float((D * x).sum())
            if tag == "a":
                XFa, Ea = XFa + x, e
            else:
                XFb, Eb = XFb + x, e
        E_ee = Ea + Eb
    da, dbt, dt, db, dp = _f(DAalpE), _f(DAbetE), _f(DAtot), _f(DBE), _f(DP)
    XFP, XSP, E_P1, S_P1, XFB, XSB, E_B1, S_B1 = _omg1(ints, DBE, DP)
    fa2, fb2 = np.zeros(ne * ne), np.zeros(ne * ne)
    fp2, fbe2 = np.zeros(np_ * np_), np.zeros(ne * ne)
    E2a, E_P2, E_B2 = np.zeros(1), np.zeros(1), np.zeros(1)
    if addexch:
        L.orc_rxcuhfne_fe_omg2(ne, np_, O.ptr(da), O.ptr(dt), O.ptr(db), O.ptr(dp),
                               O.ptr(ints.G2), O.ptr(ints.G2ex), O.ptr(fa2), O.ptr(fb2),
                               O.ptr(E2a))
        L.orc_rxcuhfne_fp_omg2(ne, np_, O.ptr(da), O.ptr(dt), O.ptr(db), O.ptr(dp),
                               O.ptr(ints.G2), O.ptr(ints.G2ex), O.ptr(fp2), O.ptr(E_P2))
        L.orc_rxcuhfne_fbe_omg2(ne, np_, O.ptr(da), O.ptr(dt), O.ptr(db), O.ptr(dp),
                                O.ptr(ints.G2), O.ptr(ints.G2ex), O.ptr(fbe2), O.ptr(E_B2))
    else:
        e1, e2 = np.zeros(1), np.zeros(1)
        L.orc_rxchfne_fae_omg2(ne, np_, O.ptr(da), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                               O.ptr(fa2), O.ptr(e1))
        L.orc_rxchfne_fae_omg2(ne, np_, O.ptr(dbt), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                               O.ptr(fb2), O.ptr(e2))
        E2a[0] = e1[0] + e2[0]
        L.orc_rxchfne_fp_omg2(ne, np_, O.ptr(dt), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                              O.ptr(fp2), O.ptr(E_P2))
        L.orc_rxchfne_fbe_omg2(ne, np_, O.ptr(dt), O.ptr(db), O.ptr(dp), O.ptr(ints.G2),
                               O.ptr(fbe2), O.ptr(E_B2))
    XFP = XFP + _m(fp2, np_)
    XFB = XFB + _m(fbe2, ne)
    return _assemble(XFa, [_m(fa2, ne), _m(fb2, ne)], XFP, XSP, XFB, XSB, E_ecore, E_ee,
                     E_P1, float(E_P2[0]), S_P1, float(E2a[0]), E_B1, float(E_B2[0]),
                     XF1b=XFb)


def uroothan(F, S):
    """xcuhf/xcuhf_scf.f:642 UROOTHAN: MOs (columns) and eigenvalues of
    F C = S C e, ascending, by symmetric orthogonalisation."""
    _, C, e = roothan(F, S, 1, 1.0)
    return C, e


def occ_density(C, nocc, prefac=1.0):
    occ = C[:, :nocc]
    return prefac * occ @ occ.T


def guess(ints: RxIntegrals, nae=None, nalp=None, nbet=None, nucst=1):
    """RXCHF_guess_elec (closed: nae) or RXCUHF_guess_elec (open: nalp, nbet)
    and guess_prot2.  Returns a state dict with densities and MOs."""
    C, _ = uroothan(ints.ecore(), ints.S_e())
    st = {}
    if nae is not None:
        nocca = nae // 2 if nae > 1 else nae
        st["CAE"] = C.copy()
        st["DAE"] = occ_density(C, nocca, 2.0 if nae > 1 else 1.0)
    else:
        nocca = nalp
        st["CAE"] = C.copy()
        st["DAE"] = occ_density(C, nalp)            # RXCUHF_construct_DAE
        st["CAbetE"] = C.copy()                      # RXCUHF_guess_A_elec(NAbetE)
        st["DAbetE"] = occ_density(C, nbet)
    CBE = np.zeros_like(C)
    CBE[:, :C.shape[1] - nocca] = C[:, nocca:]
    st["CBE"] = CBE
    st["DBE"] = occ_density(CBE, 1)
    Cp, _ = uroothan(ints.pcore(), ints.S_p())
    st["DP"] = np.outer(Cp[:, nucst - 1], Cp[:, nucst - 1])
    return st


def ocbse2(ints: RxIntegrals, nocca, CAE, CBE0, FBE):
    """rxchf/rxchf_scf.f:1124-1330 RXCHF_OCBSE2 (and rxcuhf_scf.f:935
    RXCUHF_OCBSE2 with nocca = NAalpE): the special electron's orbital from
    the space orthogonal to the occupied regular orbitals."""
    S = ints.S_e()
    ne = S.shape[0]
    nvirt = ne - nocca - 1
    ov = np.array([float(CAE[:, k] @ S @ CBE0[:, 0]) for k in range(ne)])
    motodiscard, best = 0, 0.0
    for k in range(1, ne):                   # mo1 > 1 in 1-based terms
        if abs(ov[k]) > best:
            best, motodiscard = abs(ov[k]), k
    WB = np.zeros((ne, nvirt + 1))
    for i in range(nvirt):
        col = nocca + i
        WB[:, i] = CAE[:, col] if col != motodiscard else CAE[:, ne - 1]
    proj = CBE0[:, 0].copy()
    for k in range(ne):
        if k != motodiscard:
            proj = proj - ov[k] * CAE[:, k]
    nrm = float(proj @ S @ proj)
    WB[:, nvirt] = proj / np.sqrt(nrm)
    Cx, e = uroothan(WB.T @ FBE @ WB, WB.T @ S @ WB)
    CBE = np.zeros((ne, ne))
    CBE[:, :nvirt + 1] = WB @ Cx
    return CBE, e


def rx_scf(ints: RxIntegrals, nae=None, nalp=None, nbet=None, addexch=False, nucst=1,
           maxit=100, maxmicro=200, tole=1.0e-6, tolp=1.0e-4, ocbse=True):
    """The SCF of rxchfne_scf.f / rxcuhfne_scf.f with UROOTHAN for the
    regular electrons: the LOCBSE2 branch (ocbse=True: OCBSE guess, one Fock
    build per micro-iteration after RXCHF_OCBSE2) or the plain branch
    (ocbse=False: RXCHF_guess_A/B_elec, rxchf_scf.f:733-784, a Fock build at
    the top of every micro-iteration and UROOTHAN for the special electron's
    lowest orbital).  Returns (initial energetics, final energetics, history
    of (iteration, micro-iterations, E_total), converged)."""
    open_shell = nae is None
    st = guess(ints, nae=nae, nalp=nalp, nbet=nbet, nucst=nucst)
    nocca = nalp if open_shell else (nae // 2 if nae > 1 else nae)
    if not ocbse:   # RXCHF_guess_B_elec: the lowest core orbital
        C, _ = uroothan(ints.ecore(), ints.S_e())
        st["CBE"] = C.copy()
        st["DBE"] = occ_density(C, 1)

    def fock():
        if open_shell:
            r = rxcuhfne_fock(ints, nalp, nbet, st["DAE"], st["DAbetE"], st["DBE"], st["DP"],
                              addexch)
        else:
            r = rxchfne_fock(ints, nae, st["DAE"], st["DBE"], st["DP"])
        r["E_total"] = r["E_total"] + ints.E_nuc
        return r

    D0 = {k: np.zeros_like(st[k]) for k in ("DAE", "DBE", "DP")}
    if open_shell:
        D0["DAbetE"] = np.zeros_like(st["DAbetE"])
    hist, initial, r = [], None, None
    for it in range(1, maxit + 1):
        r = fock()
        if it == 1:
            initial = dict(r)
        Cp, _ = uroothan(r["FP"], ints.S_p())
        st["DP"] = np.outer(Cp[:, nucst - 1], Cp[:, nucst - 1])
        diffP = float(np.abs(D0["DP"] - st["DP"]).max())
        D0["DP"] = st["DP"].copy()
        for micro in range(1, maxmicro + 1):
            if micro == 1 or not ocbse:
                r = fock()
            C, _ = uroothan(r["FAE"], ints.S_e())
            st["CAE"] = C
            st["DAE"] = occ_density(C, nocca, 1.0 if open_shell or nae == 1 else 2.0)
            diffA = float(np.abs(D0["DAE"] - st["DAE"]).max())
            D0["DAE"] = st["DAE"].copy()
            if open_shell:
                Cb, _ = uroothan(r["FAbetE"], ints.S_e())
                st["DAbetE"] = occ_density(Cb, nbet)
                diffA = max(diffA, float(np.abs(D0["DAbetE"] - st["DAbetE"]).max()))
                D0["DAbetE"] = st["DAbetE"].copy()
            if ocbse:
                st["CBE"], _ = ocbse2(ints, nocca, st["CAE"], st["CBE"], r["FBE"])
            else:
                st["CBE"], _ = uroothan(r["FBE"], ints.S_e())
            st["DBE"] = occ_density(st["CBE"], 1)
            diffB = float(np.abs(D0["DBE"] - st["DBE"]).max())
            D0["DBE"] = st["DBE"].copy()
            if ocbse:
                r = fock()
            if diffA < tole and diffB < tole:
                break
        hist.append((it, micro, r["E_total"]))
        if diffP < tolp:
            return initial, r, hist, True
    return initial, r, hist, False
