"""Pin the CPU oracle to the reference's own known answers.

* CS_Integrals/Spot_Check/TEST_G{2,3,4}/out: single-primitive MD values
  (mapping of gamma1/gamma2 to each term: DRIVER_G3.f:12-445,
  DRIVER_G4.f:13-60, DRIVER_G2.f:11-40; Coulomb terms carry coul_sign*Z).
* examples/xchf/answer/XCHF.log: E_GAM2, E_GAM3, E_GAM4 of one Fock build
  at the initial guess (XCHF.log:306-321) and at convergence (:335-350).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import fmat


def _prims(O, rows):
    return O.prims([(int(r[0]), int(r[1]), int(r[2]), r[3], r[4], r[5], r[6]) for r in rows])


def _gam(**kw):
    g = np.zeros(6)
    names = ["A12", "A13", "A23", "B12", "B13", "B23"]
    for k, v in kw.items():
        g[names.index(k)] = v
    return g


def test_spot_check_g3(orc, golden_spot):
    O, L = orc, orc.lib()
    t = golden_spot["TEST_G3"]
    inp, md = t["input"], t["md"]
    A, B = _prims(O, inp["bra"]), _prims(O, inp["ket"])
    g1, g2 = inp["gamma1"], inp["gamma2"]
    Cm, Z = np.array(inp["C"]), inp["Z"]
    A312, B312 = O.prims([A[2], A[0], A[1]]), O.prims([B[2], B[0], B[1]])
    A132, B132 = O.prims([A[0], A[2], A[1]]), O.prims([B[0], B[2], B[1]])
    p = O.ptr
    got = {
        "xgSg": L.orc_g3_xggs(A, B, p(_gam(A13=g1, B23=g2))),
        "xgTE": L.orc_g3_ke(A, B, p(_gam(A23=g1)), 1.0),
        "xgTEg1": L.orc_g3_ke(A, B, p(_gam(A13=g1, B23=g2)), 1.0),
        "xgTEg3": L.orc_g3_ke(A, B, p(_gam(A23=g1, B23=g2)), 1.0),
        "xgTEg2": L.orc_g3_ke(A, B, p(_gam(A23=g1, B13=g2)), 1.0),
        "xgTPg": L.orc_g3_ke(A312, B312, p(_gam(A12=g1, B13=g2)), 1836.0),
        "xgVEC": -Z * L.orc_g3_xgvxcg(A, B, p(_gam(A23=g1)), p(Cm)),
        "xgVPCg": Z * L.orc_g3_xgvxcg(A312, B312, p(_gam(A12=g1, B13=g2)), p(Cm)),
        "xgVECg1": -Z * L.orc_g3_xgvxcg(A, B, p(_gam(A13=g1, B23=g2)), p(Cm)),
        "xgVECg2": -Z * L.orc_g3_xgvxcg(A, B, p(_gam(A23=g1, B23=g2)), p(Cm)),
        "xgVEP": -L.orc_g3_xgveeg(A132, B132, p(_gam(A23=g1))),
        "xgVEE": L.orc_g3_xgveeg(A, B, p(_gam(A23=g1))),
        "xgVEEg2": L.orc_g3_xgveeg(A, B, p(_gam(A13=g1, B23=g2))),
        "xgVEEg1": L.orc_g3_xgveeg(A, B, p(_gam(A13=g1, B13=g2))),
        "xgVEPg1": -L.orc_g3_xgveeg(A132, B132, p(_gam(A12=g1, B23=g2))),
        "xgVEPg2": -L.orc_g3_xgveeg(A132, B132, p(_gam(A23=g1, B23=g2))),
    }
    assert set(got) == set(md)
    for k, v in md.items():
        # `out` prints 15 significant digits
        assert got[k] == pytest.approx(v, rel=1e-12), k


def test_spot_check_g4(orc, golden_spot):
    O, L = orc, orc.lib()
    t = golden_spot["TEST_G4"]
    inp, md = t["input"], t["md"]
    A, B = _prims(O, inp["bra"]), _prims(O, inp["ket"])
    g1, g2 = inp["gamma1"], inp["gamma2"]
    assert L.orc_g4_xgveeg(A, B, g1, g2) == pytest.approx(md["xgVEEg2"], rel=1e-12)
    assert -L.orc_g4_xgvepg(A, B, g1, g2) == pytest.approx(md["xgVEPg"], rel=1e-12)


def test_spot_check_g2(orc, golden_spot):
    O, L = orc, orc.lib()
    t = golden_spot["TEST_G2"]
    inp, md = t["input"], t["md"]
    A, B = _prims(O, inp["bra"]), _prims(O, inp["ket"])
    x = L.orc_g2_xggs(C.byref(A[0]), C.byref(A[1]), C.byref(B[0]), C.byref(B[1]),
                      inp["gamma1"], inp["gamma2"])
    assert x == pytest.approx(md["XGGS"], rel=1e-12)


def _energies(O, xchf, T, DE, DP, with_gam3=True):
    s = xchf["sys"]
    L = O.lib()
    ne, np_ = s.nebf, s.npbf
    de, dp = fmat(DE), fmat(DP)
    FE, SE, FP, SP = (np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(np_ * np_),
                      np.zeros(np_ * np_))
    E2, S2 = np.zeros(1), np.zeros(1)
    L.orc_eg2ic1(ne, np_, O.ptr(de), O.ptr(dp), O.ptr(T.get("g2")), O.ptr(T.get("g2s")),
                 O.ptr(FE), O.ptr(SE), O.ptr(FP), O.ptr(SP), O.ptr(E2), O.ptr(S2))
    fe, fp, E4 = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    L.orc_gam4_dscf(ne, np_, O.ptr(T.get("gee")), O.ptr(T.get("g2s")), O.ptr(de),
                    O.ptr(dp), O.ptr(fe), O.ptr(fp), O.ptr(E4))
    out = {"E_GAM2": E2[0], "E_GAM4": E4[0]}
    if with_gam3:
        E3 = np.zeros(1)
        L.orc_eg3ic1(ne, np_, O.ptr(de), O.ptr(dp), O.ptr(T.get("g3")), O.ptr(fe),
                     O.ptr(fp), O.ptr(E3))
        out["E_GAM3"] = E3[0]
    return out


def test_xchf_initial_guess_energetics(orc, xchf, xchf_tensors, golden_xchf):
    """One Fock build at the guessCE density reproduces XCHF.log:313-315 to
    the 10 printed decimals."""
    e = _energies(orc, xchf, xchf_tensors, xchf["DE0"], xchf["DP0"])
    ref = golden_xchf["initial"]
    for k in ("E_GAM2", "E_GAM3", "E_GAM4"):
        assert abs(e[k] - ref[k]) <= 6e-11, (k, e[k], ref[k])


def test_xchf_converged_energetics(orc, xchf, xchf_tensors, golden_xchf):
    """At the converged MOs (FinalCE.dat / FinalCP.dat, 8 printed digits) the
    components match XCHF.log:345-347 to the precision of those MOs."""
    e = _energies(orc, xchf, xchf_tensors, xchf["DEf"], xchf["DPf"])
    ref = golden_xchf["final"]
    for k in ("E_GAM2", "E_GAM3", "E_GAM4"):
        assert e[k] == pytest.approx(ref[k], rel=2e-7), (k, e[k], ref[k])


def test_direct_restatement_matches_in_core(orc):
    """The oracle's direct-SCF loops (gam2_DSCF_OMP.f, gam3_DSCF_OMP.f), which
    evaluate every particle ordering of every tuple, agree with its in-core
    pipeline (GAM2_IC1/GAM3_IC1 tensors contracted by EG2IC1/EG3IC1)."""
    from neoxc import basis
    s = basis.synthetic(seed=113, nat=2, nebf=2, nprim=1, npbf=2, ngtg=2, lmax_e=1, lmax_p=1)
    ne, np_ = s.nebf, s.npbf
    L, h = orc.lib(), orc.SystemHandle(s)
    DE = fmat(basis.random_density(ne, 2, 113, 2.0))
    DP = fmat(basis.random_density(np_, 1, 114, 1.0))
    g2, g2s, g3 = np.zeros(s.ng2), np.zeros(s.ng2), np.zeros(s.ng3)
    L.orc_gam2_ic1(h.ref, orc.ptr(g2), orc.ptr(g2s))
    L.orc_gam3_ic1(h.ref, orc.ptr(g3))
    m = lambda n: np.zeros(n * n)  # noqa: E731
    ic2 = [m(ne), m(ne), m(np_), m(np_), np.zeros(1), np.zeros(1)]
    L.orc_eg2ic1(ne, np_, orc.ptr(DE), orc.ptr(DP), orc.ptr(g2), orc.ptr(g2s),
                 *[orc.ptr(x) for x in ic2])
    d2 = [m(ne), m(np_), m(ne), m(np_), np.zeros(1), np.zeros(1)]
    L.orc_gam2_dscf(h.ref, orc.ptr(DE), orc.ptr(DP), *[orc.ptr(x) for x in d2])
    # EG2IC1 order: FE, SE, FP, SP, E, S; GAM2_DSCF order: focke, fockp, se2, sp2, E, S
    for a, b in zip(d2, [ic2[0], ic2[2], ic2[1], ic2[3], ic2[4], ic2[5]]):
        assert np.allclose(a, b, rtol=1e-11, atol=1e-14 * max(1.0, np.abs(b).max()))
    ic3 = [m(ne), m(np_), np.zeros(1)]
    L.orc_eg3ic1(ne, np_, orc.ptr(DE), orc.ptr(DP), orc.ptr(g3), *[orc.ptr(x) for x in ic3])
    d3 = [m(ne), m(np_), np.zeros(1)]
    L.orc_gam3_dscf(h.ref, orc.ptr(DE), orc.ptr(DP), *[orc.ptr(x) for x in d3])
    for a, b in zip(d3, ic3):
        assert np.allclose(a, b, rtol=1e-11, atol=1e-14 * max(1.0, np.abs(b).max()))
    assert abs(d2[4][0]) > 1e-3 and abs(d3[2][0]) > 1e-6


def test_xchf_scf_oracle_pinned(xchf, golden_xchf):
    """The oracle's XCHF SCF (xcscf.f plain Roothaan over its own integrals:
    overlaps, core Hamiltonians, GAM_ep, GAM_1/GAM_1s, GAM_ee, gam_2, gam_3,
    gam_4) reproduces examples/xchf: every initial-guess component of
    XCHF.log:306-321 to the printed 10 decimals, and the converged total
    energy of XCHF.log:335 (the reference converged with SOSCF; the plain
    Roothaan sequence reaches the same stationary point).  The orbital
    energies printed at XCHF.log:353-384: the electronic ones are those of
    the first ROOTHAN diagonalisation (from the second iteration on, SOSCF
    rotates the orbitals without diagonalising, xcscf.f:463-484, so EE is
    never refreshed), the nuclear one is the last iteration's."""
    import xchf_scf as X
    s = xchf["sys"]
    ints = X.XchfIntegrals(s)
    orb = []
    hist, r, DE, DP, ok = X.xchf_scf(ints, xchf["DE0"], orbitals=orb)
    init = hist[0][1]
    ref = golden_xchf["initial"]
    for k in ("E_NUC", "E_ECORE", "E_PCORE", "E_EP", "E_EE", "E_GAM1", "E_GAM2", "E_GAM3",
              "E_GAM4", "S_TOTAL", "E_TOTAL"):
        mine = {"E_NUC": "E_nuc", "E_ECORE": "E_ecore", "E_PCORE": "E_pcore", "E_EP": "E_ep",
                "E_EE": "E_ee", "E_GAM1": "E_gam1", "E_GAM2": "E_gam2", "E_GAM3": "E_gam3",
                "E_GAM4": "E_gam4", "S_TOTAL": "S_total", "E_TOTAL": "E_total"}[k]
        assert abs(init[mine] - ref[k]) <= 6e-11, (k, init[mine], ref[k])
    assert ok
    # iteration 2 precedes the reference's first SOSCF step: same number
    assert abs(hist[2][1] - (-5.7737887409)) <= 6e-11
    fin = golden_xchf["final"]
    assert abs(r["E_total"] - fin["E_TOTAL"]) <= 1e-9
    for k, mine in (("E_ECORE", "E_ecore"), ("E_EP", "E_ep"), ("E_GAM1", "E_gam1"),
                    ("E_GAM2", "E_gam2"), ("S_TOTAL", "S_total")):
        assert abs(r[mine] - fin[k]) <= 1e-5 * max(1.0, abs(fin[k])), k
    eig = golden_xchf["orbital_energies"]
    assert np.abs(orb[0][1] - eig["electronic"]).max() <= 5.001e-5
    assert np.abs(orb[-1][2] - eig["nuclear"]).max() <= 5.001e-5
