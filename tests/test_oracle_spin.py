"""The oracle's open-shell XCUHF contractions (oracle/spin.c, restating
xcuhf/xcuhf_omg{1..4}.f) pinned against its closed-shell XCHF contractions,
which are themselves pinned to examples/xchf/answer/XCHF.log.

With alpha = beta = D/2 and every spin term switched on (NAE = NBE = 4),
the UHF expressions reduce term by term to the closed-shell ones:
UFP_OMGk's energy equals EG2IC1 / EG3IC1 / EG4ICR's, the alpha Fock matrix
equals the closed-shell electronic Fock matrix, and the proton Fock
matrices agree.  With NAE = NBE = 2 and densities of rank 2 the skipped
three- and four-same-spin terms vanish identically, so the energies and the
proton Fock matrix still agree.  OMG4_ICR's raw elements, recombined with
symm_gam4's 24 coefficients, give GAM4_ICR's elements.  CPU only.
"""
from __future__ import annotations

import numpy as np
import pytest


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


@pytest.fixture(scope="module")
def spin_case(orc):
    from neoxc import basis
    O = orc
    L = O.lib()
    s = basis.synthetic(seed=7, nat=2, nebf=3, nprim=2, npbf=2, ngtg=2, lmax_e=1,
                        lmax_p=1, nelec=8)
    h = O.SystemHandle(s)
    ne, np_ = s.nebf, s.npbf
    G2, G2s = np.zeros(s.ng2), np.zeros(s.ng2)
    L.orc_gam2_ic1(h.ref, O.ptr(G2), O.ptr(G2s))
    G3 = np.zeros(s.ng3)
    L.orc_gam3_ic1(h.ref, O.ptr(G3))
    Gee = np.zeros(ne ** 4)
    L.orc_calc_gam_ee(h.ref, O.ptr(Gee))
    G4s = np.zeros(s.ng4)
    L.orc_gam4_icr(ne, np_, O.ptr(G2s), O.ptr(Gee), O.ptr(G4s))
    G4r = np.zeros(s.ng4)
    L.orc_omg4_icr(ne, np_, O.ptr(G2s), O.ptr(Gee), O.ptr(G4r))
    G1, G1s = np.zeros(ne * ne * np_ * np_), np.zeros(ne * ne * np_ * np_)
    L.orc_gam1(h.ref, O.ptr(G1), O.ptr(G1s))
    return dict(s=s, ne=ne, np=np_, G1=G1, G1s=G1s, G2=G2, G2s=G2s, G3=G3, Gee=Gee,
                G4s=G4s, G4r=G4r)


def _dens(rng, ne, np_, rank):
    if rank is None:
        A = rng.standard_normal((ne, ne))
        D = A @ A.T / ne
    else:
        Cm = rng.standard_normal((ne, rank))
        D = 2.0 * Cm @ Cm.T
    P = rng.standard_normal((np_, np_))
    return D, P @ P.T / np_


def _uhf(orc, c, k, nae, nbe, DA, DB, DP):
    """(FAE, FP, E_AE, E_P, SAE, SP, S_P) of the oracle's FAE_OMGk / UFP_OMGk."""
    L, P = orc.lib(), orc.ptr
    ne, np_ = c["ne"], c["np"]
    da, db, dp = _f(DA), _f(DB), _f(DP)
    fa, fp = np.zeros(ne * ne), np.zeros(np_ * np_)
    sa, sp = np.zeros(ne * ne), np.zeros(np_ * np_)
    ea, ep, s1, s2 = np.zeros(1), np.zeros(1), np.zeros(1), np.zeros(1)
    if k == 2:
        L.orc_fae_omg2(ne, np_, nae, nbe, P(da), P(db), P(dp), P(c["G2"]), P(c["G2s"]),
                       P(fa), P(sa), P(ea), P(s1))
        L.orc_ufp_omg2(ne, np_, nae, nbe, P(da), P(db), P(dp), P(c["G2"]), P(c["G2s"]),
                       P(fp), P(sp), P(ep), P(s2))
    elif k == 3:
        L.orc_fae_omg3(ne, np_, nae, nbe, P(da), P(db), P(dp), P(c["G3"]), P(fa), P(ea))
        L.orc_ufp_omg3(ne, np_, nae, nbe, P(da), P(db), P(dp), P(c["G3"]), P(fp), P(ep))
    else:
        L.orc_fae_omg4(ne, np_, nae, nbe, P(da), P(db), P(dp), P(c["G4r"]), P(fa), P(ea))
        L.orc_ufp_omg4(ne, np_, nae, nbe, P(da), P(db), P(dp), P(c["G4r"]), P(fp), P(ep))
    return fa, fp, ea[0], ep[0], sa, sp, s2[0]


def _xchf(orc, c, k, D, DP):
    """(FE, FP, E, SE, SP, S) of EG2IC1 / EG3IC1 / EG4ICR at DE = D."""
    L, P = orc.lib(), orc.ptr
    ne, np_ = c["ne"], c["np"]
    de, dp = _f(D), _f(DP)
    fe, fp, se, sp = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(ne * ne), np.zeros(np_ * np_)
    E, S = np.zeros(1), np.zeros(1)
    if k == 2:
        L.orc_eg2ic1(ne, np_, P(de), P(dp), P(c["G2"]), P(c["G2s"]), P(fe), P(se), P(fp),
                     P(sp), P(E), P(S))
    elif k == 3:
        L.orc_eg3ic1(ne, np_, P(de), P(dp), P(c["G3"]), P(fe), P(fp), P(E))
    else:
        L.orc_eg4icr(ne, np_, P(de), P(dp), P(c["G4s"]), P(fe), P(fp), P(E))
    return fe, fp, E[0], se, sp, S[0]


@pytest.mark.parametrize("k", [2, 3, 4])
def test_closed_shell_reduction_all_terms(orc, spin_case, k):
    rng = np.random.default_rng(100 + k)
    D, DP = _dens(rng, spin_case["ne"], spin_case["np"], None)
    fa, fp, ea, ep, sa, sp, sP = _uhf(orc, spin_case, k, 4, 4, D / 2, D / 2, DP)
    fe, fpx, E, se, spx, S = _xchf(orc, spin_case, k, D, DP)
    tol = 1e-12 * max(1.0, abs(E))
    assert abs(ep - E) <= tol, (ep, E)
    assert abs(2.0 * ea - E) <= tol
    assert np.abs(fa - fe).max() <= 1e-12 * max(1.0, np.abs(fe).max())
    assert np.abs(fp - fpx).max() <= 1e-12 * max(1.0, np.abs(fpx).max())
    if k == 2:
        # SAE2 carries EFAC = 2 where EG2IC1's SE does not
        assert np.abs(sa - 2.0 * se).max() <= 1e-12 * max(1.0, np.abs(se).max())
        assert np.abs(sp - spx).max() <= 1e-12 * max(1.0, np.abs(spx).max())
        assert abs(sP - S) <= 1e-12 * max(1.0, abs(S))


@pytest.mark.parametrize("k", [2, 3, 4])
def test_closed_shell_reduction_rank_two(orc, spin_case, k):
    rng = np.random.default_rng(200 + k)
    D, DP = _dens(rng, spin_case["ne"], spin_case["np"], 2)
    fa, fp, ea, ep, *_ = _uhf(orc, spin_case, k, 2, 2, D / 2, D / 2, DP)
    fe, fpx, E, *_ = _xchf(orc, spin_case, k, D, DP)
    assert abs(ep - E) <= 1e-11 * max(1.0, abs(E)), (ep, E)
    assert np.abs(fp - fpx).max() <= 1e-11 * max(1.0, np.abs(fpx).max())


@pytest.mark.parametrize("k", [2, 3, 4])
def test_proton_terms_symmetric_in_spin(orc, spin_case, k):
    """UFP_OMGk is unchanged when alpha and beta (densities and counts) are
    exchanged."""
    rng = np.random.default_rng(300 + k)
    DA, DP = _dens(rng, spin_case["ne"], spin_case["np"], None)
    DB, _ = _dens(rng, spin_case["ne"], spin_case["np"], None)
    _, fp1, _, ep1, *_ = _uhf(orc, spin_case, k, 3, 1, DA, DB, DP)
    _, fp2, _, ep2, *_ = _uhf(orc, spin_case, k, 1, 3, DB, DA, DP)
    assert abs(ep1 - ep2) <= 1e-12 * max(1.0, abs(ep1))
    assert np.abs(fp1 - fp2).max() <= 1e-12 * max(1.0, np.abs(fp1).max())


def test_omg4_icr_recombines_to_gam4_icr(orc, spin_case):
    """GAM4_ICR element = 1/16 sum_sigma c_sigma * raw(sigma) (symm_gam4's
    coefficients 16, -8, 4, -2) over OMG4_ICR's raw tensor; and the direct
    OMG4 contractions equal the stored-tensor ones."""
    c = spin_case
    ne, np_ = c["ne"], c["np"]
    L = orc.lib()
    raw = c["G4r"].reshape(np_, np_, ne, ne, ne, ne, ne, ne, ne, ne)
    sym = c["G4s"].reshape(raw.shape)
    rng = np.random.default_rng(5)
    perms = [((0, 1, 2, 3), 16), ((1, 0, 2, 3), -8), ((2, 0, 1, 3), 4), ((0, 2, 1, 3), -8),
             ((1, 2, 0, 3), 4), ((2, 1, 0, 3), -8), ((3, 1, 0, 2), 4), ((1, 3, 0, 2), -2),
             ((0, 3, 1, 2), 4), ((3, 0, 1, 2), -2), ((1, 0, 3, 2), 4), ((0, 1, 3, 2), -8),
             ((0, 2, 3, 1), 4), ((2, 0, 3, 1), -2), ((3, 0, 2, 1), 4), ((0, 3, 2, 1), -8),
             ((2, 3, 0, 1), 4), ((3, 2, 0, 1), -2), ((3, 2, 1, 0), 4), ((2, 3, 1, 0), -2),
             ((1, 3, 2, 0), 4), ((3, 1, 2, 0), -8), ((2, 1, 3, 0), 4), ((1, 2, 3, 0), -2)]
    for _ in range(40):
        ip, jp = rng.integers(np_, size=2)
        i = rng.integers(ne, size=4)
        j = rng.integers(ne, size=4)
        val, big = 0.0, 1.0
        for p, cf in perms:
            k = [j[p[m]] for m in range(4)]
            x = raw[ip, jp, i[0], k[0], i[1], k[1], i[2], k[2], i[3], k[3]]
            val += cf * x
            big = max(big, abs(x))
        ref = sym[ip, jp, i[0], j[0], i[1], j[1], i[2], j[2], i[3], j[3]]
        assert abs(val / 16.0 - ref) <= 1e-13 * big
    D, DP = _dens(rng, ne, np_, None)
    da, dp = _f(D / 2), _f(DP)
    for nae, nbe in ((2, 2), (4, 1), (1, 3)):
        F1, E1, F2, E2 = np.zeros(np_ * np_), np.zeros(1), np.zeros(np_ * np_), np.zeros(1)
        L.orc_ufp_omg4(ne, np_, nae, nbe, orc.ptr(da), orc.ptr(da), orc.ptr(dp),
                       orc.ptr(c["G4r"]), orc.ptr(F1), orc.ptr(E1))
        L.orc_ufp_omg4_direct(ne, np_, nae, nbe, orc.ptr(da), orc.ptr(da), orc.ptr(dp),
                              orc.ptr(c["G2s"]), orc.ptr(c["Gee"]), orc.ptr(F2),
                              orc.ptr(E2))
        assert np.array_equal(F1, F2) and E1[0] == E2[0]


def test_omg1_matches_closed_shell(orc, spin_case):
    """UFP_OMG1 with DETOT is E_from_GAM_1's energy and proton Fock term."""
    c = spin_case
    ne, np_ = c["ne"], c["np"]
    rng = np.random.default_rng(9)
    DA, DP = _dens(rng, ne, np_, None)
    DB, _ = _dens(rng, ne, np_, None)
    DT = DA + DB
    L, P = orc.lib(), orc.ptr
    F, S, E, Sv = np.zeros(np_ * np_), np.zeros(np_ * np_), np.zeros(1), np.zeros(1)
    L.orc_ufp_omg1(ne, np_, P(_f(DT)), P(_f(DP)), P(c["G1"]), P(c["G1s"]), P(F), P(S), P(E),
                   P(Sv))
    g1 = c["G1"].reshape(np_, np_, ne, ne)
    g1s = c["G1s"].reshape(np_, np_, ne, ne)
    assert abs(E[0] - np.einsum("ij,pq,pqij->", DT, DP, g1)) <= 1e-12 * abs(E[0])
    assert abs(Sv[0] - np.einsum("ij,pq,pqij->", DT, DP, g1s)) <= 1e-12 * abs(Sv[0])
    assert np.allclose(F.reshape(np_, np_, order="F"), np.einsum("ij,pqij->pq", DT, g1),
                       rtol=1e-12, atol=0)
    Fa, Sa, Ea, Sva = np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(1), np.zeros(1)
    L.orc_fae_omg1(ne, np_, P(_f(DA)), P(_f(DP)), P(c["G1"]), P(c["G1s"]), P(Fa), P(Sa),
                   P(Ea), P(Sva))
    assert np.allclose(Fa.reshape(ne, ne, order="F"), np.einsum("pq,pqij->ij", DP, g1),
                       rtol=1e-12, atol=0)
    assert abs(Ea[0] - np.einsum("ij,pq,pqij->", DA, DP, g1)) <= 1e-12 * abs(Ea[0])
