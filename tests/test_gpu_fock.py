"""The integral phase of xcneo_driver and the whole XCHF Fock build
(xchf1_fock.f) through the C-ABI: neoxc_onebody_integrals,
neoxc_class_nuc_rep, neoxc_xchf1_fock and the by-reference shims that write
and read the reference's files (elec_ovlap_, nuc_ovlap_, calc_gam_epcore_,
calc_gam_ep_, gam1_omp_md_, class_nuc_rep_, gam2_conv_, gam3_conv_,
e_from_gam_2_, s_from_gam_2s_, e_from_gam_3_, e_from_gam_4_, xchf1_fock_).

Tolerances: one-body tables within 1e-12 of the oracle (relative to the
table's largest element); the first Fock build of examples/xchf within
6e-11 Eh of XCHF.log:306-321 (the log's 10 decimals); Fock matrices within
1e-11 of the oracle's xchf1_fock restatement; the branches of xchf1_fock
(in-core, direct, disk) within 1e-12 of one another, and a disk branch fed
the in-core tables through the files bit-identical to the in-core call.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOG_NAMES = {"E_NUC": "E_nuc", "E_ECORE": "E_ecore", "E_PCORE": "E_pcore", "E_EP": "E_ep",
             "E_EE": "E_ee", "E_GAM1": "E_gam1", "E_GAM2": "E_gam2", "E_GAM3": "E_gam3",
             "E_GAM4": "E_gam4", "S_TOTAL": "S_total", "E_TOTAL": "E_total"}
ENERGIES = ("E_total", "E_ecore", "E_pcore", "E_ep", "E_ee", "E_gam1", "E_gam2", "E_gam3",
            "E_gam4", "S_total", "S_gam1", "S_gam2")


def _rel_close(got, ref, tol, what=""):
    got, ref = np.asarray(got, float).ravel(), np.asarray(ref, float).ravel()
    scale = max(1.0, float(np.abs(ref).max()))
    err = float(np.abs(got - ref).max())
    assert err <= tol * scale, (what, err, scale)


def _i64(v):
    return C.byref(C.c_int64(int(v)))


def _dbl(v):
    return C.byref(C.c_double(float(v)))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.fixture
def in_tmp(tmp_path):
    old = os.getcwd()
    os.chdir(tmp_path)
    yield tmp_path
    os.chdir(old)


@pytest.fixture(scope="module")
def tables(nx, xchf):
    """examples/xchf tables from the device builders."""
    s = xchf["sys"]
    t = dict(nx.onebody_integrals(s))
    t["GAM_ee"] = nx.calc_gam_ee(s)
    t["GM2ICR"], t["GM2SICR"] = nx.gam2_ic1(s)
    t["GM3IC1"] = nx.gam3_ic1(s)
    t["GM4ICR"] = nx.gam4_icr(s.nebf, s.npbf, t["GM2SICR"], t["GAM_ee"])
    t["E_nuc"] = nx.class_nuc_rep(s)
    return t


def _oracle_onebody(orc, s):
    L, h = orc.lib(), orc.SystemHandle(s)
    ne, np_ = s.nebf, s.npbf
    Se, Sp = np.zeros(ne * ne), np.zeros(np_ * np_)
    L.orc_overlaps(h.ref, orc.ptr(Se), orc.ptr(Sp))
    He, Hp = np.zeros(ne * ne), np.zeros(np_ * np_)
    L.orc_gam_epcore(h.ref, orc.ptr(He), orc.ptr(Hp))
    Gep = np.zeros(s.ng1)
    L.orc_gam_ep(h.ref, orc.ptr(Gep))
    G1, G1s = np.zeros(s.ng1), np.zeros(s.ng1)
    L.orc_gam1(h.ref, orc.ptr(G1), orc.ptr(G1s))
    return {"Se": Se, "Sp": Sp, "GAM_ecore": He, "GAM_pcore": Hp, "GAM_ep": Gep,
            "GAM_1": G1, "GAM_1s": G1s, "E_nuc": float(L.orc_nuc_rep(h.ref))}


@pytest.mark.parametrize("case", ["example", "synthetic_d"])
def test_onebody_tables_match_oracle(nx, orc, xchf, case):
    from neoxc import basis
    if case == "example":
        s = xchf["sys"]
    else:
        s = basis.synthetic(seed=411, nat=3, nebf=5, nprim=2, npbf=4, ngtg=2, lmax_e=2,
                            lmax_p=2, nelec=4)
    got = nx.onebody_integrals(s)
    ref = _oracle_onebody(orc, s)
    for k in ("Se", "Sp", "GAM_ecore", "GAM_pcore", "GAM_ep", "GAM_1", "GAM_1s"):
        _rel_close(got[k], ref[k], 1e-12, k)
    assert abs(nx.class_nuc_rep(s) - ref["E_nuc"]) <= 1e-13 * max(1.0, abs(ref["E_nuc"]))


def test_onebody_skips_outputs_not_asked_for(nx, xchf):
    s = xchf["sys"]
    full = nx.onebody_integrals(s)
    part = nx.onebody_integrals(s, which=("Sp", "GAM_ep"))
    assert set(part) == {"Sp", "GAM_ep"}
    assert np.array_equal(part["Sp"], full["Sp"])
    assert np.array_equal(part["GAM_ep"], full["GAM_ep"])


def test_xchf1_fock_first_build_matches_log(nx, xchf, tables, golden_xchf):
    """xchf1_fock at guessCE + the core-Hamiltonian proton guess (in-core
    gam_2 / gam_3, direct gam_4): XCHF.log:306-321."""
    r = nx.xchf1_fock(xchf["sys"], xchf["DE0"], xchf["DP0"], tables, tables["E_nuc"])
    for k, mine in LOG_NAMES.items():
        assert abs(r[mine] - golden_xchf["initial"][k]) <= 6e-11, (k, r[mine])


def test_xchf1_fock_matches_oracle(nx, xchf, tables):
    import xchf_scf as X
    ints = X.XchfIntegrals(xchf["sys"])
    ref = X.xchf1_fock(ints, xchf["DE0"], xchf["DP0"])
    r = nx.xchf1_fock(xchf["sys"], xchf["DE0"], xchf["DP0"], tables, tables["E_nuc"])
    _rel_close(r["focke"], ref["focke"], 1e-11, "focke")
    _rel_close(r["fockp"], ref["fockp"], 1e-11, "fockp")
    for k in ENERGIES:
        assert abs(r[k] - ref[k]) <= 1e-11 * max(1.0, abs(ref[k])), k


@pytest.mark.parametrize("modes", [
    ("gam4", "g4dscf", "g3dscf", "g2dscf"),
    ("gam4", "g4ic", "g3ic1", "g2ic1"),
    ("gam4", "g4dscf", "gam4_factored", "g3ic1", "g2ic1"),
    ("gam4",),                       # disk branches: tables in the IC arguments
])
def test_xchf1_fock_branches_agree(nx, xchf, tables, modes):
    s = xchf["sys"]
    base = nx.xchf1_fock(s, xchf["DEf"], xchf["DPf"], tables, tables["E_nuc"])
    r = nx.xchf1_fock(s, xchf["DEf"], xchf["DPf"], tables, tables["E_nuc"], modes=modes)
    _rel_close(r["focke"], base["focke"], 1e-12, "focke")
    _rel_close(r["fockp"], base["fockp"], 1e-12, "fockp")
    for k in ENERGIES:
        assert abs(r[k] - base[k]) <= 1e-12 * max(1.0, abs(base[k])), k


def test_xchf1_fock_neohf_and_gam4_off(nx, xchf, tables):
    s = xchf["sys"]
    full = nx.xchf1_fock(s, xchf["DE0"], xchf["DP0"], tables, tables["E_nuc"])
    hf = nx.xchf1_fock(s, xchf["DE0"], xchf["DP0"], tables, tables["E_nuc"], modes=("neohf",))
    # xchf1_fock.f:218-235: the NEO-HF part, E_NEOHF, S_total = 1
    assert np.array_equal(hf["focke"], hf["Xfocke"]) and np.array_equal(hf["fockp"], hf["Xfockp"])
    assert np.array_equal(hf["Xfocke"], full["Xfocke"])
    e = hf["E_ecore"] + hf["E_pcore"] + hf["E_ep"] + hf["E_ee"] + tables["E_nuc"]
    assert hf["E_total"] == e and hf["S_total"] == 1.0
    assert hf["E_gam1"] == hf["E_gam2"] == hf["E_gam3"] == hf["E_gam4"] == 0.0
    no4 = nx.xchf1_fock(s, xchf["DE0"], xchf["DP0"], tables, tables["E_nuc"],
                        modes=("g3ic1", "g2ic1"))
    assert no4["E_gam4"] == 0.0
    assert no4["E_gam3"] == full["E_gam3"] and no4["S_total"] == full["S_total"]


def test_xchf1_fock_argument_checks(nx, xchf, tables):
    """A table the selected branch needs is checked before any device work."""
    s = xchf["sys"]
    for missing in ("GM3IC1", "GAM_1", "GAM_ee"):
        t = dict(tables)
        t[missing] = None
        with pytest.raises(nx.NeoxcError):
            nx.xchf1_fock(s, xchf["DE0"], xchf["DP0"], t, tables["E_nuc"])


def _basis_args(s):
    return [_p(a) for a in (s.AMPEB2C_f, s.AGEBFCC_f, s.AGNBFCC_f, s.ELCEX_f, s.NUCEX_f,
                            s.ELCAM_f, s.NUCAM_f, s.ELCBFC_f, s.NUCBFC_f)]


def test_driver_shims_write_the_reference_files(nx, xchf, tables, in_tmp):
    """The integral phase through the by-reference shims: each file holds the
    C entry's table record for record."""
    from neoxc import formats as F
    s, L = xchf["sys"], nx.lib()
    ne, np_ = s.nebf, s.npbf
    b = _basis_args(s)
    L.class_nuc_rep_(_i64(s.nat), _p(s.zan_f), _p(s.cat_f))
    L.elec_ovlap_(_i64(s.npebf), _i64(ne), _i64(ne * ne), b[0], b[1], b[3], b[5], b[7])
    L.nuc_ovlap_(_i64(np_), _i64(np_ * np_), b[2], b[4], b[6], b[8])
    L.calc_gam_epcore_(_i64(ne), _i64(s.npebf), _i64(np_), _i64(ne * ne), _i64(np_ * np_),
                       _i64(s.nat), _dbl(s.pmass), _p(s.zan_f), _p(s.cat_f), *b)
    L.calc_gam_ep_(_i64(ne), _i64(s.npebf), _i64(np_), _i64(s.ng1), *b)
    L.gam1_omp_md_(_i64(ne), _i64(s.npebf), _i64(np_), _i64(s.ng1),
                   _i64(s.npebf ** 2 * np_ ** 2), _i64(s.nat), _i64(s.ngtg), _dbl(s.pmass),
                   _p(s.cat_f), _p(s.zan_f), _p(s.bgem_f), _p(s.ggem_f), *b)
    sysb = [_p(a) for a in (s.cat_f, s.zan_f, s.bgem_f, s.ggem_f, s.KPESTR_f, s.KPEEND_f)] + b
    L.gam2_conv_(_i64(1), _i64(ne), _i64(s.npebf), _i64(np_), _i64(s.ng2), _i64(s.ng2prm),
                 _i64(s.nat), _i64(s.ngtg), _dbl(s.pmass), *sysb)
    L.gam3_conv_(_i64(1), _i64(ne), _i64(s.npebf), _i64(np_), _i64(s.ng3), _i64(s.ng3prm),
                 _i64(s.nat), _i64(s.ngtg), _dbl(s.pmass), *sysb)
    assert F.read_enuc("ENUCRP.dat") == pytest.approx(tables["E_nuc"], rel=1e-15, abs=0)
    files = {"eovlap.ufm": "Se", "novlap.ufm": "Sp", "GAM_ecr.ufm": "GAM_ecore",
             "GAM_pcr.ufm": "GAM_pcore", "GAM_ep.ufm": "GAM_ep", "GAM_1.ufm": "GAM_1",
             "GAM_1s.ufm": "GAM_1s", "GAM_2.ufm": "GM2ICR", "GAM_2s.ufm": "GM2SICR",
             "GAM_3.ufm": "GM3IC1"}
    for f, k in files.items():
        assert np.array_equal(F.read_ufm(f, tables[k].size), tables[k]), f


def test_disk_contractions_and_xchf1_fock_shim(nx, xchf, tables, in_tmp):
    """E_from_GAM_2/3/4, S_from_GAM_2s and xchf1_fock_'s disk branches read
    the files and give the in-core results bit for bit."""
    from neoxc import formats as F
    s, L = xchf["sys"], nx.lib()
    ne, np_ = s.nebf, s.npbf
    for f, k in (("GAM_1.ufm", "GAM_1"), ("GAM_1s.ufm", "GAM_1s"), ("GAM_2.ufm", "GM2ICR"),
                 ("GAM_2s.ufm", "GM2SICR"), ("GAM_3.ufm", "GM3IC1")):
        F.write_ufm(f, tables[k])
    F.write_ufm("GAM_4.ufm", tables["GM4ICR"] * 16.0)
    DE = np.asfortranarray(xchf["DEf"], dtype=np.float64)
    DP = np.asfortranarray(xchf["DPf"], dtype=np.float64)
    # E_from_GAM_2 / S_from_GAM_2s against EG2IC1
    fe, fp, E = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    L.e_from_gam_2_(_i64(ne), _i64(np_), _i64(s.ng2), _p(DE), _p(DP), _p(fe), _p(fp), _p(E))
    se, sp, S = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    L.s_from_gam_2s_(_i64(ne), _i64(np_), _i64(s.ng2), _p(DE), _p(DP), _p(se), _p(sp), _p(S))
    FE, SE, FP, SP, E2, S2 = nx.eg2ic1(ne, np_, DE, DP, tables["GM2ICR"], tables["GM2SICR"])
    assert np.array_equal(fe.reshape(ne, ne, order="F"), FE) and E[0] == E2
    assert np.array_equal(fp.reshape(np_, np_, order="F"), FP)
    assert np.array_equal(se.reshape(ne, ne, order="F"), SE) and S[0] == S2
    # E_from_GAM_3 / E_from_GAM_4 against EG3IC1 / EG4ICR
    for fn, ng, ref in ((L.e_from_gam_3_, s.ng3, nx.eg3ic1(ne, np_, DE, DP, tables["GM3IC1"])),
                        (L.e_from_gam_4_, s.ng4, nx.eg4icr(ne, np_, DE, DP, tables["GM4ICR"]))):
        fe, fp, E = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
        fn(_i64(ne), _i64(np_), _i64(ng), _p(DE), _p(DP), _p(fe), _p(fp), _p(E))
        assert np.array_equal(fe.reshape(ne, ne, order="F"), ref[0]) and E[0] == ref[2]
    # xchf1_fock_ with every geminal term on its disk branch
    ic = nx.xchf1_fock(s, DE, DP, tables, tables["E_nuc"], modes=("gam4", "g4ic", "g3ic1",
                                                                   "g2ic1"))
    T, Fl = np.int64(-1), np.int64(0)    # ifort LOGICAL*8 .TRUE. / .FALSE.
    lg = [C.byref(C.c_int64(int(v))) for v in (Fl, T, Fl, Fl, Fl, Fl, Fl, Fl, Fl)]
    one = np.zeros(1)
    out = [np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(ne * ne), np.zeros(np_ * np_)]
    en = {k: np.zeros(1) for k in nx.FOCK_ENERGIES}
    en["E_nuc"][0] = tables["E_nuc"]
    sysb = [_p(a) for a in (s.cat_f, s.zan_f, s.bgem_f, s.ggem_f, s.KPESTR_f,
                            s.KPEEND_f)] + _basis_args(s)
    L.xchf1_fock_(*lg, _i64(1), _i64(1), _i64(1), _i64(1), _i64(1), _i64(1),
                  _i64(s.npebf), _i64(ne), _i64(ne * ne), _i64(np_), _i64(np_ * np_),
                  _i64(s.nelec), _i64(s.ngee), _i64(s.ng1), _i64(s.ng2), _i64(s.ng3),
                  _i64(s.ng4), _p(DE), _p(DP), _p(tables["GAM_ecore"]), _p(tables["GAM_pcore"]),
                  _p(tables["GAM_ep"]), _p(tables["GAM_ee"]), _p(one), _p(one), _p(one), _p(one),
                  _i64(s.ng2prm), _i64(s.ngtg), _i64(s.ng3prm), _i64(s.nat), _dbl(s.pmass),
                  *sysb, *[_p(a) for a in out], *[_p(en[k]) for k in nx.FOCK_ENERGIES])
    assert np.array_equal(out[0].reshape(ne, ne, order="F"), ic["focke"])
    assert np.array_equal(out[1].reshape(np_, np_, order="F"), ic["fockp"])
    for k in ENERGIES:
        assert en[k][0] == ic[k], k
