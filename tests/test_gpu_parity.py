"""GPU parity: every C-ABI entry point against the CPU oracle.

Tolerances: integer index maps bit-exact; FP64 integral tensors within
1e-10 relative (element-wise on significant elements, scale-relative on
cancellation-dominated tiny ones); energies within 1e-10 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import OracleTensors, assert_close_scaled, fmat

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def _system(seed, **kw):
    from neoxc import basis
    return basis.synthetic(seed=seed, **kw)


def _dens(n, nocc, seed, prefac=2.0):
    from neoxc import basis
    return basis.random_density(n, nocc, seed, prefac)


# ---------------------------------------------------------------- index maps
@pytest.mark.parametrize("kind,ne,np_", [(0, 5, 1), (2, 4, 3), (3, 3, 2), (4, 2, 3)])
def test_index_map_bit_exact(nx, orc, kind, ne, np_):
    dev = nx.index_map(kind, ne, np_)
    L = orc.lib()
    ref = []
    if kind == 0:
        for i1 in range(1, ne + 1):
            for j1 in range(1, ne + 1):
                for i2 in range(1, ne + 1):
                    for j2 in range(1, ne + 1):
                        ref.append(L.orc_pack_4d(ne, ne, ne, j2, i2, j1, i1))
    else:
        import itertools
        nidx = 2 * kind
        fn = {2: L.orc_index_gam_2pk, 3: L.orc_index_gam_3pk, 4: L.orc_index_gam_4pk2}[kind]
        for ip, jp in itertools.product(range(1, np_ + 1), repeat=2):
            for e in itertools.product(range(1, ne + 1), repeat=nidx):
                ref.append(fn(ne, np_, ip, jp, *e))
    assert np.array_equal(dev, np.array(ref, np.int64))


def test_index_map_int64_range(nx, orc):
    """index_GAM_4PK2 at nebf=12, npbf=8 exceeds 2**31 (integer*8 path)."""
    n = 12 ** 8 * 8 ** 2
    head = nx.index_map(4, 12, 8, count=1 << 20)
    assert head[0] == 1 and np.all(np.diff(head) == 1)
    L = orc.lib()
    assert L.orc_index_gam_4pk2(12, 8, 8, 8, 12, 12, 12, 12, 12, 12, 12, 12) == n
    assert nx.index_gam_4pk2(12, 8, 8, 8, 12, 12, 12, 12, 12, 12, 12, 12) == n > 2 ** 31


# ----------------------------------------------------------- gam_4 element path
@pytest.mark.parametrize("seed,ne,np_", [(11, 3, 2), (12, 4, 1), (13, 2, 3), (14, 5, 2)])
def test_gam4_dscf_icr_eg4(nx, orc, seed, ne, np_):
    rng = np.random.default_rng(seed)
    gee = rng.standard_normal(ne ** 4)
    g2s = rng.standard_normal(ne ** 4 * np_ ** 2)
    DE = _dens(ne, max(1, ne // 2), seed)
    DP = _dens(np_, 1, seed + 1, 1.0)
    L, O = orc.lib(), orc
    # element-wise tensor (GAM4_ICR)
    g4 = nx.gam4_icr(ne, np_, g2s, gee)
    r4 = np.zeros(ne ** 8 * np_ ** 2)
    L.orc_gam4_icr(ne, np_, O.ptr(g2s), O.ptr(gee), O.ptr(r4))
    assert_close_scaled(g4, r4, RTOL, "GAM_4")
    # fused DSCF contraction, accumulating into pre-filled Fock matrices
    fe0, fp0 = rng.standard_normal((ne, ne)), rng.standard_normal((np_, np_))
    fe, fp, E = nx.gam4_dscf(ne, np_, gee, g2s, DE, DP, fe0, fp0)
    rfe, rfp, rE = fmat(fe0), fmat(fp0), np.zeros(1)
    L.orc_gam4_dscf_range(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(fmat(DE)), O.ptr(fmat(DP)),
                          0, ne ** 8 * np_ ** 2, O.ptr(rfe), O.ptr(rfp), O.ptr(rE))
    assert E == pytest.approx(rE[0], rel=RTOL, abs=1e-12)
    assert_close_scaled(fmat(fe), rfe, RTOL, "focke")
    assert_close_scaled(fmat(fp), rfp, RTOL, "fockp")
    # in-core contraction of the stored tensor (EG4ICR)
    fe2, fp2, E2 = nx.eg4icr(ne, np_, DE, DP, g4, fe0, fp0)
    assert E2 == pytest.approx(rE[0], rel=RTOL, abs=1e-12)
    assert_close_scaled(fmat(fe2), rfe, RTOL, "focke (EG4ICR)")


# ------------------------------------------------- factorised gam_4 Fock build
def _pair_symmetric_tables(rng, ne, np_):
    """Random tables with the symmetry of the reference's inputs:
    gs(p; ab; cd) = gs(p; cd; ab) (GAM2_IC1 pair symmetrisation) and
    (ab|cd) = (cd|ab) (ERIs)."""
    gs = rng.standard_normal((np_, np_, ne, ne, ne, ne))
    gs = 0.5 * (gs + gs.transpose(0, 1, 4, 5, 2, 3))
    ee = rng.standard_normal((ne,) * 4)
    ee = 0.5 * (ee + ee.transpose(2, 3, 0, 1))
    return np.ascontiguousarray(ee.ravel()), np.ascontiguousarray(gs.ravel())


@pytest.mark.parametrize("seed,ne,np_", [(51, 3, 2), (52, 4, 1), (53, 5, 2), (54, 2, 3)])
def test_gam4_fock_factored_vs_oracle(nx, orc, seed, ne, np_):
    """The factorised build reproduces the oracle's element-wise GAM4_DSCF
    (all ne^8 np^2 elements) on pair-symmetric tables, accumulating into
    pre-filled Fock matrices."""
    rng = np.random.default_rng(seed)
    gee, g2s = _pair_symmetric_tables(rng, ne, np_)
    DE, DP = _dens(ne, max(2, ne // 2), seed), _dens(np_, 1, seed + 1, 1.0)
    fe0, fp0 = rng.standard_normal((ne, ne)), rng.standard_normal((np_, np_))
    fe, fp, E = nx.gam4_fock_factored(ne, np_, gee, g2s, DE, DP, fe0, fp0)
    O, L = orc, orc.lib()
    rfe, rfp, rE = fmat(fe0), fmat(fp0), np.zeros(1)
    L.orc_gam4_dscf_range(ne, np_, O.ptr(gee), O.ptr(g2s), O.ptr(fmat(DE)), O.ptr(fmat(DP)),
                          0, ne ** 8 * np_ ** 2, O.ptr(rfe), O.ptr(rfp), O.ptr(rE))
    assert E == pytest.approx(rE[0], rel=RTOL, abs=1e-12)
    assert_close_scaled(fmat(fe), rfe, RTOL, "focke (factorised)")
    assert_close_scaled(fmat(fp), rfp, RTOL, "fockp (factorised)")


@pytest.mark.parametrize("ne,np_", [(8, 3), (12, 2)])
def test_gam4_fock_factored_vs_element_kernel(nx, ne, np_):
    """Against the GPU element-wise kernel at sizes beyond the oracle's reach;
    the two sum ~1e9-1e10 terms in different orders, so the check is against
    the matrices' scale."""
    rng = np.random.default_rng(60 + ne)
    gee, g2s = _pair_symmetric_tables(rng, ne, np_)
    DE, DP = _dens(ne, 3, ne), _dens(np_, 1, ne + 1, 1.0)
    a = nx.gam4_fock_factored(ne, np_, gee, g2s, DE, DP)
    b = nx.gam4_dscf(ne, np_, gee, g2s, DE, DP)
    for x, y, w in ((a[0], b[0], "focke"), (a[1], b[1], "fockp")):
        scale = np.abs(y).max()
        assert np.abs(x - y).max() <= 1e-10 * scale, w
    assert a[2] == pytest.approx(b[2], rel=1e-10)


def test_gam4_fock_factored_xchf_example(nx, xchf, golden_xchf):
    """examples/xchf through the factorised build: GAM_ee and GAM_2s from the
    GPU builders at the guessCE density give E_GAM4 of XCHF.log:315."""
    s, DE, DP = xchf["sys"], xchf["DE0"], xchf["DP0"]
    gee = nx.calc_gam_ee(s)
    _, g2s = nx.gam2_ic1(s)
    E4 = nx.gam4_fock_factored(s.nebf, s.npbf, gee, g2s, DE, DP)[2]
    assert abs(E4 - golden_xchf["initial"]["E_GAM4"]) <= 6e-11


def test_gam4_fock_factored_properties_large(nx):
    """nebf=40, npbf=6: E is linear in DP and quartic in DE, E = sum DP fockp,
    and sum DE focke = 4 E (focke is dE/dDE)."""
    ne, np_ = 40, 6
    rng = np.random.default_rng(7)
    gee, g2s = _pair_symmetric_tables(rng, ne, np_)
    DE, DP = _dens(ne, 5, 8), _dens(np_, 1, 9, 1.0)
    fe, fp, E = nx.gam4_fock_factored(ne, np_, gee, g2s, DE, DP)
    assert np.isfinite(E) and abs(E) > 0
    assert float((DP * fp).sum()) == pytest.approx(E, rel=1e-12)
    E2 = nx.gam4_fock_factored(ne, np_, gee, g2s, DE, 2.0 * DP)[2]
    assert E2 == pytest.approx(2.0 * E, rel=1e-12)
    E3 = nx.gam4_fock_factored(ne, np_, gee, g2s, 0.5 * DE, DP)[2]
    assert E3 == pytest.approx(E / 16.0, rel=1e-12)
    # focke is dE/dDE: DE-weighted trace gives 4 E (degree-4 homogeneity)
    assert float((DE * fe).sum()) == pytest.approx(4.0 * E, rel=1e-10)


def test_gam4_fock_factored_rejects_asymmetric_tables(nx):
    rng = np.random.default_rng(3)
    ne, np_ = 3, 2
    gee, g2s = _pair_symmetric_tables(rng, ne, np_)
    bad = g2s.copy()
    bad[5] += 1e-3
    with pytest.raises(nx.NeoxcError, match="GAM_2s is not pair-symmetric"):
        nx.gam4_fock_factored(ne, np_, gee, bad, np.eye(ne), np.eye(np_))
    bad = gee.copy()
    bad[7] += 1e-3
    with pytest.raises(nx.NeoxcError, match="GAM_ee is not symmetric"):
        nx.gam4_fock_factored(ne, np_, bad, g2s, np.eye(ne), np.eye(np_))


def test_gam4_dscf_deterministic(nx):
    rng = np.random.default_rng(5)
    ne, np_ = 6, 2
    gee, g2s = rng.standard_normal(ne ** 4), rng.standard_normal(ne ** 4 * np_ ** 2)
    DE, DP = _dens(ne, 3, 1), _dens(np_, 1, 2, 1.0)
    a = nx.gam4_dscf(ne, np_, gee, g2s, DE, DP)
    b = nx.gam4_dscf(ne, np_, gee, g2s, DE, DP)
    assert a[2] == b[2]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


# ------------------------------------------------------------ in-core contractions
@pytest.mark.parametrize("seed,ne,np_", [(21, 3, 2), (22, 5, 1), (23, 4, 3)])
def test_eg3ic1(nx, orc, seed, ne, np_):
    rng = np.random.default_rng(seed)
    g3 = rng.standard_normal(ne ** 6 * np_ ** 2)
    DE, DP = _dens(ne, 2, seed), _dens(np_, 1, seed + 1, 1.0)
    fe0, fp0 = rng.standard_normal((ne, ne)), rng.standard_normal((np_, np_))
    fe, fp, E = nx.eg3ic1(ne, np_, DE, DP, g3, fe0, fp0)
    O, L = orc, orc.lib()
    rfe, rfp, rE = fmat(fe0), fmat(fp0), np.zeros(1)
    L.orc_eg3ic1(ne, np_, O.ptr(fmat(DE)), O.ptr(fmat(DP)), O.ptr(g3), O.ptr(rfe), O.ptr(rfp),
                 O.ptr(rE))
    assert E == pytest.approx(rE[0], rel=RTOL, abs=1e-12)
    assert_close_scaled(fmat(fe), rfe, RTOL, "focke")
    assert_close_scaled(fmat(fp), rfp, RTOL, "fockp")


@pytest.mark.parametrize("seed,ne,np_", [(31, 3, 2), (32, 6, 1), (33, 4, 3)])
def test_eg2ic1(nx, orc, seed, ne, np_):
    rng = np.random.default_rng(seed)
    g2, g2s = rng.standard_normal(ne ** 4 * np_ ** 2), rng.standard_normal(ne ** 4 * np_ ** 2)
    DE, DP = _dens(ne, 2, seed), _dens(np_, 1, seed + 1, 1.0)
    FE0, FP0 = rng.standard_normal((ne, ne)), rng.standard_normal((np_, np_))
    FE, SE, FP, SP, E, S = nx.eg2ic1(ne, np_, DE, DP, g2, g2s, FE0, FP0)
    O, L = orc, orc.lib()
    rFE, rSE, rFP, rSP = fmat(FE0), np.full(ne * ne, 7.0), fmat(FP0), np.full(np_ * np_, 7.0)
    rE, rS = np.zeros(1), np.zeros(1)
    L.orc_eg2ic1(ne, np_, O.ptr(fmat(DE)), O.ptr(fmat(DP)), O.ptr(g2), O.ptr(g2s), O.ptr(rFE),
                 O.ptr(rSE), O.ptr(rFP), O.ptr(rSP), O.ptr(rE), O.ptr(rS))
    assert E == pytest.approx(rE[0], rel=RTOL, abs=1e-12)
    assert S == pytest.approx(rS[0], rel=RTOL, abs=1e-12)
    for a, b, w in ((FE, rFE, "FE"), (SE, rSE, "SE"), (FP, rFP, "FP"), (SP, rSP, "SP")):
        assert_close_scaled(fmat(a), b, RTOL, w)


@pytest.mark.parametrize("seed,ne,np_", [(41, 3, 2), (42, 7, 1), (43, 5, 3)])
def test_rxchfne_omg2(nx, orc, seed, ne, np_):
    rng = np.random.default_rng(seed)
    g2 = rng.standard_normal(ne ** 4 * np_ ** 2)
    DAE, DBE = _dens(ne, 2, seed), _dens(ne, 1, seed + 7, 1.0)
    DP = _dens(np_, 1, seed + 1, 1.0)
    O, L = orc, orc.lib()
    F0 = rng.standard_normal((ne, ne))
    P0 = rng.standard_normal((np_, np_))
    fae, e1 = nx.rxchfne_fae_omg2(ne, np_, DAE, DBE, DP, g2, F0)
    fp, e2 = nx.rxchfne_fp_omg2(ne, np_, DAE, DBE, DP, g2, P0)
    fbe, e3 = nx.rxchfne_fbe_omg2(ne, np_, DAE, DBE, DP, g2, F0)
    args = [O.ptr(fmat(DAE)), O.ptr(fmat(DBE)), O.ptr(fmat(DP)), O.ptr(g2)]
    r1, r2, r3 = fmat(F0), fmat(P0), fmat(F0)
    E1, E2, E3 = np.zeros(1), np.zeros(1), np.zeros(1)
    L.orc_rxchfne_fae_omg2(ne, np_, *args, O.ptr(r1), O.ptr(E1))
    L.orc_rxchfne_fp_omg2(ne, np_, *args, O.ptr(r2), O.ptr(E2))
    L.orc_rxchfne_fbe_omg2(ne, np_, *args, O.ptr(r3), O.ptr(E3))
    assert_close_scaled(fmat(fae), r1, RTOL, "FAE")
    assert_close_scaled(fmat(fp), r2, RTOL, "FP")
    assert_close_scaled(fmat(fbe), r3, RTOL, "FBE")
    for e, r in ((e1, E1), (e2, E2), (e3, E3)):
        assert e == pytest.approx(r[0], rel=RTOL, abs=1e-12)
    fa2, fp2, fb2, ef = nx.rxchfne_omg2_fused(ne, np_, DAE, DBE, DP, g2)
    assert ef == pytest.approx(E1[0], rel=RTOL, abs=1e-12)
    assert_close_scaled(fmat(fa2) + fmat(F0), r1, RTOL, "FAE fused")


def test_xcfock_correction(nx, orc):
    rng = np.random.default_rng(3)
    ne, np_ = 5, 3
    m = [rng.standard_normal(n * n) for n in (ne, np_, ne, np_, ne, np_)]
    fe, fp = nx.xcfock_correction(ne, np_, -5.7, 170.97, -0.03, *[x.copy() for x in m])
    O, L = orc, orc.lib()
    rfe, rfp = m[4].copy(), m[5].copy()
    L.orc_xcfock_correction(ne, np_, 170.97, -0.03, *[O.ptr(x) for x in m[:4]], O.ptr(rfe),
                            O.ptr(rfp))
    assert_close_scaled(fmat(fe), rfe, 1e-14, "focke")
    assert_close_scaled(fmat(fp), rfp, 1e-14, "fockp")


# ---------------------------------------------------------------- builders (MD)
SMALL = [
    dict(seed=101, nat=2, nebf=2, nprim=2, npbf=2, ngtg=2, lmax_e=1, lmax_p=1),
    dict(seed=102, nat=3, nebf=3, nprim=1, npbf=1, ngtg=3, lmax_e=1, lmax_p=0),
    dict(seed=103, nat=2, nebf=2, nprim=(1, 2), npbf=2, ngtg=2, lmax_e=2, lmax_p=2),
]


@pytest.mark.parametrize("kw", SMALL)
def test_gam_ee(nx, orc, kw):
    s = _system(**kw)
    T = OracleTensors(orc, s)
    assert_close_scaled(nx.calc_gam_ee(s), T.get("gee"), RTOL, "GAM_ee")


@pytest.mark.parametrize("kw", SMALL)
def test_gam2_ic1(nx, orc, kw):
    s = _system(**kw)
    T = OracleTensors(orc, s)
    g2, g2s = nx.gam2_ic1(s)
    assert_close_scaled(g2, T.get("g2"), RTOL, "GM2ICR")
    assert_close_scaled(g2s, T.get("g2s"), RTOL, "GM2sICR")


@pytest.mark.parametrize("kw", SMALL)
def test_rxchfne_gam2_ic1(nx, orc, kw):
    s = _system(**kw)
    T = OracleTensors(orc, s)
    g, gx = nx.rxchfne_gam2_ic1(s)
    assert_close_scaled(g, T.get("rx2"), RTOL, "GM2ICR (RXCHF-ne)")
    assert_close_scaled(gx, T.get("rx2ex"), RTOL, "GM2exICR")


# gam_3 cases: the s/p systems above and one with an electronic d shell
# (nebf=5 cycles s, px, py, pz, dxx; the oracle needs ~10 s of CPU for it)
GAM3_CASES = SMALL[:2] + [dict(seed=105, nat=2, nebf=5, nprim=1, npbf=1, ngtg=2,
                               lmax_e=2, lmax_p=0)]


@pytest.mark.parametrize("kw", GAM3_CASES)
def test_gam3_ic1(nx, orc, kw):
    s = _system(**kw)
    T = OracleTensors(orc, s)
    assert_close_scaled(nx.gam3_ic1(s), T.get("g3"), RTOL, "GM3ICR")


# Direct-SCF builders.  Every case is checked against the oracle's in-core
# pipeline (GAM3_IC1 + EG3IC1, GAM2_IC1 + EG2IC1); the tiny cases (one
# primitive per contracted function) also against the oracle's restatement of
# the direct loops, which re-evaluates every particle ordering of every tuple.
DSCF_CASES = [
    (True, dict(seed=113, nat=2, nebf=2, nprim=1, npbf=2, ngtg=2, lmax_e=1, lmax_p=1)),
    (False, dict(seed=111, nat=2, nebf=3, nprim=1, npbf=2, ngtg=2, lmax_e=1, lmax_p=1)),
    (False, dict(seed=112, nat=2, nebf=2, nprim=(1, 2), npbf=3, ngtg=2, lmax_e=2, lmax_p=1)),
]


def _dscf_inputs(kw, n_extra):
    s = _system(**kw)
    ne, np_ = s.nebf, s.npbf
    rng = np.random.default_rng(kw["seed"] + 7)
    DE, DP = _dens(ne, 2, kw["seed"]), _dens(np_, 1, kw["seed"] + 1, 1.0)
    m0 = [rng.standard_normal((n, n)) for n in (ne, np_, ne, np_)[:n_extra]]
    return s, ne, np_, DE, DP, m0


def _close_e(got, want, what):
    assert abs(got - want) <= RTOL * max(1.0, abs(want)), (what, got, want)


@pytest.mark.parametrize("direct,kw", DSCF_CASES)
def test_gam3_dscf(nx, orc, direct, kw):
    """GAM3_DSCF (proton-pair slices built and contracted on the fly):
    focke/fockp accumulate into pre-filled matrices, E_gam3 overwritten."""
    s, ne, np_, DE, DP, m0 = _dscf_inputs(kw, 2)
    fe, fp, E = nx.gam3_dscf(s, DE, DP, *m0)
    L, T = orc.lib(), OracleTensors(orc, s)
    rfe, rfp, rE = m0[0].ravel("F").copy(), m0[1].ravel("F").copy(), np.zeros(1)
    L.orc_eg3ic1(ne, np_, orc.ptr(fmat(DE)), orc.ptr(fmat(DP)), orc.ptr(T.get("g3")),
                 orc.ptr(rfe), orc.ptr(rfp), orc.ptr(rE))
    assert_close_scaled(fe.ravel("F"), rfe, RTOL, "focke (GAM3_DSCF vs in-core)")
    assert_close_scaled(fp.ravel("F"), rfp, RTOL, "fockp (GAM3_DSCF vs in-core)")
    _close_e(E, rE[0], "E_gam3")
    if direct:
        dfe, dfp, dE = m0[0].ravel("F").copy(), m0[1].ravel("F").copy(), np.zeros(1)
        L.orc_gam3_dscf(T.h.ref, orc.ptr(fmat(DE)), orc.ptr(fmat(DP)),
                        orc.ptr(dfe), orc.ptr(dfp), orc.ptr(dE))
        assert_close_scaled(fe.ravel("F"), dfe, RTOL, "focke (direct oracle)")
        assert_close_scaled(fp.ravel("F"), dfp, RTOL, "fockp (direct oracle)")
        _close_e(E, dE[0], "E_gam3 (direct oracle)")


@pytest.mark.parametrize("direct,kw", DSCF_CASES)
def test_gam2_dscf(nx, orc, direct, kw):
    """GAM2_DSCF: focke/fockp/se2/sp2 accumulate, E_gam2/S_gam2 overwritten."""
    s, ne, np_, DE, DP, m0 = _dscf_inputs(kw, 4)
    out = nx.gam2_dscf(s, DE, DP, *m0)
    L, T = orc.lib(), OracleTensors(orc, s)
    fe, fp = m0[0].ravel("F").copy(), m0[1].ravel("F").copy()
    se, sp, E, S = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1), np.zeros(1)
    L.orc_eg2ic1(ne, np_, orc.ptr(fmat(DE)), orc.ptr(fmat(DP)), orc.ptr(T.get("g2")),
                 orc.ptr(T.get("g2s")), orc.ptr(fe), orc.ptr(se), orc.ptr(fp),
                 orc.ptr(sp), orc.ptr(E), orc.ptr(S))
    ref = [fe, fp, m0[2].ravel("F") + se, m0[3].ravel("F") + sp]
    names = ("focke", "fockp", "se2", "sp2")
    for got, want, name in zip(out[:4], ref, names):
        assert_close_scaled(got.ravel("F"), want, RTOL, name + " (GAM2_DSCF vs in-core)")
    _close_e(out[4], E[0], "E_gam2")
    _close_e(out[5], S[0], "S_gam2")
    if direct:
        d = [m.ravel("F").copy() for m in m0]
        dE, dS = np.zeros(1), np.zeros(1)
        L.orc_gam2_dscf(T.h.ref, orc.ptr(fmat(DE)), orc.ptr(fmat(DP)),
                        *[orc.ptr(x) for x in d], orc.ptr(dE), orc.ptr(dS))
        for got, want, name in zip(out[:4], d, names):
            assert_close_scaled(got.ravel("F"), want, RTOL, name + " (direct oracle)")
        _close_e(out[4], dE[0], "E_gam2 (direct oracle)")
        _close_e(out[5], dS[0], "S_gam2 (direct oracle)")


def test_xchf_example_full_pipeline(nx, xchf, golden_xchf):
    """examples/xchf end to end on the GPU: GAM_ee, GAM2_IC1, GAM3_IC1 and
    the EG2/EG3/GAM4_DSCF contractions at the guessCE density reproduce
    XCHF.log:313-315."""
    s, DE, DP = xchf["sys"], xchf["DE0"], xchf["DP0"]
    gee = nx.calc_gam_ee(s)
    g2, g2s = nx.gam2_ic1(s)
    g3 = nx.gam3_ic1(s)
    ne, np_ = s.nebf, s.npbf
    E2 = nx.eg2ic1(ne, np_, DE, DP, g2, g2s)[4]
    E3 = nx.eg3ic1(ne, np_, DE, DP, g3)[2]
    E4 = nx.gam4_dscf(ne, np_, gee, g2s, DE, DP)[2]
    ref = golden_xchf["initial"]
    assert abs(E2 - ref["E_GAM2"]) <= 6e-11
    assert abs(E3 - ref["E_GAM3"]) <= 6e-11
    assert abs(E4 - ref["E_GAM4"]) <= 6e-11


# ------------------------------------------------------------------ error paths
def test_unsupported_shapes_are_errors(nx):
    rng = np.random.default_rng(0)
    with pytest.raises(nx.NeoxcError, match="ne <= 24"):
        nx.gam4_dscf(25, 1, np.zeros(25 ** 4), np.zeros(25 ** 4), np.eye(25), np.eye(1))
    s = _system(seed=1, nat=1, nebf=1, nprim=1, npbf=1, ngtg=1, lmax_e=0, lmax_p=0)
    s.ELCAM[0] = (2, 1, 0)
    with pytest.raises(nx.NeoxcError, match="total l > 2"):
        nx.gam2_ic1(s)
    with pytest.raises(nx.NeoxcError, match="ng4"):
        nx.lib()  # noqa: B018
        import ctypes as C
        a = np.zeros(16)
        rc = nx.lib().neoxc_gam4_dscf(1, 2, 1, 16, 16, 17, *([a.ctypes.data_as(C.c_void_p)] * 7))
        assert rc == 1
        raise nx.NeoxcError(nx.lib().neoxc_last_error().decode())
