"""GPU special-electron contractions (k_rx.cu) against the oracle's
restatement (oracle/rx.c) of rxchf/rxchf_omg{2,3,4}.f (RXCHF-fe),
rxchf/rxcuhf_omg{2,3}.f (RXCUHF-fe), rxchfne/rxcuhfne_omg2.f (RXCUHF-ae) and
rxchf/rxchf_omg1.f.

The contractions are linear in the stored tensors, so seeded random tensors
and densities exercise every index pattern, including the bra/ket-mixed
partners of the rank-3 exchange terms.  Every output matrix accumulates into
a nonzero starting matrix, as the reference's add2fock does.  Tolerance:
1e-12 relative to the largest entry (FP64; sums in a different order).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


def _close(a, b, tol=1e-12):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.abs(a - b).max()) <= tol * max(1.0, float(np.abs(b).max()))


def _eclose(a, b):
    return abs(a - b) <= 1e-12 * max(1.0, abs(b))


def _case(seed, ne, np_, k, ntens):
    rng = np.random.default_rng(seed)
    T = [rng.standard_normal(ne ** (2 * k) * np_ ** 2) for _ in range(ntens)]
    sym = lambda n: (lambda A: A @ A.T / n)(rng.standard_normal((n, n)))
    Da, Db, Dsp, DP = sym(ne), sym(ne), sym(ne), sym(np_)
    F0 = {n: rng.standard_normal((n, n)) for n in (ne, np_)}
    return T, Da, Db, Da + Db, Dsp, DP, F0


def _oracle(orc, name, ne, np_, dens, tens, nmats, nen):
    L, P = orc.lib(), orc.ptr
    mats = [np.zeros(n * n) for n in nmats]
    ens = [np.zeros(1) for _ in range(nen)]
    args = [_f(d) for d in dens] + [np.ascontiguousarray(t) for t in tens]
    getattr(L, name)(ne, np_, *[P(a) for a in args], *[P(m) for m in mats],
                     *[P(e) for e in ens])
    return [m.reshape(n, n, order="F") for n, m in zip(nmats, mats)], [e[0] for e in ens]


@pytest.mark.parametrize("ne,np_", [(3, 2), (5, 1)])
def test_rxcuhfne_omg2(nx, orc, ne, np_):
    (G, X), Da, Db, Dt, Dsp, DP, F0 = _case(11 + ne, ne, np_, 2, 2)
    got = nx.rxcuhfne_omg2("fe", ne, np_, Da, Db, Dt, Dsp, DP, G, X, F=F0[ne], F2=F0[ne])
    (ra, rb), (re,) = _oracle(orc, "orc_rxcuhfne_fe_omg2", ne, np_, (Da, Dt, Dsp, DP), (G, X),
                              (ne, ne), 1)
    assert _close(got[0] - F0[ne], ra) and _close(got[1] - F0[ne], rb) and _eclose(got[2], re)
    for which, n in (("fp", np_), ("fbe", ne)):
        got = nx.rxcuhfne_omg2(which, ne, np_, Da, Db, Dt, Dsp, DP, G, X, F=F0[n])
        (rf,), (re,) = _oracle(orc, "orc_rxcuhfne_%s_omg2" % which, ne, np_,
                               (Da, Dt, Dsp, DP), (G, X), (n,), 1)
        assert _close(got[0] - F0[n], rf) and _eclose(got[1], re), which


@pytest.mark.parametrize("k,ne,np_", [(2, 3, 2), (2, 5, 1), (3, 3, 2), (3, 4, 1), (4, 3, 1),
                                      (4, 2, 2)])
def test_rxchf_fe(nx, orc, k, ne, np_):
    ntens = {2: 3, 3: 2, 4: 1}[k]
    T, Da, Db, Dt, Dsp, DP, F0 = _case(100 * k + 7 * ne + np_, ne, np_, k, ntens)
    for which in ("fae", "fp", "fbe"):
        n = np_ if which == "fp" else ne
        if k == 2:
            F, S, E, Es = nx.rxchf_omg(which, k, ne, np_, Da, Dsp, DP, T, F=F0[n], S=F0[n])
            (rf, rs), (re, res) = _oracle(orc, "orc_rxchf_%s_omg2" % which, ne, np_,
                                          (Da, Dsp, DP), T, (n, n), 2)
            assert _close(S - F0[n], rs) and _eclose(Es, res), which
        else:
            F, E = nx.rxchf_omg(which, k, ne, np_, Da, Dsp, DP, T, F=F0[n])
            (rf,), (re,) = _oracle(orc, "orc_rxchf_%s_omg%d" % (which, k), ne, np_,
                                   (Da, Dsp, DP), T, (n,), 1)
        assert _close(F - F0[n], rf), (k, which)
        assert _eclose(E, re), (k, which, E, re)


@pytest.mark.parametrize("k,ne,np_", [(2, 3, 2), (2, 4, 1), (3, 3, 2), (3, 4, 1)])
def test_rxcuhf_fe(nx, orc, k, ne, np_):
    ntens = 3 if k == 2 else 2
    T, Da, Db, Dt, Dsp, DP, F0 = _case(300 * k + 5 * ne + np_, ne, np_, k, ntens)
    F = F0[ne]
    if k == 2:
        got = nx.rxcuhf_omg("fe", 2, ne, np_, Da, Db, Dt, Dsp, DP, T, F=F, F2=F, F3=F)
        (ra, rb, rs), (re, res) = _oracle(orc, "orc_rxcuhf_fe_omg2", ne, np_,
                                          (Da, Dt, Dsp, DP), T, (ne, ne, ne), 2)
        assert _close(got[0] - F, ra) and _close(got[1] - F, rb) and _close(got[2] - F, rs)
        assert _eclose(got[3], re) and _eclose(got[4], res)
        for which, n in (("fp", np_), ("fbe", ne)):
            g = nx.rxcuhf_omg(which, 2, ne, np_, Da, Db, Dt, Dsp, DP, T, F=F0[n], F2=F0[n])
            (rf, rs), (re, res) = _oracle(orc, "orc_rxcuhf_%s_omg2" % which, ne, np_,
                                          (Da, Dt, Dsp, DP), T, (n, n), 2)
            assert _close(g[0] - F0[n], rf) and _close(g[1] - F0[n], rs), which
            assert _eclose(g[2], re) and _eclose(g[3], res), which
    else:
        got = nx.rxcuhf_omg("fe", 3, ne, np_, Da, Db, Dt, Dsp, DP, T, F=F, F2=F)
        (ra, rb), (re,) = _oracle(orc, "orc_rxcuhf_fe_omg3", ne, np_,
                                  (Da, Db, Dt, Dsp, DP), T, (ne, ne), 1)
        assert _close(got[0] - F, ra) and _close(got[1] - F, rb) and _eclose(got[2], re)
        for which, n in (("fp", np_), ("fbe", ne)):
            g = nx.rxcuhf_omg(which, 3, ne, np_, Da, Db, Dt, Dsp, DP, T, F=F0[n])
            (rf,), (re,) = _oracle(orc, "orc_rxcuhf_%s_omg3" % which, ne, np_,
                                   (Da, Db, Dt, Dsp, DP), T, (n,), 1)
            assert _close(g[0] - F0[n], rf) and _eclose(g[1], re), which


def test_rxchf_omg1(nx, orc):
    """RXCHF_FP_OMG1 / RXCHF_FBE_OMG1 are UFP_OMG1 / FAE_OMG1 with the
    special electron's density."""
    rng = np.random.default_rng(3)
    ne, np_ = 4, 3
    G1, G1s = rng.standard_normal(ne * ne * np_ * np_), rng.standard_normal(ne * ne * np_ * np_)
    B, P = rng.standard_normal((ne, ne)), rng.standard_normal((np_, np_))
    DB, DP = B @ B.T, P @ P.T
    L, Pt = orc.lib(), orc.ptr
    F, S, E, Sv = np.zeros(np_ * np_), np.zeros(np_ * np_), np.zeros(1), np.zeros(1)
    L.orc_ufp_omg1(ne, np_, Pt(_f(DB)), Pt(_f(DP)), Pt(G1), Pt(G1s), Pt(F), Pt(S), Pt(E), Pt(Sv))
    gF, gS, gE, gSv = nx.rxchf_omg1("fp", ne, np_, DB, DP, G1, G1s)
    assert _close(gF, F.reshape(np_, np_, order="F")) and _eclose(gE, E[0]) and _eclose(gSv, Sv[0])
    F, S = np.zeros(ne * ne), np.zeros(ne * ne)
    L.orc_fae_omg1(ne, np_, Pt(_f(DB)), Pt(_f(DP)), Pt(G1), Pt(G1s), Pt(F), Pt(S), Pt(E), Pt(Sv))
    gF, gS, gE, gSv = nx.rxchf_omg1("fbe", ne, np_, DB, DP, G1, G1s)
    assert _close(gF, F.reshape(ne, ne, order="F")) and _close(gS, S.reshape(ne, ne, order="F"))
    assert _eclose(gE, E[0]) and _eclose(gSv, Sv[0])
