"""GPU open-shell XCUHF contractions (k_spin.cu) against the oracle's
restatement of xcuhf/xcuhf_omg{1..4}.f, and the XCUHF example's
initial-guess energetics against examples/xcuhf/answer/XCUHF.log.

The contractions are linear in the stored tensor, so seeded random tensors
exercise every index path; the spin flags are covered by electron counts
that switch each term set on and off.  Tolerance: 1e-12 relative to the
largest output entry (FP64 throughout; sums run in a different order).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUNTS = [(2, 2), (3, 1), (1, 3), (4, 0), (0, 3), (5, 4), (1, 1)]


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


def _close(a, b, tol=1e-12):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = max(1.0, float(np.abs(b).max()) if b.size else 1.0)
    return float(np.abs(a - b).max()) <= tol * scale


def _rand_case(seed, ne, np_, k):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal(ne ** (2 * k) * np_ ** 2)
    Gs = rng.standard_normal(G.size) if k == 2 else None
    A, B = rng.standard_normal((ne, ne)), rng.standard_normal((ne, ne))
    P = rng.standard_normal((np_, np_))
    return G, Gs, A @ A.T / ne, B @ B.T / ne, P @ P.T / np_


def _oracle(orc, k, ne, np_, nae, nbe, G, Gs, DA, DB, DP, proton):
    L, P = orc.lib(), orc.ptr
    n = np_ if proton else ne
    F, S, E, Sv = np.zeros(n * n), np.zeros(n * n), np.zeros(1), np.zeros(1)
    da, db, dp = _f(DA), _f(DB), _f(DP)
    name = ("orc_ufp_omg%d" if proton else "orc_fae_omg%d") % k
    if k == 2:
        getattr(L, name)(ne, np_, nae, nbe, P(da), P(db), P(dp), P(G), P(Gs), P(F), P(S), P(E),
                         P(Sv))
    else:
        getattr(L, name)(ne, np_, nae, nbe, P(da), P(db), P(dp), P(G), P(F), P(E))
    return F.reshape(n, n, order="F"), S.reshape(n, n, order="F"), E[0], Sv[0]


@pytest.mark.parametrize("k,ne,np_", [(2, 3, 2), (2, 5, 1), (2, 4, 3), (3, 3, 2), (3, 4, 1),
                                      (3, 5, 2), (4, 3, 2), (4, 4, 1)])
def test_fae_ufp_match_oracle(nx, orc, k, ne, np_):
    G, Gs, DA, DB, DP = _rand_case(10 * k + ne + np_, ne, np_, k)
    F0 = np.random.default_rng(1).standard_normal((ne, ne))
    P0 = np.random.default_rng(2).standard_normal((np_, np_))
    for nae, nbe in COUNTS:
        # alpha, beta (the reference's second FAE call swaps the spins), proton
        for spin in (0, 1):
            a, b = (DA, DB) if spin == 0 else (DB, DA)
            na, nb = (nae, nbe) if spin == 0 else (nbe, nae)
            rF, rS, rE, rSv = _oracle(orc, k, ne, np_, na, nb, G, Gs, a, b, DP, False)
            if k == 2:
                F, S, E, Sv = nx.fae_omg2(ne, np_, na, nb, a, b, DP, G, Gs, FAE=F0)
                assert _close(S, rS) and abs(Sv - rSv) <= 1e-12 * max(1, abs(rSv))
            else:
                fn = nx.fae_omg3 if k == 3 else nx.fae_omg4
                F, E = fn(ne, np_, na, nb, a, b, DP, G, FAE=F0)
            assert _close(F - F0, rF), (k, nae, nbe, spin)
            assert abs(E - rE) <= 1e-12 * max(1.0, abs(rE)), (k, nae, nbe, spin, E, rE)
        rF, rS, rE, rSv = _oracle(orc, k, ne, np_, nae, nbe, G, Gs, DA, DB, DP, True)
        if k == 2:
            F, S, E, Sv = nx.ufp_omg2(ne, np_, nae, nbe, DA, DB, DP, G, Gs, FP=P0)
            assert _close(S, rS) and abs(Sv - rSv) <= 1e-12 * max(1, abs(rSv))
        else:
            fn = nx.ufp_omg3 if k == 3 else nx.ufp_omg4
            F, E = fn(ne, np_, nae, nbe, DA, DB, DP, G, FP=P0)
        assert _close(F - P0, rF), (k, nae, nbe)
        assert abs(E - rE) <= 1e-12 * max(1.0, abs(rE)), (k, nae, nbe, E, rE)


def test_omg2_global_memory_path(nx, orc):
    """nebf = 90: the rank-2 kernel gathers from global memory (the ket block
    of one bra no longer fits in shared memory)."""
    ne, np_ = 90, 1
    G, Gs, DA, DB, DP = _rand_case(77, ne, np_, 2)
    for nae, nbe in ((3, 2), (1, 0)):
        rF, rS, rE, rSv = _oracle(orc, 2, ne, np_, nae, nbe, G, Gs, DA, DB, DP, False)
        F, S, E, Sv = nx.fae_omg2(ne, np_, nae, nbe, DA, DB, DP, G, Gs)
        assert _close(F, rF) and _close(S, rS) and abs(E - rE) <= 1e-12 * abs(rE)
        rF, rS, rE, rSv = _oracle(orc, 2, ne, np_, nae, nbe, G, Gs, DA, DB, DP, True)
        F, S, E, Sv = nx.ufp_omg2(ne, np_, nae, nbe, DA, DB, DP, G, Gs)
        assert _close(F, rF) and _close(S, rS) and abs(E - rE) <= 1e-12 * abs(rE)


def test_fused_device_entry_equals_reference_calls(nx, orc):
    """neoxc_dev_xcuhf_omg: FAE, FBE and FP of one rank from one call equal
    the three reference routines' results."""
    import torch
    dev = torch.device("cuda:0")
    st = torch.cuda.current_stream(dev).cuda_stream
    for k, ne, np_ in ((2, 4, 2), (3, 4, 2), (4, 3, 2)):
        G, Gs, DA, DB, DP = _rand_case(500 + k, ne, np_, k)
        for nae, nbe in ((2, 2), (3, 1), (0, 2)):
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
            dG = t(G)
            dGs = t(Gs) if Gs is not None else None
            dA, dB, dP = t(_f(DA)), t(_f(DB)), t(_f(DP))
            FA, FB = torch.zeros(ne * ne, dtype=torch.float64, device=dev), \
                torch.zeros(ne * ne, dtype=torch.float64, device=dev)
            FP = torch.zeros(np_ * np_, dtype=torch.float64, device=dev)
            SA, SB = torch.zeros_like(FA), torch.zeros_like(FB)
            SP = torch.zeros_like(FP)
            E = torch.zeros(6, dtype=torch.float64, device=dev)
            two = k == 2
            nx.dev_xcuhf_omg(st, k, ne, np_, nae, nbe, dG, dGs, dA, dB, dP, FA, FB, FP,
                             SA if two else None, SB if two else None, SP if two else None,
                             E)
            torch.cuda.synchronize()
            e = E.cpu().numpy()
            for spin, Fd, Sd in ((0, FA, SA), (1, FB, SB)):
                a, b = (DA, DB) if spin == 0 else (DB, DA)
                na, nb = (nae, nbe) if spin == 0 else (nbe, nae)
                rF, rS, rE, rSv = _oracle(orc, k, ne, np_, na, nb, G, Gs, a, b, DP, False)
                assert _close(Fd.cpu().numpy().reshape(ne, ne, order="F"), rF)
                assert abs(e[spin] - rE) <= 1e-12 * max(1.0, abs(rE))
                if two:
                    assert _close(Sd.cpu().numpy().reshape(ne, ne, order="F"), rS)
                    assert abs(e[3 + spin] - rSv) <= 1e-12 * max(1.0, abs(rSv))
            rF, rS, rE, rSv = _oracle(orc, k, ne, np_, nae, nbe, G, Gs, DA, DB, DP, True)
            assert _close(FP.cpu().numpy().reshape(np_, np_, order="F"), rF)
            assert abs(e[2] - rE) <= 1e-12 * max(1.0, abs(rE))


def test_omg1_match_oracle(nx, orc):
    rng = np.random.default_rng(41)
    ne, np_ = 5, 3
    G1, G1s = rng.standard_normal(ne * ne * np_ * np_), rng.standard_normal(ne * ne * np_ * np_)
    A, P = rng.standard_normal((ne, ne)), rng.standard_normal((np_, np_))
    DA, DP = A @ A.T, P @ P.T
    L, Pt = orc.lib(), orc.ptr
    F, S, E, Sv = np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(1), np.zeros(1)
    L.orc_fae_omg1(ne, np_, Pt(_f(DA)), Pt(_f(DP)), Pt(G1), Pt(G1s), Pt(F), Pt(S), Pt(E), Pt(Sv))
    gF, gS, gE, gSv = nx.fae_omg1(ne, np_, DA, DP, G1, G1s)
    assert _close(gF, F.reshape(ne, ne, order="F")) and _close(gS, S.reshape(ne, ne, order="F"))
    assert abs(gE - E[0]) <= 1e-12 * abs(E[0]) and abs(gSv - Sv[0]) <= 1e-12 * abs(Sv[0])
    F, S = np.zeros(np_ * np_), np.zeros(np_ * np_)
    L.orc_ufp_omg1(ne, np_, Pt(_f(DA)), Pt(_f(DP)), Pt(G1), Pt(G1s), Pt(F), Pt(S), Pt(E), Pt(Sv))
    gF, gS, gE, gSv = nx.ufp_omg1(ne, np_, DA, DP, G1, G1s)
    assert _close(gF, F.reshape(np_, np_, order="F")) and _close(gS, S.reshape(np_, np_, order="F"))
    assert abs(gE - E[0]) <= 1e-12 * abs(E[0]) and abs(gSv - Sv[0]) <= 1e-12 * abs(Sv[0])


def test_omg4_icr_matches_oracle(nx, orc):
    """OMG4_ICR: the same operations in the same order as the oracle (no
    fused multiply-add), so the tensors agree to the last bit."""
    rng = np.random.default_rng(8)
    for ne, np_ in ((3, 2), (4, 1)):
        g2s = rng.standard_normal(ne ** 4 * np_ ** 2)
        gee = rng.standard_normal(ne ** 4)
        g2s[::7] *= 1e-101   # below the underflow cut
        ref = np.zeros(ne ** 8 * np_ ** 2)
        orc.lib().orc_omg4_icr(ne, np_, orc.ptr(g2s), orc.ptr(gee), orc.ptr(ref))
        got = nx.omg4_icr(ne, np_, g2s, gee)
        assert np.array_equal(got, ref), np.abs(got - ref).max()


def test_limits_are_reported(nx):
    """Rank 4 stages ne^4 kets per bra in shared memory: nebf = 13 is
    refused before any array is read (all array pointers are NULL here)."""
    ne, np_ = 13, 1
    rc = nx.lib().neoxc_fae_omg4(1, ne, np_, ne ** 8 * np_ ** 2, 2, 2, None, None, None,
                                 None, None, None)
    assert rc == 4 and b"nebf <= 12" in nx.lib().neoxc_last_error()


@pytest.fixture(scope="module")
def xcuhf_example(nx, golden_xcuhf):
    """examples/xcuhf at the core-Hamiltonian guess: GM2ICR / GM2sICR /
    GM3ICR built on the GPU, one-body integrals, GAM_1 and GAM_ee from the
    oracle."""
    import re
    import xcuhf as U
    from neoxc import basis
    s = basis.parse_inp(golden_xcuhf["inp"], name="examples/xcuhf")
    m = re.search(r"&XCUHF\s*nae=(\d+),\s*nbe=(\d+)", golden_xcuhf["inp"], re.I)
    nae, nbe = int(m.group(1)), int(m.group(2))
    G2, G2s = nx.gam2_ic1(s)
    G3 = nx.gam3_ic1(s)
    ints = U.XcuhfIntegrals(s, G2=G2, G2s=G2s, G3=G3)
    DAE, DBE, DP = U.guess(ints, nae, nbe, s.nucst)
    return dict(s=s, nae=nae, nbe=nbe, ints=ints, DAE=DAE, DBE=DBE, DP=DP)


def test_xcuhf_example_oracle_pinned(xcuhf_example, golden_xcuhf):
    """The oracle's UHF_FOCK energetics at the guess reproduce
    XCUHF.log:337-352 to its 10 printed decimals."""
    import xcuhf as U
    x = xcuhf_example
    r = U.uhf_energetics(x["ints"], x["nae"], x["nbe"], x["DAE"], x["DBE"], x["DP"])
    for key, ref in golden_xcuhf["initial"].items():
        assert abs(r[key] - ref) <= 6e-11 * max(1.0, abs(ref)), (key, r[key], ref)


def test_xcuhf_example_gpu_energetics(nx, xcuhf_example, golden_xcuhf):
    """The same energetics with every open-shell contraction on the GPU
    (OMG4_ICR built on the device and contracted there)."""
    import torch
    x = xcuhf_example
    s, ints = x["s"], x["ints"]
    ne, np_ = s.nebf, s.npbf
    DAE, DBE, DP = x["DAE"], x["DBE"], x["DP"]
    DT = DAE + DBE
    _, _, E1, S1 = nx.ufp_omg1(ne, np_, DT, DP, ints.G1, ints.G1s)
    _, _, E2, S2 = nx.ufp_omg2(ne, np_, x["nae"], x["nbe"], DAE, DBE, DP, ints.G2, ints.G2s)
    _, E3 = nx.ufp_omg3(ne, np_, x["nae"], x["nbe"], DAE, DBE, DP, ints.G3)
    dev = torch.device("cuda:0")
    st = torch.cuda.current_stream(dev).cuda_stream
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
    g4 = torch.empty(ne ** 8 * np_ ** 2, dtype=torch.float64, device=dev)
    nx.dev_omg4_icr(st, ne, np_, t(ints.Gee), t(ints.G2s), g4)
    FP = torch.zeros(np_ * np_, dtype=torch.float64, device=dev)
    E = torch.zeros(6, dtype=torch.float64, device=dev)
    nx.dev_xcuhf_omg(st, 4, ne, np_, x["nae"], x["nbe"], g4, None, t(_f(DAE)), t(_f(DBE)),
                     t(_f(DP)), None, None, FP, None, None, None, E)
    torch.cuda.synchronize()
    E4 = float(E[2].item())
    del g4
    S_total = 1.0 + S1 + S2
    ref = golden_xcuhf["initial"]
    assert abs(S_total - ref["S_TOTAL"]) <= 6e-11 * ref["S_TOTAL"]
    for key, val in (("E_OMG1", E1), ("E_OMG2", E2), ("E_OMG3", E3), ("E_OMG4", E4)):
        assert abs(val / S_total - ref[key]) <= 6e-11, (key, val / S_total, ref[key])


def test_xcuhf_device_scf_example(nx, xcuhf_example, golden_xcuhf):
    """neoxc_xcuhf_scf on examples/xcuhf from the core-Hamiltonian guesses:
    the initial energetics reproduce XCUHF.log:337-352 and the SCF reaches
    the log's converged energy (XCUHF.log:366, reached there with SOSCF;
    plain Roothaan and DIIS find the same stationary point)."""
    x = xcuhf_example
    s = x["s"]
    names = {"E_NUC": "E_nuc", "E_ECORE": "E_ecore", "E_PCORE": "E_pcore", "E_EP": "E_ep",
             "E_EE": "E_ee", "E_OMG1": "E_omg1", "E_OMG2": "E_omg2", "E_OMG3": "E_omg3",
             "E_OMG4": "E_omg4", "S_TOTAL": "S_total", "E_TOTAL": "E_total"}
    iters = {}
    for diis in (False, True):
        r = nx.xcuhf_scf(s, x["nae"], x["nbe"], diis=diis, maxit=250)
        for key, mine in names.items():
            ref = golden_xcuhf["initial"][key]
            assert abs(r["initial"][mine] - ref) <= 6e-11 * max(1.0, abs(ref)), (key, diis)
        assert r["converged"], (diis, r["history"][-3:])
        fin = golden_xcuhf["final"]
        print("XCUHF device SCF diis=%s: %d iterations, E = %.10f (log %.10f)"
              % (diis, r["niter"], r["final"]["E_total"], fin["E_TOTAL"]))
        assert abs(r["final"]["E_total"] - fin["E_TOTAL"]) <= 1e-8, r["final"]["E_total"]
        for key in ("E_ECORE", "E_EP", "E_EE", "E_OMG1", "E_OMG2", "E_OMG3", "E_OMG4",
                    "S_TOTAL"):
            assert abs(r["final"][names[key]] - fin[key]) <= 2e-5 * max(1.0, abs(fin[key])), key
        iters[diis] = r["niter"]
    assert iters[True] < iters[False]
