"""The reference's positional regression decks (tests/golden/ref_tests.json)
on the CPU: every deck parses into the system its log echoes, and the
oracle reproduces the initial-guess energetics of one XCHF run
(tests/TEST_RXCHFmult/RXCHFmult_TEST_03/answer/XCHF.log: He-based, 2
electrons + proton, contracted s/p basis with 11 primitives) from the
core-Hamiltonian guesses (guess_elec, guess_prot), to the log's 10 printed
decimals (6e-11 Eh).
"""
from __future__ import annotations

import re

import numpy as np


def test_positional_parser_reads_the_decks(golden_ref_tests, golden_rx_ref_tests):
    from neoxc import basis
    for name, g in list(golden_ref_tests.items()) + list(golden_rx_ref_tests.items()):
        s, tags = basis.parse_positional_inp(g["inp"], name=name)
        assert s.nebf >= 1 and s.npbf >= 1 and s.ngtg >= 1
        assert int(tags["nelec"]) == s.nelec
        m = re.search(r"^\s*(\d+)\s*=NEBF", g["inp"], re.M)
        assert int(m.group(1)) == s.nebf
        assert s.ggem.shape == (s.ngtg,) and np.all(s.ggem > 0)


def test_oracle_initial_energetics_of_a_reference_run(orc, golden_ref_tests):
    import xchf_scf as X
    from neoxc import basis
    g = golden_ref_tests["xchf_mult03"]
    s, tags = basis.parse_positional_inp(g["inp"], name="xchf_mult03")
    ints = X.XchfIntegrals(s)
    noccE = s.nelec // 2
    DE, _, _ = X.roothan(ints.ecore(), ints.S_e(), noccE, 2.0)          # guess_elec
    DP, _, _ = X.roothan(ints.pcore(), ints.S_p(), 1, 1.0, s.nucst - 1)  # guess_prot
    r = X.xchf1_fock(ints, DE, DP)
    names = {"E_NUC": "E_nuc", "E_ECORE": "E_ecore", "E_PCORE": "E_pcore", "E_EP": "E_ep",
             "E_EE": "E_ee", "E_GAM1": "E_gam1", "E_GAM2": "E_gam2", "S_TOTAL": "S_total",
             "E_TOTAL": "E_total"}
    for k, mine in names.items():
        assert abs(r[mine] - g["initial"][k]) <= 6e-11, (k, r[mine], g["initial"][k])


def _true(tag):
    return tag is not None and tag.strip(".").lower().startswith("t")


def rx_case(tags, name):
    """rx_scf arguments of one RX regression deck: RXCHF-ne (NAE closed-shell
    regular electrons) or RXCUHF (NAalpE / NAbetE, EXCHLEV 1 = ae), and the
    LOCBSE switch."""
    ocbse = _true(tags.get("locbse"))
    if name.startswith("rxchf"):
        return "rxchf_ne", dict(nae=int(tags["nae"])), ocbse
    kind = "rxcuhf_ae" if int(tags["exchlev"]) == 1 else "rxcuhf_ne"
    return kind, dict(nalp=int(tags["naalpe"]), nbet=int(tags["nabete"])), ocbse


def test_oracle_rx_reference_runs(orc, golden_rx_ref_tests):
    """tests/TEST_RXCHF/RXCHF_TEST_01 (RXCHF-ne with LOCBSE = .false., the
    plain branch) and tests/TEST_RXCUHF/RXCUHF_TEST_03/rxchf-ae: the oracle
    reaches the READMEs' converged energies (-0.6666367359, -7.4259664751)
    within 1e-9 Eh in their iteration counts (7, 4)."""
    import rxne
    from neoxc import basis
    for name in ("rxchf_t01", "rxcuhf_t03_ae"):
        g = golden_rx_ref_tests[name]
        s, tags = basis.parse_positional_inp(g["inp"], name=name)
        kind, kw, ocbse = rx_case(tags, name)
        if kind == "rxcuhf_ae":
            kw["addexch"] = True
        _, fin, hist, ok = rxne.rx_scf(rxne.RxIntegrals(s), ocbse=ocbse, **kw)
        assert ok and len(hist) == g["iterations"], (name, len(hist))
        assert abs(fin["E_total"] - g["final_energy"]) <= 1e-9, (name, fin["E_total"])
