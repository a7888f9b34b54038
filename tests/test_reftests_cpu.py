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


def test_positional_parser_reads_the_decks(golden_ref_tests):
    from neoxc import basis
    for name, g in golden_ref_tests.items():
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
