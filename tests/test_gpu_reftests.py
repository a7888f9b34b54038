"""The device SCFs on the reference's own regression runs (tests/ of the
reference, fixture tests/golden/ref_tests.json), read from their older
positional basis_definition.inp decks (neoxc.basis.parse_positional_inp):

* XCHF RHF (neoxc_xchf_scf) on tests/TEST_RXCHFmult/*/answer: PsH (3-21G and
  6-311G runs, 2 electrons + positron), LiPs (4 electrons, 8 geminal
  terms), RXCHFmult_TEST_03/04/05 (He-based, 2 and 4 electrons, contracted
  s/p basis, 11 primitives), from the core-Hamiltonian guesses; and on
  tests/TEST_XCRHF (TEST_02, 03 with NUCST = 4 and 38 nuclear functions,
  04/TEST_MD, 05 with NUCST = 2, 06, 07, TEST_NUCST), mostly started from
  the runs' guessCE / guessCP files;
* XCUHF (neoxc_xcuhf_scf) on tests/TEST_XCUHF/XCUHF_TEST_0{2,3,4,5}: e+Li
  and LiPs with 1-8 geminal terms, started from the runs' guessCAE /
  guessCBE / guessCP files where the deck sets read_CE / read_CP.  The two
  19-primitive runs (XCUHF_TEST_06, 08) take about a minute each in FP64
  and run only with NEOXC_SLOW=1.

Checks: the initial-guess energy components within 6e-11 Eh + 2e-10 of
their size of the logs' 10 decimals (the relative part covers the geminal
terms whose integrals, with exponents up to ~2000, cancel: XCHF
RXCHFmult_TEST_05's E_GAM2 is -1378 Eh; measured deviations are 9e-11 to
3.5e-10 Eh on such terms, FP64 summation-order differences), and the
converged energy within 1e-8 Eh.  E_GAM4 / E_OMG4 sum ~6e8 signed terms
(ne^8 np^2) and carry 5e-9 of their size (measured 3.5e-10 and 2.2e-9
relative on LiPs with 8 geminal terms).  The reference converged with
second-order SCF steps, the device with Roothaan + DIIS, so the iteration
counts are not compared.  Two runs need the second-order steps themselves
and are solved with NEOXC_SCF_SOSCF: RXCHFmult_TEST_03 (its reference run
wandered, proton density changes up to 292 per iteration, until the
second-order steps brought it to -2.7643081827 after 37 iterations;
Roothaan + DIIS does not settle it within 200) and TEST_XCRHF/TEST_06 (3
contracted electronic functions, 2 occupied: Roothaan + DIIS falls into a
two-cycle between -5.4306 and -5.4164 where the second-order steps reach
-5.4788705945).  TEST_NUCST's log
predates the current GAM_1 for p-type nuclear functions: E_GAM1 and
S_TOTAL carry 2e-8 of their size there (the oracle's restatement of the
current source differs from the log by the same 4.6e-9 and 1.9e-9).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

XCHF_CASES = ("xchf_mult01_321g", "xchf_mult01_6311g", "xchf_mult02_lips", "xchf_mult03",
              "xchf_mult04", "xchf_mult05", "xcrhf_02", "xcrhf_03", "xcrhf_04md", "xcrhf_05",
              "xcrhf_06", "xcrhf_07", "xcrhf_nucst")
XCUHF_CASES = ("xcuhf_02", "xcuhf_03", "xcuhf_04", "xcuhf_05")
XCUHF_SLOW = ("xcuhf_06", "xcuhf_08")
SOSCF_CASES = ("xchf_mult03", "xcrhf_06")
# TEST_NUCST's log predates the current GAM_1 for p-type nuclear functions:
# the oracle's restatement of the current source and the device agree with
# each other and differ from the log by 4.6e-9 (E_GAM1) and 1.9e-9
# (S_TOTAL); every other component matches it
LOG_PREDATES = {"xcrhf_nucst": ("E_GAM1", "S_TOTAL")}
BIG_SUMS = ("E_GAM4", "E_OMG4")


def _tol(k, ref):
    return 6e-11 + (5e-9 if k in BIG_SUMS else 2e-10) * abs(ref)
XCHF_NAMES = {"E_NUC": "E_nuc", "E_ECORE": "E_ecore", "E_PCORE": "E_pcore", "E_EP": "E_ep",
              "E_EE": "E_ee", "E_GAM1": "E_gam1", "E_GAM2": "E_gam2", "E_GAM3": "E_gam3",
              "E_GAM4": "E_gam4", "S_TOTAL": "S_total", "E_TOTAL": "E_total"}
XCUHF_NAMES = {"E_NUC": "E_nuc", "E_ECORE": "E_ecore", "E_PCORE": "E_pcore", "E_EP": "E_ep",
               "E_EE": "E_ee", "E_OMG1": "E_omg1", "E_OMG2": "E_omg2", "E_OMG3": "E_omg3",
               "E_OMG4": "E_omg4", "S_TOTAL": "S_total", "E_TOTAL": "E_total"}


def _true(tag):
    return tag is not None and tag.strip(".").lower().startswith("t")


@pytest.mark.parametrize("name", XCHF_CASES)
def test_xchf_reference_runs(nx, golden_ref_tests, name):
    from neoxc import basis
    g = golden_ref_tests[name]
    s, tags = basis.parse_positional_inp(g["inp"], name=name)
    DE = DP = None
    if _true(tags.get("read_ce")):   # read_elec_density (GAM_IO.f)
        nocc, pref = (s.nelec // 2, 2.0) if s.nelec > 1 else (1, 1.0)
        DE = basis.density(basis.read_mo_file(g["guessCE.inp"], s.nebf), nocc, pref)
    if _true(tags.get("read_cp")):   # read_nuc_density (GAM_IO.f)
        C = basis.read_mo_file(g["guessCP.inp"], s.npbf)
        DP = np.outer(C[:, s.nucst - 1], C[:, s.nucst - 1])
    r = nx.xchf_scf(s, DE, DP, diis=True, maxit=200)
    for k, mine in XCHF_NAMES.items():
        ref = g["initial"][k]
        if k in LOG_PREDATES.get(name, ()):
            assert abs(r["initial"][mine] - ref) <= 2e-8 * abs(ref), (name, k, r["initial"][mine])
            continue
        assert abs(r["initial"][mine] - ref) <= _tol(k, ref), (name, k, r["initial"][mine])
    if name in SOSCF_CASES:
        # the reference's second-order steps (NEOXC_SCF_SOSCF) bring these
        # runs to their logged energies, where Roothaan + DIIS does not settle
        r = nx.xchf_scf(s, DE, DP, soscf=True, maxit=200)
    assert r["converged"], (name, r["history"][-5:])
    assert abs(r["final"]["E_total"] - g["final_energy"]) <= 1e-8, (name, r["final"]["E_total"])


def _xcuhf_case(nx, g, name):
    from neoxc import basis
    s, tags = basis.parse_positional_inp(g["inp"], name=name)
    nae, nbe = int(tags["nae"]), int(tags["nbe"])
    DAE = DBE = DP = None
    if _true(tags.get("read_ce")):   # read_CAE / read_CBE (xcuhf_scf.f:305-309)
        DAE = basis.density(basis.read_mo_file(g["guessCAE.inp"], s.nebf), nae, 1.0)
        DBE = basis.density(basis.read_mo_file(g["guessCBE.inp"], s.nebf), nbe, 1.0)
    if _true(tags.get("read_cp")):   # read_nuc_density (GAM_IO.f)
        C = basis.read_mo_file(g["guessCP.inp"], s.npbf)
        k = s.nucst - 1
        DP = np.outer(C[:, k], C[:, k])
    r = nx.xcuhf_scf(s, nae, nbe, DAE, DBE, DP, diis=True, maxit=200)
    for k, mine in XCUHF_NAMES.items():
        ref = g["initial"][k]
        assert abs(r["initial"][mine] - ref) <= _tol(k, ref), (name, k, r["initial"][mine])
    assert r["converged"], name
    assert abs(r["final"]["E_total"] - g["final_energy"]) <= 1e-8, (name, r["final"]["E_total"])


@pytest.mark.parametrize("name", XCUHF_CASES)
def test_xcuhf_reference_runs(nx, golden_ref_tests, name):
    _xcuhf_case(nx, golden_ref_tests[name], name)


@pytest.mark.skipif(os.environ.get("NEOXC_SLOW") != "1", reason="about a minute each in FP64")
@pytest.mark.parametrize("name", XCUHF_SLOW)
def test_xcuhf_reference_runs_large(nx, golden_ref_tests, name):
    _xcuhf_case(nx, golden_ref_tests[name], name)


RX_CASES = ("rxchf_t01", "rxchf_t02", "rxcuhf_t01_ae", "rxcuhf_t01_ne", "rxcuhf_t02_ae",
            "rxcuhf_t03_ae", "rxcuhf_t04", "rxcuhf_t05", "rxcuhf_t06")


@pytest.mark.parametrize("name", RX_CASES)
def test_rx_reference_runs(nx, golden_rx_ref_tests, name):
    """neoxc_rx_scf on tests/TEST_RXCHF and tests/TEST_RXCUHF decks
    (RXCHF-ne, RXCUHF-ne, RXCUHF-ae, with and without LOCBSE): the READMEs'
    converged energies within 1e-8 Eh (the README prints 10 decimals; the
    second-order steps of the reference's regular-electron updates are not
    ported, so only the energy is compared)."""
    from neoxc import basis
    from test_reftests_cpu import rx_case
    g = golden_rx_ref_tests[name]
    s, tags = basis.parse_positional_inp(g["inp"], name=name)
    kind, kw, ocbse = rx_case(tags, name)
    r = nx.rx_scf(s, kind, ocbse=ocbse, **kw)
    assert r["converged"], (name, r["history"][-3:])
    assert abs(r["final"]["E_total"] - g["final_energy"]) <= 1e-8, (name, r["final"]["E_total"])
