"""Generate the golden fixtures of the parity tests from the reference tree.

Run where the reference tree is available (it reads files only), giving
the tree's root as the one required argument:

    python tests/golden/make_golden.py <path-to-NEO-RXCHF>

Writes, next to this script:
  xchf_example.json   examples/xchf: input deck, initial MO guess
                      (guessCE.inp), converged MOs (answer/FinalC*.dat) and
                      the energy components printed in answer/XCHF.log for
                      the initial guess and at convergence, and the
                      orbital energies printed there;
  xcuhf_example.json  examples/xcuhf: input deck (core-Hamiltonian guess),
                      converged MOs (answer/FinalC{AE,BE,P}.dat) and the
                      energy components of answer/XCUHF.log for the initial
                      guess and at convergence;
  rx_examples.json    examples/rxchf/one_special_electron (RXCHF-ne) and
                      examples/rxcuhf/rxchf-{ne,ae} (RXCUHF, EXCHLEV 0 / 1):
                      input decks and the energy components of their logs
                      for the initial guess and at convergence;
  ref_tests.json      tests/TEST_RXCHFmult/*/answer and tests/TEST_XCRHF
                      (XCHF RHF runs) and tests/TEST_XCUHF/XCUHF_TEST_0{2..6,8}
                      (XCUHF runs):
                      the positional input decks, the MO guess files the
                      read_CE runs start from, and the energy components of
                      their logs for the initial guess and at convergence;
  rx_ref_tests.json   tests/TEST_RXCHF and tests/TEST_RXCUHF one-special-
                      electron decks (RXCHF-ne, RXCUHF-ne / -ae) with the
                      converged energies and iteration counts their READMEs
                      record;
  spot_check.json     CS_Integrals/Spot_Check/TEST_G{2,3,4}: the single-
                      primitive inputs (first record block, as SCI.f:114-152
                      reads them) and the MD values printed in each ``out``.
Nothing at test time reads the reference tree; the tests use these files.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


XCHF_KEYS = ("E_NUC", "E_ECORE", "E_PCORE", "E_EP", "E_EE", "E_GAM1", "E_GAM2",
             "E_GAM3", "E_GAM4", "S_TOTAL", "E_TOTAL")
XCUHF_KEYS = ("E_NUC", "E_ECORE", "E_PCORE", "E_EP", "E_EE", "E_OMG1", "E_OMG2",
              "E_OMG3", "E_OMG4", "S_TOTAL", "E_TOTAL")


def _components(log: str, header: str, keys=XCHF_KEYS) -> dict:
    i = log.index(header)
    block = log[i:i + 2500]
    out = {}
    for key in keys:
        m = re.search(r"\b" + key + r"=\s*(-?[0-9.]+)", block)
        out[key] = float(m.group(1))
    return out


def _eigenvalues(log: str, header: str, end: str) -> list:
    """Orbital energies of PREVNU's table (4 decimals): the rows between the
    column-number rows and the coefficient rows (those carry LABEL)."""
    i = log.index(header)
    block = log[i + len(header):log.index(end, i)]
    vals = []
    for line in block.splitlines():
        toks = line.split()
        if toks and "LABEL" not in line and all("." in t for t in toks):
            vals += [float(t) for t in toks]
    return vals


def xchf_example(ref: str) -> dict:
    d = os.path.join(ref, "examples", "xchf")
    log = open(os.path.join(d, "answer", "XCHF.log")).read()
    return {
        "source": "examples/xchf (exam_xchf.inp, guessCE.inp, answer/)",
        "inp": open(os.path.join(d, "exam_xchf.inp")).read(),
        "guessCE": open(os.path.join(d, "guessCE.inp")).read(),
        "finalCE": open(os.path.join(d, "answer", "FinalCE.dat")).read(),
        "finalCP": open(os.path.join(d, "answer", "FinalCP.dat")).read(),
        "initial": _components(log, "INITIAL GUESS ENERGETICS"),
        "final": _components(log, "FINAL NEOXCHF ENERGY"),
        "orbital_energies": {
            "electronic": _eigenvalues(log, "ELECTRONIC ORBITALS AND EIGENVALUES:",
                                       "NUCLEAR ORBITALS AND EIGENVALUES:"),
            "nuclear": _eigenvalues(log, "NUCLEAR ORBITALS AND EIGENVALUES:",
                                    "TIMING SUMMARY")},
        "log_lines": {"initial": "XCHF.log:306-321", "final": "XCHF.log:335-350",
                      "orbital_energies": "XCHF.log:353-384"},
    }


def xcuhf_example(ref: str) -> dict:
    d = os.path.join(ref, "examples", "xcuhf")
    log = open(os.path.join(d, "answer", "XCUHF.log")).read()
    ans = os.path.join(d, "answer")
    return {
        "source": "examples/xcuhf (exam_xcuhf.inp, answer/)",
        "inp": open(os.path.join(d, "exam_xcuhf.inp")).read(),
        "finalCAE": open(os.path.join(ans, "FinalCAE.dat")).read(),
        "finalCBE": open(os.path.join(ans, "FinalCBE.dat")).read(),
        "finalCP": open(os.path.join(ans, "FinalCP.dat")).read(),
        "initial": _components(log, "INITIAL GUESS ENERGETICS", XCUHF_KEYS),
        "final": _components(log, "FINAL NEOXCHF ENERGY", XCUHF_KEYS),
        "log_lines": {"initial": "XCUHF.log:337-352", "final": "XCUHF.log:366-381"},
    }


RX_KEYS = ("E_NUC", "E_ECORE", "E_EE", "E_OMG1", "E_OMG2", "S_TOTAL", "E_TOTAL")
RX_EXAMPLES = {   # name: (directory under examples/, input deck, log)
    "rxchf_ne": ("rxchf/one_special_electron", "exam_rxchf.inp", "RXCHF.log"),
    "rxcuhf_ne": ("rxcuhf/rxchf-ne", "exam_rxcuhfne.inp", "RXCHF-ne.log"),
    "rxcuhf_ae": ("rxcuhf/rxchf-ae", "exam_rxcuhfae.inp", "RXCHF-ae.log"),
}


def rx_examples(ref: str) -> dict:
    out = {}
    for name, (sub, inp, logname) in RX_EXAMPLES.items():
        d = os.path.join(ref, "examples", sub)
        log = open(os.path.join(d, "answer", logname)).read()
        m = re.search(r"FINAL NEORX\w* ENERGY IS\s+(-?[0-9.]+)\s+AFTER\s+(\d+)", log)
        out[name] = {
            "source": "examples/%s/%s, answer/%s" % (sub, inp, logname),
            "inp": open(os.path.join(d, inp)).read(),
            "initial": _components(log, "INITIAL GUESS ENERGETICS", RX_KEYS),
            "final": _components(log, m.group(0), RX_KEYS),
            "final_energy": float(m.group(1)),
            "iterations": int(m.group(2)),
        }
    return out


REF_TESTS = {   # name: (directory under tests/, log, kind)
    "xchf_mult01_321g": ("TEST_RXCHFmult/RXCHFmult_TEST_01/3-21G/answer/PsH", "XCHF.log", "xchf"),
    "xchf_mult01_6311g": ("TEST_RXCHFmult/RXCHFmult_TEST_01/6-311G/answer/PsH", "XCHF.log",
                          "xchf"),
    "xchf_mult02_lips": ("TEST_RXCHFmult/RXCHFmult_TEST_02/answer/LiPs_xchf", "XCHF.log", "xchf"),
    "xchf_mult03": ("TEST_RXCHFmult/RXCHFmult_TEST_03/answer", "XCHF.log", "xchf"),
    "xchf_mult04": ("TEST_RXCHFmult/RXCHFmult_TEST_04/answer", "XCHF.log", "xchf"),
    "xchf_mult05": ("TEST_RXCHFmult/RXCHFmult_TEST_05/answer", "XCHF.log", "xchf"),
    "xcrhf_02": ("TEST_XCRHF/TEST_02", "xcOMP_MD_out.log", "xchf"),
    "xcrhf_03": ("TEST_XCRHF/TEST_03", "xcOMP_MD_out.log_ST4", "xchf"),
    "xcrhf_04md": ("TEST_XCRHF/TEST_04/TEST_MD", "xcOMP_MD_out.log", "xchf"),
    "xcrhf_05": ("TEST_XCRHF/TEST_05", "xcOMP_MD_out.log", "xchf"),
    "xcrhf_06": ("TEST_XCRHF/TEST_06", "xcOMP_MD_out.log", "xchf"),
    "xcrhf_07": ("TEST_XCRHF/TEST_07", "xcOMP_MD_out.log", "xchf"),
    "xcrhf_nucst": ("TEST_XCRHF/TEST_NUCST", "xcOMP_MD_out.log", "xchf"),
    "xcuhf_02": ("TEST_XCUHF/XCUHF_TEST_02", "answer/xcOMPout.log", "xcuhf"),
    "xcuhf_03": ("TEST_XCUHF/XCUHF_TEST_03", "answer/xcOMPout.log", "xcuhf"),
    "xcuhf_04": ("TEST_XCUHF/XCUHF_TEST_04", "answer/xcOMPout.log", "xcuhf"),
    "xcuhf_05": ("TEST_XCUHF/XCUHF_TEST_05", "answer/xcOMPout.log", "xcuhf"),
    "xcuhf_06": ("TEST_XCUHF/XCUHF_TEST_06", "answer/xcOMPout.log", "xcuhf"),
    "xcuhf_08": ("TEST_XCUHF/XCUHF_TEST_08", "answer/xcOMPout.log", "xcuhf"),
}


# one-special-electron RX decks and the README line that records each
# run's converged energy: name -> (deck directory, README, section, label)
RX_REF_TESTS = {
    "rxchf_t01": ("TEST_RXCHF/RXCHF_TEST_01", "TEST_RXCHF/README", "TEST01", "RXCHF:"),
    "rxchf_t02": ("TEST_RXCHF/RXCHF_TEST_02", "TEST_RXCHF/README", "TEST02", "RXCHF:"),
    "rxcuhf_t01_ae": ("TEST_RXCUHF/RXCUHF_TEST_01/rxchf-ae", "TEST_RXCUHF/README", "TEST01",
                      "RXCHF-ae:"),
    "rxcuhf_t01_ne": ("TEST_RXCUHF/RXCUHF_TEST_01/rxchf-ne", "TEST_RXCUHF/README", "TEST01",
                      "RXCHF-ne:"),
    "rxcuhf_t02_ae": ("TEST_RXCUHF/RXCUHF_TEST_02/rxchf-ae", "TEST_RXCUHF/README", "TEST02",
                      "RXCHF-ae:"),
    "rxcuhf_t03_ae": ("TEST_RXCUHF/RXCUHF_TEST_03/rxchf-ae", "TEST_RXCUHF/README", "TEST03",
                      "RXCHF-ae:"),
    "rxcuhf_t04": ("TEST_RXCUHF/RXCUHF_TEST_04", "TEST_RXCUHF/README", "TEST04", "RXCUHF:"),
    "rxcuhf_t05": ("TEST_RXCUHF/RXCUHF_TEST_05", "TEST_RXCUHF/README", "TEST05", "RXCHF:"),
    "rxcuhf_t06": ("TEST_RXCUHF/RXCUHF_TEST_06", "TEST_RXCUHF/README", "TEST06", "RXCHF:"),
}


def rx_ref_tests(ref: str) -> dict:
    out = {}
    for name, (sub, readme, section, label) in RX_REF_TESTS.items():
        text = open(os.path.join(ref, "tests", readme)).read()
        i = text.index("\n" + section + "\n")
        j = text.find("======\n" + "TEST", i + len(section) + 10)
        block = text[i:j if j > 0 else len(text)]
        m = re.search(re.escape(label) + r"\s+FINAL NEO\w* ENERGY IS\s+(-?[0-9.]+)\s+AFTER\s+"
                      r"(\d+)", block)
        out[name] = {"source": "tests/%s/basis_definition.inp, tests/%s %s %s" % (
                         sub, readme, section, label),
                     "inp": open(os.path.join(ref, "tests", sub, "basis_definition.inp")).read(),
                     "final_energy": float(m.group(1)), "iterations": int(m.group(2))}
    return out


def ref_tests(ref: str) -> dict:
    out = {}
    for name, (sub, logname, kind) in REF_TESTS.items():
        d = os.path.join(ref, "tests", sub)
        log = open(os.path.join(d, logname)).read()
        keys = XCHF_KEYS if kind == "xchf" else XCUHF_KEYS
        m = re.search(r"FINAL NEO\w* ENERGY IS\s+(-?[0-9.]+)\s+AFTER\s+(\d+)", log)
        entry = {"source": "tests/%s/basis_definition.inp, %s" % (sub, logname), "kind": kind,
                 "inp": open(os.path.join(d, "basis_definition.inp")).read(),
                 "initial": _components(log, "INITIAL GUESS ENERGETICS", keys),
                 "final": _components(log, m.group(0), keys),
                 "final_energy": float(m.group(1)), "iterations": int(m.group(2))}
        for g in ("guessCE.inp", "guessCP.inp", "guessCAE.inp", "guessCBE.inp"):
            if os.path.exists(os.path.join(d, g)):
                entry[g] = open(os.path.join(d, g)).read()
        out[name] = entry
    return out


def _first_block(path: str):
    rows = [l.split() for l in open(path).read().splitlines()]
    k = 0
    g1 = float(rows[k][0]); k += 1
    g2 = float(rows[k][0]); k += 1
    nbra = int(rows[k][0]); k += 1
    bra = [[float(x) for x in rows[k + i][:7]] for i in range(nbra)]; k += nbra
    nket = int(rows[k][0]); k += 1
    ket = [[float(x) for x in rows[k + i][:7]] for i in range(nket)]; k += nket
    cmat = [float(x) for x in rows[k][:3]]; k += 1
    znuc = float(rows[k][0])
    return {"gamma1": g1, "gamma2": g2, "bra": bra, "ket": ket, "C": cmat, "Z": znuc}


def _md_values(out: str) -> dict:
    i = out.index("MD VALUES")
    j = out.find("VALUES", i + 10)
    block = out[i:j if j > 0 else len(out)]
    vals = {}
    for m in re.finditer(r"^\s*([A-Za-z0-9]+)\s*=\s*(-?[0-9.]+(?:E[-+][0-9]+)?)\s*$", block, re.M):
        vals[m.group(1)] = float(m.group(2))
    return vals


def spot_check(ref: str) -> dict:
    base = os.path.join(ref, "source", "CS_Integrals", "Spot_Check")
    res = {}
    for t in ("TEST_G2", "TEST_G3", "TEST_G4"):
        d = os.path.join(base, t)
        res[t] = {"input": _first_block(os.path.join(d, "basis_definition.inp")),
                  "md": _md_values(open(os.path.join(d, "out")).read()),
                  "source": "source/CS_Integrals/Spot_Check/%s/{basis_definition.inp,out}" % t}
    return res


def main(ref: str):
    with open(os.path.join(HERE, "xchf_example.json"), "w") as f:
        json.dump(xchf_example(ref), f, indent=1)
    with open(os.path.join(HERE, "xcuhf_example.json"), "w") as f:
        json.dump(xcuhf_example(ref), f, indent=1)
    with open(os.path.join(HERE, "spot_check.json"), "w") as f:
        json.dump(spot_check(ref), f, indent=1)
    with open(os.path.join(HERE, "rx_examples.json"), "w") as f:
        json.dump(rx_examples(ref), f, indent=1)
    with open(os.path.join(HERE, "ref_tests.json"), "w") as f:
        json.dump(ref_tests(ref), f, indent=1)
    with open(os.path.join(HERE, "rx_ref_tests.json"), "w") as f:
        json.dump(rx_ref_tests(ref), f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path-to-NEO-RXCHF>")
    main(sys.argv[1])
