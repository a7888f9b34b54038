"""GPU XCHF RHF SCF (neoxc_xchf_scf) against the reference's example log and
the oracle's restatement of xcscf.f.

Tolerances: initial energetics within 6e-11 Eh of XCHF.log's 10 printed
decimals (the integrals are FP64 to ~1e-12 relative); per-iteration total
energies within 1e-9 of the oracle's Roothaan sequence; converged total
energy within 1e-9 Eh of XCHF.log.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOG_NAMES = {"E_NUC": "E_nuc", "E_ECORE": "E_ecore", "E_PCORE": "E_pcore", "E_EP": "E_ep",
             "E_EE": "E_ee", "E_GAM1": "E_gam1", "E_GAM2": "E_gam2", "E_GAM3": "E_gam3",
             "E_GAM4": "E_gam4", "S_TOTAL": "S_total", "E_TOTAL": "E_total"}


@pytest.fixture(scope="module")
def xchf_gpu_scf(nx, xchf):
    return nx.xchf_scf(xchf["sys"], xchf["DE0"])


def test_xchf_example_initial_energetics(xchf_gpu_scf, golden_xchf):
    """First Fock build at guessCE + guess_prot: XCHF.log:306-321."""
    init = xchf_gpu_scf["initial"]
    for k, mine in LOG_NAMES.items():
        assert abs(init[mine] - golden_xchf["initial"][k]) <= 6e-11, (k, init[mine])


def test_xchf_example_converges_to_log_energy(xchf_gpu_scf, golden_xchf):
    """The device SCF reaches XCHF.log:335 (-5.7800665094)."""
    r = xchf_gpu_scf
    assert r["converged"]
    assert abs(r["final"]["E_total"] - golden_xchf["final"]["E_TOTAL"]) <= 1e-9
    # iteration 2 precedes the reference's first SOSCF step: same value
    assert abs(r["history"][1, 0] - (-5.7737887409)) <= 6e-11
    # converged components agree with the log's to the density tolerance
    for k in ("E_ECORE", "E_EP", "E_EE", "E_GAM1", "E_GAM2", "E_GAM3", "E_GAM4", "S_TOTAL"):
        ref = golden_xchf["final"][k]
        assert abs(r["final"][LOG_NAMES[k]] - ref) <= 1e-5 * max(1.0, abs(ref)), k


def test_xchf_example_matches_oracle_iterations(xchf_gpu_scf, xchf):
    """Same Roothaan sequence as the oracle's xcscf restatement."""
    import xchf_scf as X
    ints = X.XchfIntegrals(xchf["sys"])
    hist, r, DE, DP, ok = X.xchf_scf(ints, xchf["DE0"])
    its = hist[1:]
    g = xchf_gpu_scf["history"]
    assert ok and xchf_gpu_scf["niter"] == len(its)
    for k, (it, E, dE, dP) in enumerate(its):
        assert abs(g[k, 0] - E) <= 1e-9, (it, g[k, 0], E)
    assert np.abs(xchf_gpu_scf["DE"] - DE).max() <= 1e-7


def test_scf_gam4_paths_agree(nx, xchf, xchf_gpu_scf):
    """The element-wise GAM4_DSCF inside the SCF gives the same run as the
    factorised build."""
    r = nx.xchf_scf(xchf["sys"], xchf["DE0"], gam4_element=True)
    assert r["niter"] == xchf_gpu_scf["niter"]
    assert abs(r["final"]["E_total"] - xchf_gpu_scf["final"]["E_total"]) <= 1e-10


@pytest.mark.parametrize("kw", [
    dict(seed=301, nat=2, nebf=3, nprim=2, npbf=2, ngtg=2, lmax_e=1, lmax_p=1, nelec=4),
    dict(seed=302, nat=3, nebf=4, nprim=1, npbf=3, ngtg=3, lmax_e=1, lmax_p=1, nelec=2),
])
def test_synthetic_scf_matches_oracle(nx, orc, kw):
    """Seeded synthetic systems (npbf > 1, so the nuclear density is solved
    too): initial energetics within 1e-10 relative, the same iteration count
    and final energy within 1e-9 of the oracle's SCF."""
    import xchf_scf as X
    from neoxc import basis
    s = basis.synthetic(**kw)
    rng = np.random.default_rng(kw["seed"])
    C = rng.standard_normal((s.nebf, s.nebf))
    DE = basis.density(C, max(1, s.nelec // 2), 2.0 if s.nelec > 1 else 1.0)
    g = nx.xchf_scf(s, DE, maxit=60)
    ints = X.XchfIntegrals(s)
    hist, r, DEo, DPo, ok = X.xchf_scf(ints, DE, maxit=60)
    init = hist[0][1]
    for k in ("E_nuc", "E_ecore", "E_pcore", "E_ep", "E_ee", "E_gam1", "E_gam2", "E_gam3",
              "E_gam4", "S_total", "E_total"):
        assert g["initial"][k] == pytest.approx(init[k], rel=1e-10, abs=1e-12), k
    assert g["converged"] == ok
    if ok:
        assert g["niter"] == len(hist) - 1
        assert abs(g["final"]["E_total"] - r["E_total"]) <= 1e-9


# examples/xchf/answer/XCHF.log:325-333: the reference's iteration energies
# with its second-order steps (LSOSCF), iteration 1 .. 8
XCHF_LOG_ITERATIONS = (-5.7303165793, -5.7737887409, -5.7779417176, -5.7800627999,
                       -5.7800664080, -5.7800665092, -5.7800665094, -5.7800665094)


def test_soscf_reproduces_reference_iterations(nx, xchf, golden_xchf):
    """With the second-order steps (soscf.f SOGRAD / SOHESS / SONEWT /
    SOTRAN, driven as xcscf.f:459-485) the device SCF follows the
    reference's own iteration sequence: the same 8 iterations and every
    printed energy of XCHF.log:325-333 to 1e-8 Eh."""
    r = nx.xchf_scf(xchf["sys"], xchf["DE0"], soscf=True)
    assert r["converged"] and r["niter"] == len(XCHF_LOG_ITERATIONS), r["niter"]
    for k, E in enumerate(XCHF_LOG_ITERATIONS):
        assert abs(r["history"][k, 0] - E) <= 1e-8, (k + 1, r["history"][k, 0], E)
    assert abs(r["final"]["E_total"] - golden_xchf["final"]["E_TOTAL"]) <= 1e-9


def test_diis_converges_to_same_state_faster(nx, xchf, xchf_gpu_scf, golden_xchf):
    """Pulay DIIS on the electronic Fock matrix (no reference counterpart):
    same converged energy, fewer iterations than plain Roothaan."""
    r = nx.xchf_scf(xchf["sys"], xchf["DE0"], diis=True)
    assert r["converged"]
    assert r["niter"] < xchf_gpu_scf["niter"]
    assert abs(r["final"]["E_total"] - golden_xchf["final"]["E_TOTAL"]) <= 1e-9
    assert abs(r["final"]["E_total"] - xchf_gpu_scf["final"]["E_total"]) <= 1e-9
    assert np.abs(r["DE"] - xchf_gpu_scf["DE"]).max() <= 1e-5


def test_mixed_precision_gam3_energy_error(nx, xchf, xchf_gpu_scf):
    """FP32 MD for the gam_3 integrals (FP64 Boys and sums): the converged
    total energy stays within 1 microhartree of the FP64 path."""
    r = nx.xchf_scf(xchf["sys"], xchf["DE0"], mixed="gam3")
    assert r["converged"]
    err = r["final"]["E_total"] - xchf_gpu_scf["final"]["E_total"]
    print("mixed-precision (gam_3) E error (Eh):", err)
    assert abs(err) <= 1e-6


def test_mixed_precision_all_geminal_energy_error(nx, xchf, xchf_gpu_scf):
    """FP32 MD for gam_1, gam_2 and gam_3 (FP64 sums), with DIIS: the
    converged total energy is within 1 microhartree of the FP64 path."""
    r = nx.xchf_scf(xchf["sys"], xchf["DE0"], mixed=True, diis=True)
    assert r["converged"]
    err = r["final"]["E_total"] - xchf_gpu_scf["final"]["E_total"]
    print("mixed-precision (gam_1 + gam_2 + gam_3) E error (Eh):", err)
    assert abs(err) <= 1e-6


# A reduced copy of the first configuration's seeded system: the same
# generator (3 nuclei, s/p electronic shells of 3 primitives with exponents
# in [0.1, 20], even-tempered s/p/d nuclear basis, NG = 3) at nebf = 6,
# npbf = 4, so that both solves take seconds.
SPD_SYSTEM = dict(seed=2024, nat=3, nebf=6, nprim=3, npbf=4, ngtg=3, lmax_e=1, lmax_p=2)


def test_mixed_precision_spd_energy_error(nx):
    """On an s/p electronic, s/p/d nuclear system the mixed path (FP32
    McMurchie-Davidson tables for gam_1, gam_2 and gam_3, FP64 Boys function,
    seeds, sums, Fock assembly and diagonalisation) converges within 1
    microhartree of the FP64 path."""
    from neoxc import basis
    s = basis.synthetic(**SPD_SYSTEM)
    a = nx.xchf_scf(s, None, diis=True)
    b = nx.xchf_scf(s, None, diis=True, mixed=True)
    assert a["converged"] and b["converged"]
    err = b["final"]["E_total"] - a["final"]["E_total"]
    print("mixed-precision s/p/d E error (Eh):", err, "E:", a["final"]["E_total"])
    assert abs(err) <= 1e-6


def test_mixed_gam2_dynamic_precision(nx):
    """The mixed gam_2 build re-evaluates in FP64 every primitive item whose
    FP32 contribution exceeds the threshold: at threshold 0 every item is
    FP64 and the first-iteration energy equals the FP64 path's to rounding;
    at the default threshold the FP32 error left is at most half that of
    the all-FP32 build (threshold infinity)."""
    from neoxc import basis
    s = basis.synthetic(**SPD_SYSTEM)
    ref = nx.xchf_scf(s, None, maxit=1)["initial"]["E_total"]
    old = nx.get_mixed_threshold()
    try:
        nx.set_mixed_threshold(0.0)
        e_all64 = nx.xchf_scf(s, None, maxit=1, mixed="gam2")["initial"]["E_total"]
        nx.set_mixed_threshold(float("inf"))
        e_all32 = nx.xchf_scf(s, None, maxit=1, mixed="gam2")["initial"]["E_total"]
    finally:
        nx.set_mixed_threshold(old)
    e_dyn = nx.xchf_scf(s, None, maxit=1, mixed="gam2")["initial"]["E_total"]
    print("gam_2 E error all-FP32 %.3e dynamic %.3e all-FP64 %.3e"
          % (e_all32 - ref, e_dyn - ref, e_all64 - ref))
    assert abs(e_all64 - ref) <= 1e-11
    assert abs(e_dyn - ref) <= max(0.5 * abs(e_all32 - ref), 1e-10)


def test_screened_scf_matches_unscreened(nx):
    """Schwarz-type screening at 1e-12 (NEOXC_SCF_SCREEN) moves the
    converged energy of the s/p/d system by less than 1e-8 Eh."""
    from neoxc import basis
    s = basis.synthetic(**SPD_SYSTEM)
    a = nx.xchf_scf(s, None, diis=True)
    b = nx.xchf_scf(s, None, diis=True, screen=True)
    assert a["converged"] and b["converged"]
    assert abs(b["final"]["E_total"] - a["final"]["E_total"]) <= 1e-8


def test_batch_matches_separate_solves(nx, xchf):
    """A proton-position scan of examples/xchf run as one batch on three
    worker streams gives, job by job, exactly the result of a separate
    neoxc_xchf_scf call (same kernels, same order on each stream)."""
    from neoxc import basis
    systems = basis.proton_scan(xchf["sys"], 5, 0.3, seed=7)
    DEs = [xchf["DE0"]] * len(systems)
    batch = nx.xchf_scf_batch(systems, DEs, nworkers=3, diis=True, mixed=True)
    for s, b in zip(systems, batch):
        a = nx.xchf_scf(s, xchf["DE0"], diis=True, mixed=True)
        assert b["converged"] and a["converged"]
        assert b["niter"] == a["niter"]
        assert b["final"]["E_total"] == a["final"]["E_total"]
        assert np.array_equal(b["DE"], a["DE"])
    # displacing the proton changes the energy
    Es = [b["final"]["E_total"] for b in batch]
    assert max(Es) - min(Es) > 1e-4


def test_server_requests_match_separate_solves(nx, xchf):
    """Continuous batching: requests submitted while others run (3 worker
    streams) finish with exactly the separate-solve results, and each
    request's timestamps are ordered."""
    import time
    from neoxc import basis
    systems = basis.proton_scan(xchf["sys"], 6, 0.3, seed=9)
    srv = nx.XchfServer(nworkers=3, diis=True, mixed=True)
    try:
        tickets = []
        for s in systems:
            tickets.append(srv.submit(s, xchf["DE0"]))
            time.sleep(0.01)
        results = [srv.wait(t) for t in tickets]
    finally:
        srv.stop()
    for s, r in zip(systems, results):
        a = nx.xchf_scf(s, xchf["DE0"], diis=True, mixed=True)
        assert r["converged"] and r["final"]["E_total"] == a["final"]["E_total"]
        assert r["t_submit"] <= r["t_start"] <= r["t_end"]


def test_server_failure_modes(nx, xchf):
    """Failures made on the host, reported per request while the other
    requests go on: a request whose start density holds a NaN ends with
    NEOXC_ERR_NUMERIC; with the server's budget capped below a request's
    footprint the request is refused with NEOXC_ERR_NOMEM without starting;
    a wait that runs out returns NEOXC_ERR_TIMEOUT and the request still
    completes; a request that reaches maxit ends with status 0 and
    converged = False."""
    DE0 = xchf["DE0"]
    bad = np.array(DE0, copy=True)
    bad[1, 2] = np.nan
    srv = nx.XchfServer(nworkers=1, diis=True, mixed=False)
    try:
        t_ok = srv.submit(xchf["sys"], DE0)
        with pytest.raises(nx.NeoxcError, match="error 6"):
            srv.wait(t_ok, timeout=0.0)          # still queued or running
        r_ok = srv.wait(t_ok)
        assert r_ok["status"] == 0 and r_ok["converged"]
        r_nan = srv.wait(srv.submit(xchf["sys"], bad), raise_on_error=False)
        assert r_nan["status"] == nx.ERR_NUMERIC
        srv.set_budget(1 << 20)                  # 1 MiB: below any XCHF footprint
        r_big = srv.wait(srv.submit(xchf["sys"], DE0), raise_on_error=False)
        assert r_big["status"] == nx.ERR_NOMEM and r_big["t_start"] == r_big["t_end"]
        srv.set_budget(0)
        r_again = srv.wait(srv.submit(xchf["sys"], DE0))
        assert r_again["final"]["E_total"] == r_ok["final"]["E_total"]
    finally:
        srv.stop()
    srv = nx.XchfServer(nworkers=1, maxit=2, diis=False, mixed=False)
    try:
        r = srv.wait(srv.submit(xchf["sys"], DE0))
    finally:
        srv.stop()
    assert r["status"] == 0 and not r["converged"] and r["niter"] == 2


def test_xchf_scf_job_returns_final_mos(nx, xchf, xchf_gpu_scf, tmp_path):
    """neoxc_xchf_scf_job: the same solve as neoxc_xchf_scf plus the final
    MOs and orbital energies.  C^T S C = 1; the occupied MOs rebuild the
    returned density; the orbital energies are the oracle's converged ones
    (its last ROOTHAN) to 1e-7; the occupied space matches the reference's
    answer/FinalC{E,P}.dat to the density tolerance; FinalCE.dat written from
    the MOs reads back to its 8 printed digits."""
    import xchf_scf as X
    from neoxc import formats as F
    s = xchf["sys"]
    r = nx.xchf_scf_job(s, xchf["DE0"])
    assert r["converged"] and r["niter"] == xchf_gpu_scf["niter"]
    assert abs(r["final"]["E_total"] - xchf_gpu_scf["final"]["E_total"]) <= 1e-12
    ints = X.XchfIntegrals(s)
    orb = []
    X.xchf_scf(ints, xchf["DE0"], orbitals=orb)
    CE, CP = r["CE"], r["CP"]
    assert np.abs(CE.T @ ints.S_e() @ CE - np.eye(s.nebf)).max() <= 1e-10
    assert np.abs(CP.T @ ints.S_p() @ CP - np.eye(s.npbf)).max() <= 1e-10
    assert np.all(np.diff(r["EE"]) >= 0)
    assert np.abs(r["EE"] - orb[-1][1]).max() <= 1e-7, (r["EE"], orb[-1][1])
    assert np.abs(r["EP"] - orb[-1][2]).max() <= 1e-7
    nocc = s.nelec // 2
    DE = F.mo_density(CE, 1, nocc, 2.0)
    assert np.abs(DE - r["DE"]).max() <= 1e-12
    assert np.abs(F.mo_density(CP, s.nucst, s.nucst, 1.0) - r["DP"]).max() <= 1e-12
    dmax = np.abs(DE - xchf["DEf"]).max()
    assert dmax <= 1e-5, dmax
    assert np.abs(r["DP"] - xchf["DPf"]).max() <= 1e-7
    out = tmp_path / "FinalCE.dat"
    F.write_mos(out, CE)
    assert np.abs(F.read_mos(out, s.nebf) - CE).max() <= 5e-9 * max(1.0, np.abs(CE).max())
