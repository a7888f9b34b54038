"""Shared fixtures.  The CPU oracle (oracle/) is the checker for every
parity test; GPU tests are marked ``gpu`` and call the C-ABI library."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "neo-rxchf_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def orc():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def nx():
    """The GB300 library; skips on machines without a usable GB300."""
    import neoxc
    neoxc.lib(build_if_missing=True)
    if not neoxc.device_ok():
        pytest.skip("no usable GB300: " + neoxc.lib().neoxc_last_error().decode())
    return neoxc


@pytest.fixture(scope="session")
def golden_xchf():
    with open(os.path.join(GOLDEN, "xchf_example.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_xcuhf():
    with open(os.path.join(GOLDEN, "xcuhf_example.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_rx():
    with open(os.path.join(GOLDEN, "rx_examples.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_rx_ref_tests():
    with open(os.path.join(GOLDEN, "rx_ref_tests.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_ref_tests():
    with open(os.path.join(GOLDEN, "ref_tests.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_spot():
    with open(os.path.join(GOLDEN, "spot_check.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def xchf(golden_xchf):
    """examples/xchf as the driver prepares it, plus the densities of the
    initial guess (guessCE.inp, 2 x 2 occupied) and of the converged MOs."""
    from neoxc import basis
    s = basis.parse_inp(golden_xchf["inp"], name="examples/xchf")
    vec0 = basis.read_mo_file(golden_xchf["guessCE"], s.nebf)
    vecf = basis.read_mo_file(golden_xchf["finalCE"], s.nebf)
    vecp = basis.read_mo_file(golden_xchf["finalCP"], s.npbf)
    DE0 = basis.density(vec0, s.nelec // 2, 2.0)
    DEf = basis.density(vecf, s.nelec // 2, 2.0)
    DPf = basis.density(vecp, 1, 1.0)
    DP0 = np.ones((1, 1))  # core-Hamiltonian guess of one normalised function
    return {"sys": s, "DE0": DE0, "DP0": DP0, "DEf": DEf, "DPf": DPf}


class OracleTensors:
    """Lazily computed oracle tensors of one system (cached per session)."""

    def __init__(self, O, s):
        self.O, self.s, self.h = O, s, O.SystemHandle(s)
        self._c = {}

    def get(self, key):
        if key in self._c:
            return self._c[key]
        O, s, L = self.O, self.s, self.O.lib()
        if key == "gee":
            v = np.zeros(s.ngee)
            L.orc_calc_gam_ee(self.h.ref, O.ptr(v))
        elif key in ("g2", "g2s"):
            a, b = np.zeros(s.ng2), np.zeros(s.ng2)
            L.orc_gam2_ic1(self.h.ref, O.ptr(a), O.ptr(b))
            self._c["g2"], self._c["g2s"] = a, b
            return self._c[key]
        elif key in ("rx2", "rx2ex"):
            a, b = np.zeros(s.ng2), np.zeros(s.ng2)
            L.orc_rxchfne_gam2_ic1(self.h.ref, O.ptr(a), O.ptr(b))
            self._c["rx2"], self._c["rx2ex"] = a, b
            return self._c[key]
        elif key == "g3":
            v = np.zeros(s.ng3)
            L.orc_gam3_ic1(self.h.ref, O.ptr(v))
        else:
            raise KeyError(key)
        self._c[key] = v
        return v


@pytest.fixture(scope="session")
def xchf_tensors(orc, xchf):
    return OracleTensors(orc, xchf["sys"])


def fmat(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


def assert_close_scaled(got, ref, rtol, what=""):
    """Element-wise relative check on significant elements plus a check
    against the tensor scale for the rest (cancellation-dominated tiny
    elements carry the absolute error of the large ones)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert got.shape == ref.shape, what
    scale = max(float(np.abs(ref).max()), 1e-300)
    err = np.abs(got - ref)
    big = np.abs(ref) > 1e-6 * scale
    if big.any():
        rel = (err[big] / np.abs(ref[big])).max()
        assert rel <= rtol, "%s: max relative error %.3e > %.1e" % (what, rel, rtol)
    assert err.max() <= rtol * scale, "%s: max error %.3e vs scale %.3e" % (what, err.max(), scale)
