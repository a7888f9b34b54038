"""The allocation-free gam_4 direct-SCF entry point.

neoxc_dev_gam4_dscf_noalloc serves callers that cannot allocate device
memory during a Fock build (all of it handed to their own pool allocator, or
a strict memory budget where a transient allocation could fail in the middle
of an SCF iteration).  It keeps its scratch in an array
built into the library; these tests call it through the C-ABI twice in a
row with different inputs and compare each result with the allocating entry
point neoxc_dev_gam4_dscf, and check that a system too large for the
built-in array is refused with an error.  The file name sorts last so a run
that stops at the first failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def _inputs(torch, dev, ne, np_, seed):
    from neoxc import basis
    rng = np.random.default_rng(seed)
    f64 = torch.float64
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=f64, device=dev)  # noqa: E731
    gee = t(rng.standard_normal(ne ** 4))
    g2s = t(rng.standard_normal(ne ** 4 * np_ ** 2))
    DE = t(basis.random_density(ne, 2, seed + 1).ravel(order="F"))
    DP = t(basis.random_density(np_, 1, seed + 2, 1.0).ravel(order="F"))
    return gee, g2s, DE, DP


def _call(fn, torch, dev, stream, ne, np_, ins):
    f64 = torch.float64
    fe = torch.zeros(ne * ne, dtype=f64, device=dev)
    fp = torch.zeros(np_ * np_, dtype=f64, device=dev)
    E = torch.zeros(1, dtype=f64, device=dev)
    ptrs = [C.c_void_p(x.data_ptr()) for x in (*ins, fe, fp, E)]
    rc = fn(C.c_void_p(stream), ne, np_, *ptrs)
    torch.cuda.synchronize(dev)
    return rc, fe.cpu().numpy(), fp.cpu().numpy(), float(E.item())


def _close(a, b):
    scale = max(float(np.abs(b).max()), 1e-300)
    return float(np.abs(np.asarray(a) - np.asarray(b)).max()) <= RTOL * scale


def test_noalloc_matches_allocating_entry_point_twice(nx):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    L = nx.lib()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for ne, np_, seed in ((5, 2, 11), (12, 8, 12)):
        ins = _inputs(torch, dev, ne, np_, seed)
        rc0, fe0, fp0, E0 = _call(L.neoxc_dev_gam4_dscf, torch, dev, stream, ne, np_, ins)
        assert rc0 == 0, L.neoxc_last_error()
        rc1, fe1, fp1, E1 = _call(L.neoxc_dev_gam4_dscf_noalloc, torch, dev, stream, ne, np_, ins)
        assert rc1 == 0, L.neoxc_last_error()
        assert _close(fe1, fe0) and _close(fp1, fp0)
        assert abs(E1 - E0) <= RTOL * max(abs(E0), float(np.abs(fe0).max()))


def test_noalloc_rejects_oversized_system(nx):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    L = nx.lib()
    f64 = torch.float64
    ne, np_ = 20, 8          # needs 8^2*20^3 + 8^2 = 512,064 doubles
    bufs = [torch.zeros(1, dtype=f64, device=dev) for _ in range(7)]
    rc = L.neoxc_dev_gam4_dscf_noalloc(
        C.c_void_p(torch.cuda.current_stream(dev).cuda_stream), ne, np_,
        *[C.c_void_p(b.data_ptr()) for b in bufs])
    assert rc == 4  # NEOXC_ERR_UNSUPPORTED, before any launch
    assert b"built-in array" in L.neoxc_last_error()
