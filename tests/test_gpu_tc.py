"""Tensor-core (tcgen05) form of the factorised gam_4 Fock build
(neoxc_dev_gam4_fock_factored_tc) against the FP64 factorised build.

Each FP64 operand of the transforms and of the focke contraction is split
into two TF32 halves and multiplied in three products with FP32
accumulation (~2^-21 relative per product); the GAM_2s passes, traces,
gradients and reductions stay FP64.  Tolerance: 2e-5 of each output's
scale (a few hundred ulps of the 3xTF32 products accumulated over K).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 2e-5


def _tables(rng, ne, np_):
    ee = rng.uniform(0.0, 1.0, (ne,) * 4)
    gee = 0.5 * (ee + ee.transpose(2, 3, 0, 1))
    gs = rng.uniform(0.0, 1.0, (np_, np_) + (ne,) * 4)
    g2s = 0.5 * (gs + gs.transpose(0, 1, 4, 5, 2, 3))
    return np.ascontiguousarray(gee.ravel()), np.ascontiguousarray(g2s.ravel())


@pytest.mark.parametrize("ne,np_", [(3, 2), (12, 8), (33, 3), (64, 2)])
def test_tc_factored_matches_fp64(nx, ne, np_):
    torch = pytest.importorskip("torch")
    from neoxc import basis
    dev = torch.device("cuda:0")
    f64 = torch.float64
    rng = np.random.default_rng(900 + ne)
    gee, g2s = _tables(rng, ne, np_)
    DE = basis.random_density(ne, max(2, ne // 3), ne, 2.0)
    DP = basis.random_density(np_, 1, ne + 1, 1.0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=f64, device=dev)  # noqa: E731
    d_gee, d_g2s = t(gee), t(g2s)
    d_DE, d_DP = t(DE.ravel(order="F")), t(DP.ravel(order="F"))
    s = torch.cuda.current_stream(dev).cuda_stream
    out = {}
    for name, fn in (("fp64", nx.dev_gam4_fock_factored), ("tc", nx.dev_gam4_fock_factored_tc)):
        fe = torch.zeros(ne * ne, dtype=f64, device=dev)
        fp = torch.zeros(np_ * np_, dtype=f64, device=dev)
        E = torch.zeros(1, dtype=f64, device=dev)
        fn(s, ne, np_, d_gee, d_g2s, d_DE, d_DP, fe, fp, E)
        torch.cuda.synchronize(dev)
        out[name] = (fe.cpu().numpy(), fp.cpu().numpy(), float(E.item()))
    a, b = out["fp64"], out["tc"]
    for x, y, w in ((b[0], a[0], "focke"), (b[1], a[1], "fockp")):
        scale = np.abs(y).max()
        assert np.abs(x - y).max() <= TOL * scale, (w, np.abs(x - y).max() / scale)
    assert abs(b[2] - a[2]) <= TOL * abs(a[2]), (b[2], a[2])
    # a second call accumulates into the Fock matrices and overwrites E
    fe = torch.ones(ne * ne, dtype=f64, device=dev)
    fp = torch.ones(np_ * np_, dtype=f64, device=dev)
    E = torch.zeros(1, dtype=f64, device=dev)
    nx.dev_gam4_fock_factored_tc(s, ne, np_, d_gee, d_g2s, d_DE, d_DP, fe, fp, E)
    torch.cuda.synchronize(dev)
    assert np.allclose(fe.cpu().numpy() - 1.0, b[0], rtol=0, atol=1e-12 * np.abs(b[0]).max() + 1e-300)
    assert float(E.item()) == b[2]
