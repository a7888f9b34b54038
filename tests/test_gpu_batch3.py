"""Many systems' gam_3 in persistent launches (neoxc_gam3_ic1_batch) against
the per-system builder (neoxc_gam3_ic1).

Uneven systems of three angular classes (s only; s/p electrons with s/p/d
nuclear functions; an electronic d shell) go through one persistent launch
per class over a device work queue; every system's GM3ICR must equal its
separate build (same per-block arithmetic, so to the last bit within 1e-14
of scale), in FP64 and in the mixed precision, and the autotuner must have
recorded a choice for each class used.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _systems(xchf):
    from neoxc import basis
    out = basis.proton_scan(xchf["sys"], 3, 0.3, seed=5)          # s only
    for seed, ne, np_ in ((71, 3, 2), (72, 4, 3), (73, 5, 1)):
        out.append(basis.synthetic(seed=seed, nat=2, nebf=ne, nprim=(1, 2), npbf=np_, ngtg=2,
                                   lmax_e=1, lmax_p=2))
    out.append(basis.synthetic(seed=74, nat=2, nebf=5, nprim=1, npbf=1, ngtg=2, lmax_e=2,
                               lmax_p=0))                           # electronic d shell
    return out


@pytest.mark.parametrize("mixed", [False, True])
def test_batch_equals_separate_builds(nx, xchf, mixed):
    systems = _systems(xchf)
    outs, sec = nx.gam3_ic1_batch(systems, mixed=mixed)
    assert sec > 0.0
    for s, x in zip(systems, outs):
        ref = nx.gam3_ic1(s, mixed=mixed)
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(x - ref).max() <= 1e-14 * scale, s.name
    tune = nx.gam3_batch_tuning()
    assert len(tune) >= 3 and all(t["ctas_per_sm"] >= 1 and t["chunk"] >= 1 for t in tune)
