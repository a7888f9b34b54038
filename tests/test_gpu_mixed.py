"""Accuracy of the mixed gam_3 build (NEOXC_SCF_MIXED: FP32 Gaussian-product
set-up and Hermite folds, FP64 Boys function, seeds and Hermite-Coulomb sum)
on a system with an electronic d shell and s/p/d nuclear functions, so that
every Hermite order of the general class is exercised: the dense GM3ICR
tensor stays within FP32 rounding of the FP64 build, element by element
against the tensor's scale.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gam3_mixed_tensor_within_fp32_rounding(nx):
    from neoxc import basis
    s = basis.synthetic(seed=105, nat=3, nebf=5, nprim=2, npbf=3, ngtg=2, lmax_e=2, lmax_p=2)
    ref = nx.gam3_ic1(s)
    x = nx.gam3_ic1(s, mixed=True)
    scale = float(np.abs(ref).max())
    err = float(np.abs(x - ref).max()) / scale
    print("gam_3 mixed max |diff| / max |x|: %.2e" % err)
    assert err <= 1e-6
