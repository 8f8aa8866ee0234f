"""Double-float arithmetic (FP32 pipe, and with the tensor-core digit
products) against complex128 on the 48..96-bond 64-mode tree (regularisation
1e-8): one sweep, then constant-mean-field steps of dt = 0.01 in lockstep;
the energies stay within |dE| <= 1e-8 (the headline metric's bar) and the
projected derivatives within 1e-9 relative (rho-weighted)."""
import numpy as np
import pytest

from helpers import rho_weighted
from qutree_gb300 import qtgpu
from qutree_gb300.model import config_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [qtgpu.QT_PREC_DF64, qtgpu.QT_PREC_DF64_TC])
def test_double_float_tracks_complex128_along_cmf(prec):
    tree, sop, psi = config_problem(3)
    hf = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED, eps=1e-8)
    hd = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED | prec, eps=1e-8)
    try:
        for h in (hf, hd):
            h.upload(psi.flat())
        for step in range(4):
            if step:
                hf.cmf(0.01, 1)
                hd.cmf(0.01, 1)
            hf.derivative()
            hd.derivative()
            ef, ed = hf.energy(), hd.energy()
            assert abs(ed - ef) <= 1e-8
            rho = hf.matrices(qtgpu.QT_MAT_RHO)
            a = rho_weighted(tree, hd.dpsi(), rho)
            b = rho_weighted(tree, hf.dpsi(), rho)
            assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(b)
    finally:
        hf.close()
        hd.close()
