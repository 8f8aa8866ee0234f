"""cfg1 (64 modes, p=32, bonds 32..64, 384 terms) at full size on the GPU:
size-independent properties, plus the oracle (OpenBLAS back end) once."""
import numpy as np
import pytest

import oracle as O
from helpers import deriv_errors, rel_err, rho_weighted
from qutree_gb300 import qtgpu
from qutree_gb300.model import SOP, config_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg1():
    return config_problem(1)


@pytest.fixture(scope="module")
def gpu_ref(cfg1):
    tree, sop, psi = cfg1
    out = {}
    for fl in (0, 1, 1 | qtgpu.QT_PREC_DF64, 2, 2 | qtgpu.QT_PREC_DF64, 2 | qtgpu.QT_PREC_DF64_TC):
        h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=fl)
        d = qtgpu.Derivative(h, psi.flat())
        out[fl] = (d, h.energy(), h.matrices(qtgpu.QT_MAT_RHO))
        h.close()
    return out


def test_flavours_agree(cfg1, gpu_ref):
    tree, _, _ = cfg1
    d0, e0, rho = gpu_ref[0]
    # the tensor-core mode products included: with bonds above 48 (here 51..64)
    # four level accumulators fit tensor memory, the last one rounding levels
    # 3..6 together in fp32 (~1e-10 of a typical output; stated in qtgpu.h)
    for fl, tol in ((1, 1e-12), (1 | qtgpu.QT_PREC_DF64, 1e-11), (2, 1e-12), (2 | qtgpu.QT_PREC_DF64, 1e-11),
                    (2 | qtgpu.QT_PREC_DF64_TC, 1e-10)):
        d1, e1, rho1 = gpu_ref[fl]
        assert abs(e0 - e1) <= tol * abs(e0)
        assert rel_err(rho1, rho) <= tol
        err, noise = deriv_errors(tree, d1, d0, rho)
        assert err <= tol and noise <= 1e-11


def test_tangent_space(cfg1, gpu_ref):
    # every non-top derivative is orthogonal to its node's SPFs: Phi^dag dPhi = 0
    tree, _, psi = cfg1
    d, _, _ = gpu_ref[1]
    off = tree.offsets()
    scale = np.abs(d).max()
    for n in tree.nodes:
        if n.is_top:
            continue
        phi = psi.tensors[n.address].reshape((-1, n.d_up), order="F")
        x = d[off[n.address]:off[n.address + 1]].reshape((-1, n.d_up), order="F")
        assert np.abs(phi.conj().T @ x).max() <= 1e-11 * scale


def test_linearity_in_the_operator(cfg1, gpu_ref):
    # H = H_a + H_b: the projected derivatives and energies add up
    tree, sop, psi = cfg1
    d, e, rho = gpu_ref[1]
    half = len(sop) // 2
    parts = []
    for terms in (range(half), range(half, len(sop))):
        s = SOP(sop.ops)
        for l in terms:
            s.push_back(sop.terms[l], sop.coeffs[l])
        h = qtgpu.HamiltonianRepresentation(s, tree, flavour=1)
        parts.append((qtgpu.Derivative(h, psi.flat()), h.energy()))
        h.close()
    assert abs(parts[0][1] + parts[1][1] - e) <= 1e-12 * abs(e)
    err, noise = deriv_errors(tree, parts[0][0] + parts[1][0], d, rho)
    assert err <= 1e-12 and noise <= 1e-11


@pytest.mark.slow
def test_against_oracle_full_size(cfg1, gpu_ref):
    tree, sop, psi = cfg1
    O.attach_openblas(fast=True)
    r = O.derivative(tree, sop, psi.flat(), backend=O.BLAS, fast=True)
    d, e, rho = gpu_ref[0]
    assert abs(e - r.energy) <= 1e-12 * abs(r.energy)
    assert rel_err(rho, r.rho) <= 1e-12
    err, noise = deriv_errors(tree, d, r.dpsi, r.rho)
    assert err <= 1e-12 and noise <= 1e-11
