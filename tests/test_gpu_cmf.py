"""Constant-mean-field propagation on the GPU (qt_build, qt_layer_derivatives,
qt_cmf_propagate) against the oracle's restatement of the same fixed-step
scheme."""
import numpy as np
import pytest

import oracle as O
from helpers import rel_err
from qutree_gb300 import qtgpu
from qutree_gb300.model import config_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("flavour", [qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64,
                                     qtgpu.QT_PLAN_COMPRESSED, qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64,
                                     qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC])
def test_split_graphs_equal_the_sweep(flavour):
    # build + frozen-matrix layer derivatives at the same Psi == one full sweep;
    # bit for bit where both run the same stages, within rounding where the
    # compressed sweep fuses Apply into the derivative
    from helpers import deriv_errors
    tree, sop, psi = config_problem(4)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour)
    try:
        d_full = qtgpu.Derivative(h, psi.flat())
        rho = h.matrices(qtgpu.QT_MAT_RHO)
        h.upload(psi)
        h.build()
        h.layer_derivatives()
        if flavour & 0xFF == qtgpu.QT_PLAN_COMPRESSED:
            err, noise = deriv_errors(tree, h.dpsi(), d_full, rho)
            tol = 1e-11 if flavour & qtgpu.QT_PREC_DF64 else 1e-12
            noise_tol = 1e-11
            if flavour & qtgpu.QT_PREC_DF64_TC:  # digit arithmetic: stated tolerance 1e-10
                tol = noise_tol = 1e-10
            assert err <= tol and noise <= noise_tol
        else:
            assert np.array_equal(h.dpsi(), d_full)
    finally:
        h.close()


@pytest.mark.parametrize("flavour,tol", [(qtgpu.QT_PLAN_GROUPED, 1e-11),
                                         (qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64, 1e-10),
                                         (qtgpu.QT_PLAN_COMPRESSED, 1e-11),
                                         (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64, 1e-10),
                                         (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC, 1e-10)])
def test_cmf_matches_oracle(flavour, tol):
    tree, sop, psi = config_problem(0)
    flat = psi.flat()
    ref = O.cmf(tree, sop, flat, dt=1.0, n_steps=10, n_sub=2)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour)
    try:
        h.upload(flat)
        h.cmf(1.0, 10, n_sub=2)
        got = h.psi()
    finally:
        h.close()
    assert rel_err(got, ref) <= tol


def test_cmf_conserves_energy_and_relaxes_in_imaginary_time():
    tree, sop, psi = config_problem(0)
    flat = psi.flat()
    e0 = O.derivative(tree, sop, flat).energy
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64)
    try:
        h.upload(flat)
        h.cmf(0.5, 40, n_sub=1)
        e_real = O.derivative(tree, sop, h.psi()).energy
        h.upload(flat)
        h.cmf(20.0, 20, n_sub=2, phase=-1j)
        y = h.psi()
        t = tree.top
        off = tree.offsets()
        y[off[t.address]:] /= np.linalg.norm(y[off[t.address]:])
        e_imag = O.derivative(tree, sop, y).energy
    finally:
        h.close()
    assert abs(e_real - e0) <= 1e-4 * abs(e0)
    assert e_imag < e0 - 0.1 * abs(e0)


@pytest.mark.parametrize("flavour,tol", [(qtgpu.QT_PLAN_GROUPED, 1e-9),
                                         (qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64, 1e-8)])
def test_adaptive_cmf_matches_the_restatement(flavour, tol):
    # CMFIntegrator::Integrate with Bulirsch-Stoer node integrators on the
    # device's frozen-matrix derivatives (qutree_gb300/cmf.py), against the
    # oracle's sequential restatement (oracle/cmf_bs.py) on the oracle's
    # derivatives: the same accept / refuse decisions, the same wavefunction
    import cmf_bs as B
    from helpers import tree_overlap
    from qutree_gb300.cmf import CMFIntegrator
    tree, sop, psi = config_problem(0)
    flat = psi.flat()
    want, dt_want, st = B.cmf_integrate(tree, O.Frozen(tree, sop), flat, 0.0, 2.0, 0.5, 2.0, 1e-6, 1e-7)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour)
    try:
        I = CMFIntegrator(h)
        got, dt_got = I.integrate(flat, 0.0, 2.0, 0.5, acc_root=1e-6, acc_leaf=1e-7)
        on_device = h.psi()
    finally:
        h.close()
    assert np.array_equal(on_device, got)
    assert I.stats["accepted"] == st["accepted"] and I.stats["refused"] == st["refused"]
    assert rel_err(got, want) <= tol
    ov = tree_overlap(tree, want, got) / np.sqrt(tree_overlap(tree, want, want).real *
                                                 tree_overlap(tree, got, got).real)
    assert abs(1 - abs(ov)) < tol
