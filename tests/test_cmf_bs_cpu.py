"""Adaptive CMF integrator (qutree_gb300/cmf.py) on the CPU: its
Bulirsch-Stoer core against an exactly solvable ODE, the node-batched
integrator against the oracle's sequential restatement of
CMFIntegrator::Integrate (oracle/cmf_bs.py) with the oracle's frozen-matrix
derivatives standing in for the device's, and convergence to the
fixed-step scheme."""
import numpy as np
import pytest

import cmf_bs as B
import oracle as O
from helpers import tree_overlap
from qutree_gb300 import cmf as C
from qutree_gb300 import qtgpu
from qutree_gb300.model import balanced_tree, config_problem, coupled_oscillators, random_wavefunction


class FrozenRep:
    """The calls CMFIntegrator makes on a HamiltonianRepresentation, served
    by the oracle's frozen-matrix session."""

    def __init__(self, tree, sop, phase=1.0):
        self.tree = tree
        self.f = O.Frozen(tree, sop, phase=phase)
        self._psi = self._d = None

    def upload(self, psi):
        self._psi = np.array(psi, dtype=np.complex128, copy=True)

    def build(self):
        self.f.build(self._psi)

    def layer_derivatives(self, phase=1.0):
        self._d = self.f.deriv(self._psi)

    def dpsi(self):
        return self._d.copy()

    def matrices(self, which):
        assert which == qtgpu.QT_MAT_RHO
        return self.f.rho()


def _linear_ode(n=6, seed=3):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    A = 0.5 * (A + A.conj().T)
    y0 = rng.normal(size=n) + 1j * rng.normal(size=n)
    return A, y0


def _exact(A, y0, t):
    w, U = np.linalg.eigh(A)
    return U @ (np.exp(-1j * w * t) * (U.conj().T @ y0))


def test_bs_restatement_solves_a_linear_ode():
    A, y0 = _linear_ode()
    bs = B.BSIntegrator(y0.size)
    err = lambda p, q: float(np.linalg.norm(p - q) / np.linalg.norm(p))
    y, x, dx = bs.integrate(y0.copy(), 0.0, 3.0, 0.5, 1e-11, lambda t, y: -1j * (A @ y), err)
    assert abs(x - 3.0) < 1e-9
    assert np.abs(y - _exact(A, y0, x)).max() <= 1e-9 * np.abs(y0).max()


def test_node_coroutine_equals_restatement_bit_for_bit():
    A, y0 = _linear_ode(8, 5)
    err = lambda p, q: float(np.linalg.norm(p - q) / np.linalg.norm(p))
    f = lambda y: -1j * (A @ y)
    want, _, dx_want = B.BSIntegrator(y0.size).integrate(y0.copy(), 0.0, 2.0, 0.3, 1e-9, lambda t, y: f(y), err)
    g = C._bs_node(y0.copy(), 0.0, 2.0, 0.3, 1e-9, err)
    req = next(g)
    n_calls = 1
    while True:
        try:
            req = g.send(f(req))
            n_calls += 1
        except StopIteration as stop:
            got, dx_got = stop.value
            break
    assert np.array_equal(got, want) and dx_got == dx_want and n_calls > 10


def _second_tree():
    tree = balanced_tree(8, 6, 3)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(11),
                              omega=1.0)
    return tree, sop, random_wavefunction(tree, 11)


@pytest.mark.parametrize("case,phase", [("cfg0", 1.0), ("cfg0", -1j), ("small", 1.0)])
def test_batched_integrator_equals_sequential_restatement(case, phase):
    tree, sop, psi = config_problem(0) if case == "cfg0" else _second_tree()
    flat = psi.flat()
    frozen = O.Frozen(tree, sop, phase=phase)
    calls = [0]
    node_deriv = frozen.deriv_node

    def counted(n, phi):
        calls[0] += 1
        return node_deriv(n, phi)

    frozen.deriv_node = counted
    want, dt_want, st = B.cmf_integrate(tree, frozen, flat, 0.0, 1.5, 0.4, 1.5, 1e-6, 1e-7)
    I = C.CMFIntegrator(FrozenRep(tree, sop, phase=phase), phase=phase)
    got, dt_got = I.integrate(flat, 0.0, 1.5, 0.4, acc_root=1e-6, acc_leaf=1e-7)
    assert np.array_equal(got, want) and dt_got == dt_want
    assert I.stats["accepted"] == st["accepted"] and I.stats["refused"] == st["refused"]
    # one derivative call serves every waiting node of a round: far fewer
    # device calls than the sequential scheme's per-node evaluations
    assert I.stats["derivative_rounds"] * 3 < calls[0]


def test_adaptive_cmf_converges_to_the_fixed_step_scheme():
    tree, sop, psi = config_problem(0)
    flat = psi.flat()
    I = C.CMFIntegrator(FrozenRep(tree, sop))
    got, _ = I.integrate(flat, 0.0, 2.0, 0.5, acc_root=1e-6, acc_leaf=1e-7)
    ref = O.cmf(tree, sop, flat, dt=2.0 / 400, n_steps=400, n_sub=2)
    ov = tree_overlap(tree, ref, got) / np.sqrt(tree_overlap(tree, ref, ref).real * tree_overlap(tree, got, got).real)
    assert abs(1 - abs(ov)) < 1e-9
    assert abs(O.derivative(tree, sop, got).energy - O.derivative(tree, sop, flat).energy) < 1e-6


def test_step_control_refuses_a_too_large_step():
    tree, sop, psi = config_problem(0)
    flat = psi.flat()
    I = C.CMFIntegrator(FrozenRep(tree, sop))
    got, dt = I.integrate(flat, 0.0, 3.0, 3.0, acc_root=1e-8, acc_leaf=1e-9)
    assert I.stats["refused"] > 0 and I.stats["accepted"] > 1 and dt < 3.0
    want, _, _ = B.cmf_integrate(tree, O.Frozen(tree, sop), flat, 0.0, 3.0, 3.0, 3.0, 1e-8, 1e-9)
    assert np.array_equal(got, want)


def test_orthogonal_keeps_the_state_and_orthonormalises():
    tree, sop, psi = config_problem(0)
    flat = psi.flat().copy()
    rng = np.random.default_rng(2)
    flat += 1e-3 * (rng.normal(size=flat.size) + 1j * rng.normal(size=flat.size))
    before = flat.copy()
    I = C.CMFIntegrator(FrozenRep(tree, sop))
    I.orthogonal(flat)
    off = tree.offsets()
    for n in tree.nodes:
        if n.is_top:
            continue
        P = flat[off[n.address]:off[n.address + 1]].reshape((-1, n.d_up), order="F")
        assert np.abs(P.conj().T @ P - np.eye(n.d_up)).max() < 1e-12
    want = before.copy()
    B.orthogonal(tree, want)
    assert np.allclose(flat, want, rtol=0, atol=1e-13)
    # a small non-orthonormality changes the state at second order only
    ov = tree_overlap(tree, before, flat) / np.sqrt(tree_overlap(tree, before, before).real *
                                                     tree_overlap(tree, flat, flat).real)
    assert abs(1 - abs(ov)) < 1e-4
