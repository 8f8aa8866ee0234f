"""CDVR potential path on the GPU (QT_PLAN_CDVR) against the oracle.

The several-matrix grid solve (weighted simultaneous diagonalisation) is
discontinuous in its inputs, so the oracle runs its bit-fixed restatement on
the device's own X matrices and density matrices (checked against the
oracle's to 1e-10 first); the device kernel must reproduce that restatement
bit for bit, and everything downstream must agree to rounding."""
import numpy as np
import pytest

import cdvr as C
from helpers import cdvr_device_wsd, node_matrices
from plan_emulator import B_CDVR, PlanView
from qutree_gb300 import qtgpu
from qutree_gb300.model import cdvr_problem

pytestmark = pytest.mark.gpu

CASES = [(8, 8, 6), (16, 12, 8), ("uneven6", 5, 0)]


def problem(n_modes, p, bond, seed):
    if n_modes == "uneven6":  # a three-child node and uneven depth (tests/test_cdvr_cpu.py)
        from test_cdvr_cpu import kinetic_sop, uneven6
        from qutree_gb300.model import HOBasis, PolyPotential, random_wavefunction
        tree = uneven6(p)
        basis = HOBasis(p)
        V = PolyPotential.cdvr_model(6)
        V.terms.append((0.01, [(0, 1), (3, 1), (5, 2)]))
        return tree, kinetic_sop(tree, basis), random_wavefunction(tree, seed), \
            {m: basis.x for m in range(6)}, V
    return cdvr_problem(n_modes, p, bond, seed=seed)


def run(n_modes, p, bond, flavour, aligned, seed=5):
    tree, sop, psi, xs, V = problem(n_modes, p, bond, seed)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour, potential=V, leaf_x=xs,
                                        aligned_hole_grids=aligned)
    try:
        dpsi = qtgpu.Derivative(h, psi.flat())
        h00, s00 = h.energy_parts()
        arena = h.matrices(qtgpu.QT_MAT_CDVR)
        rho = node_matrices(tree, h.matrices(qtgpu.QT_MAT_RHO))
    finally:
        h.close()
    pv = PlanView(tree, sop, flavour=flavour, cdvr=(xs, V, aligned))
    return tree, sop, psi, xs, V, dpsi, h00, arena, rho, pv


@pytest.mark.parametrize("n_modes,p,bond", CASES)
@pytest.mark.parametrize("flavour", [qtgpu.QT_PLAN_REFERENCE, qtgpu.QT_PLAN_GROUPED])
@pytest.mark.parametrize("aligned", [False, True])
def test_cdvr_sweep_matches_oracle(n_modes, p, bond, flavour, aligned):
    tree, sop, psi, xs, V, dpsi, h00, arena, rho, pv = run(n_modes, p, bond, flavour, aligned)
    wsd = cdvr_device_wsd(tree, arena, pv.tables[39], rho)
    res = C.derivative(tree, sop, psi.flat(), C.CDVROracle(tree, xs, V, aligned=aligned), wsd=wsd)
    assert wsd.calls
    assert abs(h00 - res.h00) <= 1e-12 * abs(res.h00)
    assert np.abs(dpsi - res.dpsi).max() <= 1e-10 * np.abs(res.dpsi).max()


@pytest.mark.parametrize("n_modes,p,bond", CASES)
def test_wsd_kernel_is_bit_exact(n_modes, p, bond):
    """Every several-matrix grid problem: the device's transformation and
    grid equal, bit for bit, the restatement run on the device's inputs."""
    tree, sop, psi, xs, V, dpsi, h00, arena, rho, pv = run(n_modes, p, bond, qtgpu.QT_PLAN_REFERENCE,
                                                           False)
    wsd_t, terms = pv.tables[27], pv.tables[28]
    rho_off = {n.address: n for n in tree.nodes}
    assert len(wsd_t)
    for r in wsd_t:
        wb, wo, tb, to, gb, go, sb, so, d, n, first = (int(x) for x in r)
        # the weight is the node's density matrix: find the node by its offset
        node = [a for a, o in enumerate(pv.tables[11]) if o == wo][0]
        xs_dev = []
        for q in range(first, first + n):
            xb, xo = terms[q]
            assert xb == B_CDVR
            xs_dev.append(arena[xo:xo + d * d].reshape((d, d), order="F"))
        T, grids, info = C.layer_grid_multi(xs_dev, rho[node])
        assert np.array_equal(arena[to:to + d * d], T.ravel(order="F"))
        assert np.array_equal(arena[go:go + n * d].real, np.concatenate(grids))
        assert rho_off[node].d_up == d


def test_cdvr_frozen_split_equals_sweep():
    """build + frozen-matrix layer derivatives == one sweep (CDVR update in
    the build graph, CDVR apply in the frozen-matrix graph)."""
    tree, sop, psi, xs, V = cdvr_problem(8, 8, 6, seed=3)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_GROUPED, potential=V, leaf_x=xs)
    try:
        d_full = qtgpu.Derivative(h, psi.flat())
        h.upload(psi)
        h.build()
        h.layer_derivatives()
        assert np.array_equal(h.dpsi(), d_full)
    finally:
        h.close()


def test_cdvr_rejects_unsupported_plans():
    tree, sop, psi, xs, V = cdvr_problem(8, 8, 6)
    for fl in (qtgpu.QT_PLAN_COMPRESSED, qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64,
               qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PLAN_GRADIENT):
        with pytest.raises(qtgpu.QtError):
            qtgpu.HamiltonianRepresentation(sop, tree, flavour=fl, potential=V, leaf_x=xs).close()
