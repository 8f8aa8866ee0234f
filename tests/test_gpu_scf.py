"""SCF / Krylov sweep (qt_scf) on the GPU against the oracle's restatement of
QuTree's scf() (oracle/scf.py).  Compared: the lowest Ritz value of every
Krylov solve (gauge invariant) and the energy of the final wavefunction."""
import numpy as np
import pytest

import scf as S
from tree_energy import energy
from qutree_gb300 import qtgpu
from qutree_gb300.model import (MLO, OP_DENSE, SOP, HOBasis, OperatorTable, TensorTree, Tree, _Build,
                                balanced_tree, config_problem, coupled_oscillators, random_wavefunction)

pytestmark = pytest.mark.gpu
FL = qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PLAN_SCF


def _gpu_scf(tree, sop, psi, prec=qtgpu.QT_PREC_F64, **kw):
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=FL | prec)
    try:
        h.upload(psi.flat())
        E = h.scf(**kw)
        fin = TensorTree.from_flat(tree, h.psi())
    finally:
        h.close()
    return E, fin


def _check(tree, sop, psi, tol=1e-11, prec=qtgpu.QT_PREC_F64, **kw):
    E0, fin0 = S.scf(tree, sop, psi.tensors, **kw)
    E1, fin1 = _gpu_scf(tree, sop, psi, prec=prec, **kw)
    assert len(E1) == len(E0) == kw.get("n_iter", 1) * (2 * tree.n_nodes - 1)
    scale = max(1.0, np.abs(E0).max())
    assert np.abs(E1 - E0).max() <= tol * scale
    e1 = energy(tree, sop, fin1.tensors)
    assert abs(e1 - energy(tree, sop, fin0)) <= tol * scale
    assert abs(e1 - E1[-1]) <= tol * scale  # the last solve is at the top
    return E1


@pytest.mark.parametrize("n_itp", [0, 1])
def test_scf_cfg0(n_itp):
    tree, sop, psi = config_problem(0)
    _check(tree, sop, psi, n_iter=2, n_krylov=6, n_itp=n_itp, beta=200.0)


def test_scf_cfg4():
    tree, sop, psi = config_problem(4)
    _check(tree, sop, psi, n_iter=1, n_krylov=4)


@pytest.mark.parametrize("prec", [qtgpu.QT_PREC_DF64, qtgpu.QT_PREC_DF64_TC])
@pytest.mark.parametrize("cfg", [0, 4])
def test_scf_double_float(cfg, prec):
    # effective Hamiltonian in double-float (mode products on the FP32 pipe
    # or on the tensor cores), Lanczos and QR in complex128
    tree, sop, psi = config_problem(cfg)
    _check(tree, sop, psi, tol=1e-10, prec=prec, n_iter=1, n_krylov=5, n_itp=1, beta=200.0)


def test_scf_ternary_tree_three_body_terms():
    groups = [_Build([3, 3, 3, 3], [_Build([4, 3], leaf=True) for _ in range(3)]) for _ in range(3)]
    tree = Tree(_Build([3, 3, 3, 1], groups))
    rng = np.random.default_rng(17)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    b = HOBasis(4, omega=1.0)
    x = sop.ops.add("x3", 1, b.x.astype(complex))
    for (i, j, k) in [(0, 4, 8), (1, 2, 7), (3, 5, 6), (0, 1, 2)]:
        sop.push_back(MLO([(i, x), (j, x), (k, x)]), 0.05 * (i + 1))
    psi = random_wavefunction(tree, 17)
    _check(tree, sop, psi, n_iter=2, n_krylov=5, n_itp=1, beta=2.0)


def _partial():
    tree = balanced_tree(8, 4, 3)
    ops = OperatorTable()
    b = HOBasis(4, omega=1.0)
    kin = ops.add("k", OP_DENSE, b.kin)
    x = ops.add("x", 1, b.x.astype(complex))
    sop = SOP(ops)
    sop.push_back(MLO([(0, kin)]), 1.0)
    sop.push_back(MLO([(1, x), (2, x)]), 0.3)
    sop.push_back(MLO([(5, x)]), 0.7)
    return tree, sop, random_wavefunction(tree, 21)


def test_scf_rank_deficient_nodes_use_householder():
    # leaves no term touches end up rank 1: Cholesky-QR cannot isometrise them
    tree, sop, psi = _partial()
    _check(tree, sop, psi, n_iter=1, n_krylov=3)


def test_scf_invariant_krylov_space_ends_the_lanczos_recursion():
    # at leaves no term touches, H_eff = 1 x Eout spans d_up = 3 directions:
    # a fourth Lanczos vector would be rounding noise
    tree, sop, psi = _partial()
    E0, fin0 = S.scf(tree, sop, psi.tensors, n_iter=1, n_krylov=4, breakdown=1e-12)
    E1, fin1 = _gpu_scf(tree, sop, psi, n_iter=1, n_krylov=4)
    assert np.all(np.isfinite(E1))
    assert np.abs(E1 - E0).max() <= 1e-11 * max(1.0, np.abs(E0).max())
    e1 = energy(tree, sop, fin1.tensors)
    assert abs(e1 - E1[-1]) <= 1e-11 * max(1.0, abs(e1))


def test_scf_needs_its_plan():
    tree, sop, psi = config_problem(0)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED)
    try:
        h.upload(psi.flat())
        with pytest.raises(qtgpu.QtError, match="QT_ERR_STATE"):
            h.scf()
    finally:
        h.close()


@pytest.mark.parametrize("prec", [qtgpu.QT_PREC_F64, qtgpu.QT_PREC_DF64])
def test_scf_full_size_64_modes(prec):
    # one SCF sweep on the 64-mode workload: the energy of the final state,
    # from an independent compressed sweep on the same context, equals the
    # last Ritz value, and the sweep lowers the energy
    tree, sop, psi = config_problem(1)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=FL | prec)
    try:
        h.upload(psi.flat())
        h.derivative()
        e_start = h.energy()
        E = h.scf(n_iter=1, n_krylov=5)
        h.derivative()
        e_end = h.energy()
    finally:
        h.close()
    assert len(E) == 2 * tree.n_nodes - 1
    assert abs(e_end - E[-1]) <= 1e-10 * abs(e_end)
    assert e_end < e_start
