"""SCF / Krylov sweep with tail=false corrections on the CPU: the oracle's
restatement of QuTree's SCF (oracle/scf.py) against independent checks, and
the planner's SCF segments (interpreted with numpy) against the oracle."""
import numpy as np
import pytest

import scf as S
from plan_emulator import PlanView, scf_emulated
from tree_energy import energy
from qutree_gb300.model import (MLO, OP_DENSE, SOP, HOBasis, OperatorTable, Tree, TensorTree,
                                _Build, balanced_tree, config_problem, coupled_oscillators,
                                random_wavefunction)

QT_PLAN_COMPRESSED, QT_PLAN_SCF = 2, 0x2000


def _exact_ground(tree, sop, omega):
    """Ground-state energy of sum_i (T_i + w^2 x_i^2 / 2) + sum c_ij x_i x_j."""
    f = tree.n_leaves
    K = np.eye(f) * omega ** 2
    for term, c in zip(sop.terms, sop.coeffs):
        modes = [m for m, _ in term.factors]
        if len(modes) == 2 and modes[0] != modes[1]:
            i, j = modes
            K[i, j] += c.real
            K[j, i] += c.real
    return 0.5 * np.sqrt(np.linalg.eigvalsh(K)).sum()


def test_oracle_effective_hamiltonian_at_top_is_the_energy():
    # bottom-up orthonormal Psi is in canonical gauge toward the top: there
    # <Phi_top|H_eff|Phi_top> / <Phi_top|Phi_top> is the full tree energy
    for cfg in (0, 4):
        tree, sop, psi = config_problem(cfg)
        rep = S.SCFOracle(tree, sop)
        rep.initial_build(psi.tensors)
        top = tree.top.address
        x = psi.tensors[top]
        e = np.vdot(x, rep.apply(x, top)).real / np.vdot(x, x).real
        assert abs(e - energy(tree, sop, psi.tensors)) <= 1e-12 * abs(e)


def test_oracle_converges_to_the_exact_ground_state():
    # 4 coupled oscillators, p = 12, bonds 6: the SCF reaches the harmonic
    # ground state; the last Ritz value equals the final tree energy
    from qutree_gb300.model import OMEGA_AU
    tree = balanced_tree(4, 12, 6)
    rng = np.random.default_rng(3)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.1, rng=rng)
    psi = random_wavefunction(tree, 5)
    E, fin = S.scf(tree, sop, psi.tensors, n_iter=6, n_krylov=8, n_itp=2, beta=400.0)
    exact = _exact_ground(tree, sop, OMEGA_AU)
    assert abs(E[-1] - energy(tree, sop, fin)) <= 1e-12 * abs(E[-1])
    # 1.2e-9 relative is the 12-point DVR / bond-6 truncation, not the sweep
    assert abs(E[-1] - exact) <= 5e-9 * exact
    assert E[-1] >= exact - 1e-12 * exact  # variational


@pytest.mark.parametrize("n_itp", [0, 1])
def test_plan_scf_cfg0(n_itp):
    tree, sop, psi = config_problem(0)
    E0, fin0 = S.scf(tree, sop, psi.tensors, n_iter=2, n_krylov=6, n_itp=n_itp, beta=200.0)
    pv = PlanView(tree, sop, QT_PLAN_COMPRESSED | QT_PLAN_SCF)
    E1, fin1 = scf_emulated(pv, tree, psi.flat(), n_iter=2, n_krylov=6, n_itp=n_itp, beta=200.0)
    assert len(E0) == len(E1) == 2 * (2 * tree.n_nodes - 1)
    assert np.abs(E0 - E1).max() <= 1e-12 * np.abs(E0).max()
    e1 = energy(tree, sop, TensorTree.from_flat(tree, fin1).tensors)
    assert abs(e1 - energy(tree, sop, fin0)) <= 1e-12 * abs(e1)


def test_plan_scf_ternary_tree_three_body_terms():
    # nodes with three children: LCA terms over several legs, environment
    # blocks of two siblings; 3-body terms and several factors on one leaf
    groups = [_Build([3, 3, 3, 3], [_Build([4, 3], leaf=True) for _ in range(3)]) for _ in range(3)]
    tree = Tree(_Build([3, 3, 3, 1], groups))
    rng = np.random.default_rng(17)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    b = HOBasis(4, omega=1.0)
    x = sop.ops.add("x3", 1, b.x.astype(complex))
    kin = sop.ops.add("k3", OP_DENSE, b.kin)
    for (i, j, k) in [(0, 4, 8), (1, 2, 7), (3, 5, 6), (0, 1, 2)]:
        sop.push_back(MLO([(i, x), (j, x), (k, x)]), 0.05 * (i + 1))
    sop.push_back(MLO([(4, kin), (4, x)]), 0.3)
    psi = random_wavefunction(tree, 17)
    E0, fin0 = S.scf(tree, sop, psi.tensors, n_iter=2, n_krylov=5, n_itp=1, beta=2.0)
    pv = PlanView(tree, sop, QT_PLAN_COMPRESSED | QT_PLAN_SCF)
    E1, _ = scf_emulated(pv, tree, psi.flat(), n_iter=2, n_krylov=5, n_itp=1, beta=2.0)
    assert np.abs(E0 - E1).max() <= 1e-11 * np.abs(E0).max()


def test_plan_scf_partial_sop():
    # terms on a few leaves only: zero environments and empty blocks
    tree = balanced_tree(8, 4, 3)
    ops = OperatorTable()
    b = HOBasis(4, omega=1.0)
    kin = ops.add("k", OP_DENSE, b.kin)
    x = ops.add("x", 1, b.x.astype(complex))
    sop = SOP(ops)
    sop.push_back(MLO([(0, kin)]), 1.0)
    sop.push_back(MLO([(1, x), (2, x)]), 0.3)
    sop.push_back(MLO([(5, x)]), 0.7)
    psi = random_wavefunction(tree, 21)
    # on a leaf no term touches, H_eff = 1 x Eout spans at most d_up = 3 Krylov
    # vectors: a fourth would be zero (the reference divides by its norm)
    E0, _ = S.scf(tree, sop, psi.tensors, n_iter=1, n_krylov=3)
    pv = PlanView(tree, sop, QT_PLAN_COMPRESSED | QT_PLAN_SCF)
    E1, _ = scf_emulated(pv, tree, psi.flat(), n_iter=1, n_krylov=3)
    assert np.abs(E0 - E1).max() <= 1e-12 * max(1.0, np.abs(E0).max())


def test_plan_scf_needs_the_compressed_plan():
    tree, sop, _ = config_problem(0)
    with pytest.raises(ValueError, match="SCF"):
        PlanView(tree, sop, 1 | QT_PLAN_SCF)


def test_plan_scf_double_float_segments():
    # the double-float plan's SCF segments (conversions are copies here)
    tree, sop, psi = config_problem(0)
    E0, _ = S.scf(tree, sop, psi.tensors, n_iter=1, n_krylov=6)
    pv = PlanView(tree, sop, QT_PLAN_COMPRESSED | QT_PLAN_SCF, prec=1)
    E1, _ = scf_emulated(pv, tree, psi.flat(), n_iter=1, n_krylov=6)
    assert np.abs(E0 - E1).max() <= 1e-12 * np.abs(E0).max()


@pytest.mark.parametrize("cfg,kw", [(0, dict(n_iter=2, n_krylov=6, n_itp=1, beta=200.0)),
                                    (0, dict(n_iter=1, n_krylov=4, breakdown=1e-12))])
def test_compiled_scf_equals_the_numpy_restatement(cfg, kw):
    # orc_scf (the compiled twin, used as the bench's CPU baseline) against
    # oracle/scf.py: the same Ritz value for every Krylov solve
    import oracle as O
    tree, sop, psi = config_problem(cfg)
    E0, _ = S.scf(tree, sop, psi.tensors, **kw)
    E1, fin = O.scf(tree, sop, psi.flat(), **kw)
    assert len(E1) == len(E0)
    assert np.abs(E1 - E0).max() <= 1e-12 * max(1.0, np.abs(E0).max())
    # the final state's energy equals the last Ritz value (the last solve is at the top)
    assert abs(O.derivative(tree, sop, fin).energy - E1[-1]) <= 1e-11 * max(1.0, abs(E1[-1]))
