"""The sweep planner on the CPU: the plan libqtgpu executes, interpreted with
numpy (tests/plan_emulator.py) and compared with the oracle."""
import numpy as np
import pytest

import oracle as O
from helpers import rel_err, rho_weighted
from plan_emulator import PlanView
from helpers import deriv_errors
from qutree_gb300.model import (MLO, OP_DENSE, SOP, HOBasis, OperatorTable, balanced_tree,
                                batched_problem, config_problem, config_tree_sop,
                                coupled_oscillators, forest, forest_psi, forest_sop,
                                random_wavefunction)


def _check(tree, sop, psi, flavour, budget=1 << 28, tol=1e-12, prec=0):
    flat = psi.flat()
    r = O.derivative(tree, sop, flat)
    pv = PlanView(tree, sop, flavour, budget, prec=prec)
    pv.run(flat)
    h00, s00 = pv.energy_parts()
    assert abs(h00.real / s00.real - r.energy) < tol * max(1, abs(r.energy))
    if flavour != 2:  # the compressed plan keeps no per-term matrices
        assert rel_err(pv.sparse(0), r.hmat) < tol
        assert rel_err(pv.sparse(1), r.hcon) < tol
    assert rel_err(rho_weighted(tree, pv.dpsi(), r.rho), rho_weighted(tree, r.dpsi, r.rho)) < tol
    return pv


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("flavour", [0, 1, 2])
def test_plan_cfg0(flavour, prec):
    tree, sop, psi = config_problem(0)
    pv = _check(tree, sop, psi, flavour, prec=prec)
    if flavour >= 1:
        assert pv.stats["exec_flops"] < pv.stats["ref_flops"]


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("flavour", [0, 1, 2])
def test_plan_small_budget_chunks(flavour, prec):
    # a tiny scratch budget forces every level into many chunks
    tree, sop, psi = config_problem(0)
    _check(tree, sop, psi, flavour, budget=200, prec=prec)


@pytest.mark.parametrize("leaves,p,b,seed", [(5, 4, 3, 1), (7, 5, 4, 2), (12, 3, 2, 3), (9, 6, 5, 4)])
@pytest.mark.parametrize("flavour", [0, 1, 2])
def test_plan_random_trees(leaves, p, b, seed, flavour):
    tree = balanced_tree(leaves, p, b)
    rng = np.random.default_rng(seed)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    psi = random_wavefunction(tree, seed)
    _check(tree, sop, psi, flavour)
    _check(tree, sop, psi, flavour, prec=1)


def test_plan_multi_factor_terms():
    # several factors on the same leaf (applied in list order) and 3-body terms
    tree = balanced_tree(6, 4, 3)
    ops = OperatorTable()
    b = HOBasis(4, omega=1.0)
    kin = ops.add("k", OP_DENSE, b.kin)
    x = ops.add("x", 1, b.x.astype(complex))
    rng = np.random.default_rng(5)
    m = ops.add("m", OP_DENSE, rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))
    sop = SOP(ops)
    sop.push_back(MLO([(0, kin), (0, x)]), 0.7)
    sop.push_back(MLO([(0, x), (0, kin)]), 0.3 - 0.2j)
    sop.push_back(MLO([(1, m), (3, x), (5, kin)]), 0.11)
    sop.push_back(MLO([(2, m), (2, m)]), 0.5)
    for k in range(6):
        sop.push_back(MLO([(k, kin)]), 1.0)
    psi = random_wavefunction(tree, 9)
    for fl in (0, 1, 2):
        _check(tree, sop, psi, fl)


@pytest.mark.parametrize("flavour", [0, 1, 2])
def test_plan_nodes_without_terms(flavour):
    # an SOP acting on a few leaves only: the other nodes get H Phi = 0
    tree = balanced_tree(8, 4, 3)
    ops = OperatorTable()
    b = HOBasis(4, omega=1.0)
    kin = ops.add("k", OP_DENSE, b.kin)
    x = ops.add("x", 1, b.x.astype(complex))
    sop = SOP(ops)
    sop.push_back(MLO([(0, kin)]), 1.0)
    sop.push_back(MLO([(1, x), (2, x)]), 0.3)
    psi = random_wavefunction(tree, 21)
    _check(tree, sop, psi, flavour)


def test_plan_reference_flops_cfg1():
    # the reference call sequence of one cfg1 sweep (represent, mean fields,
    # Apply, projector, Expectation): ~0.89 TFLOP
    tree, sop = config_tree_sop(1)
    pv = PlanView(tree, sop, 0)
    assert 0.85e12 < pv.stats["ref_flops"] < 0.95e12
    pv1 = PlanView(tree, sop, 1)
    assert pv1.stats["exec_flops"] < 0.6 * pv.stats["exec_flops"]
    assert pv1.stats["ref_flops"] == pv.stats["ref_flops"]
    pv2 = PlanView(tree, sop, 2)  # compressed: ~0.13 TFLOP per sweep
    assert pv2.stats["exec_flops"] < 0.3 * pv1.stats["exec_flops"]
    assert pv2.stats["ref_flops"] == pv.stats["ref_flops"]


def test_plan_rejects_bad_input():
    tree, sop = config_tree_sop(0)
    # operator dimension that does not match the leaf
    ops = OperatorTable()
    bad = ops.add("bad", OP_DENSE, np.eye(3))
    s = SOP(ops)
    s.push_back(MLO([(0, bad)]), 1.0)
    with pytest.raises(ValueError, match="operator dim"):
        PlanView(tree, s, 0)


@pytest.mark.parametrize("flavour,prec", [(0, 1), (1, 0), (2, 1)])
def test_plan_forest(flavour, prec):
    # many uneven trees in one plan: each tree's slice equals its own sweep
    trees, sops, psis = batched_problem(5)
    f, node_off, mode_off = forest(trees)
    pv = PlanView(f, forest_sop(sops, mode_off), flavour, prec=prec)
    pv.run(forest_psi(f, psis).flat())
    d = pv.dpsi()
    off = f.offsets()
    for k, (t, s, p) in enumerate(zip(trees, sops, psis)):
        r = O.derivative(t, s, p.flat())
        seg = d[off[node_off[k]]:off[node_off[k] + t.n_nodes]]
        err, noise = deriv_errors(t, seg, r.dpsi, r.rho)
        assert err <= 1e-12 and noise <= 1e-11


def test_plan_rejects_cross_tree_terms():
    trees, sops, psis = batched_problem(2)
    f, node_off, mode_off = forest(trees)
    s = forest_sop(sops, mode_off)
    a = s.ops.add(None, 1, np.ones(trees[0].leaf_dim(0), complex))
    b = s.ops.add(None, 1, np.ones(trees[1].leaf_dim(0), complex))
    s.push_back(MLO([(0, a), (mode_off[1], b)]), 1.0)
    with pytest.raises(ValueError, match="several trees"):
        PlanView(f, s, 1)


@pytest.mark.parametrize("flavour,prec", [(0, 0), (1, 1), (2, 0), (2, 1)])
def test_plan_gradient_finite_differences(flavour, prec):
    # dE/dPhi^* of every node: 2 Re <G, delta> equals the central difference
    # of E along random directions delta (all node tensors at once)
    from tree_energy import energy, fd_directional
    tree = balanced_tree(6, 4, 3)
    rng = np.random.default_rng(31)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    psi = random_wavefunction(tree, 32)
    pv = PlanView(tree, sop, flavour | 0x1000, prec=prec)
    pv.run(psi.flat())
    h00, s00 = pv.energy_parts()
    assert abs(h00.real / s00.real - energy(tree, sop, psi.tensors)) < 1e-12
    G = pv.gradient()
    off = tree.offsets()
    for k in range(4):
        dirs = [rng.standard_normal(n.shape) + 1j * rng.standard_normal(n.shape) for n in tree.nodes]
        flat_d = np.concatenate([d.ravel(order="F") for d in dirs])
        analytic = 2.0 * np.vdot(G, flat_d).real
        fd = fd_directional(tree, sop, psi, dirs)
        assert abs(analytic - fd) <= 1e-7 * max(1.0, abs(fd)), (analytic, fd)


def test_plan_compressed_frozen_stages():
    # the frozen-matrix derivative stages (constant-mean-field steps) recompute
    # the kept chains from Psi; on the Psi the matrices were built from they
    # reproduce the sweep's derivative
    tree, sop, psi = config_problem(0)
    pv = PlanView(tree, sop, 2)
    pv.run(psi.flat())
    d_sweep = pv.dpsi()
    pv.run(psi.flat(), frozen_after=True)
    assert len(pv.tables[0]) > pv.main_end
    assert np.abs(pv.dpsi() - d_sweep).max() <= 1e-14 * np.abs(d_sweep).max()


def test_plan_compressed_general_arity():
    # nodes with three children: cover groups over several free legs
    from qutree_gb300.model import Tree, _Build
    groups = [_Build([3, 3, 3, 3], [_Build([4, 3], leaf=True) for _ in range(3)]) for _ in range(3)]
    tree = Tree(_Build([3, 3, 3, 1], groups))
    rng = np.random.default_rng(17)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    ops = sop.ops
    b = HOBasis(4, omega=1.0)
    x = ops.add("x3", 1, b.x.astype(complex))
    for (i, j, k) in [(0, 4, 8), (1, 2, 7), (3, 5, 6), (0, 1, 2)]:
        sop.push_back(MLO([(i, x), (j, x), (k, x)]), 0.05 * (i + 1))
    psi = random_wavefunction(tree, 17)
    for fl in (1, 2):
        _check(tree, sop, psi, fl)
        _check(tree, sop, psi, fl, prec=1)




def test_plan_compressed_gradient_equals_grouped_on_a_ternary_tree():
    # environments with several siblings (LCA cover groups, sibling blocks):
    # the compressed plan's gradient equals the grouped plan's
    from qutree_gb300.model import Tree, _Build
    groups = [_Build([3, 3, 3, 3], [_Build([4, 3], leaf=True) for _ in range(3)]) for _ in range(3)]
    tree = Tree(_Build([3, 3, 3, 1], groups))
    rng = np.random.default_rng(41)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    b = HOBasis(4, omega=1.0)
    x = sop.ops.add("x3", 1, b.x.astype(complex))
    for (i, j, k) in [(0, 4, 8), (1, 2, 7), (3, 5, 6), (0, 1, 2)]:
        sop.push_back(MLO([(i, x), (j, x), (k, x)]), 0.05 * (i + 1))
    psi = random_wavefunction(tree, 41)
    grads = []
    for fl in (1, 2):
        pv = PlanView(tree, sop, fl | 0x1000)
        pv.run(psi.flat())
        grads.append(pv.gradient())
    assert np.abs(grads[1] - grads[0]).max() <= 1e-12 * np.abs(grads[0]).max()
