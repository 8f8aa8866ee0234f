"""The tensor-core sums of products (QT_PREC_DF64_TC) at the level of a
whole sweep, on the CPU: the plan interpreter (tests/plan_emulator.py) runs every
eligible mode product, hole product and accumulation through the same digit arithmetic
as qt_umma.cu (double-float operands, seven signed digits from error-free
splits against row exponents, exact level sums for L <= 2, one
float32-rounded sum of the levels 3..6) and the sweep is compared with the
oracle at the double-float tolerances the GPU tests use."""
import numpy as np
import pytest

import oracle as O
from helpers import deriv_errors, rel_err, rho_weighted
from plan_emulator import PlanView, oz_mode_product
from qutree_gb300.model import balanced_tree, config_problem, coupled_oscillators, random_wavefunction

TENSOR = 0x8000
TOL_DF = 1e-11


def test_digit_mode_product_within_bound():
    rng = np.random.default_rng(4)
    for bef, ain, aout, aft in ((3, 16, 16, 5), (1, 40, 33, 7), (6, 64, 64, 2)):
        h = (rng.standard_normal((aout, ain)) + 1j * rng.standard_normal((aout, ain))) * 10.0 ** rng.uniform(-3, 3)
        x = rng.standard_normal((bef, ain, aft)) + 1j * rng.standard_normal((bef, ain, aft))
        x[:, : ain // 3] *= 1e-6  # rows with a wide dynamic range
        got = oz_mode_product(h, x)
        want = np.einsum("ja,bac->bjc", h, x)
        xmax = np.abs(np.moveaxis(x, 1, -1)).max(axis=-1)  # per row (b, c)
        hmax = np.abs(h).max(axis=1)
        bound = 2.0 ** -43 * ain * np.sqrt(2) * xmax[:, None, :] * hmax[None, :, None]
        assert np.all(np.abs(got - want) <= bound)


def _check(tree, sop, psi, flavour, tol=TOL_DF, noise_tol=1e-11):
    flat = psi.flat()
    r = O.derivative(tree, sop, flat)
    pv = PlanView(tree, sop, flavour | TENSOR, prec=1)
    pv.run(flat)
    h00, s00 = pv.energy_parts()
    assert abs(h00.real / s00.real - r.energy) < tol * max(1, abs(r.energy))
    assert rel_err(rho_weighted(tree, pv.dpsi(), r.rho), rho_weighted(tree, r.dpsi, r.rho)) < tol
    err, noise = deriv_errors(tree, pv.dpsi(), r.dpsi, r.rho)
    print(f"emulated tensor-core sweep: dE {abs(h00.real / s00.real - r.energy):.2e} dpsi {err:.2e} noise {noise:.2e}")
    assert err <= tol and noise <= noise_tol
    # where the planner put contractions on the tensor cores (shapes 32..64)
    # the digit arithmetic ran: the plan without the tensor bit differs at
    # rounding level; elsewhere the two plans are the same
    exact = PlanView(tree, sop, flavour, prec=1)
    exact.run(flat)
    tc = len(pv.tables[40]) + len(pv.tables[53]) + len(pv.tables[57])
    assert np.array_equal(pv.dpsi(), exact.dpsi()) == (tc == 0)
    return tc


@pytest.mark.parametrize("flavour", [0, 1, 2])
def test_emulated_tensor_core_sweep_cfg0(flavour):
    # bonds 4, leaves 16: nothing qualifies for the tensor cores
    tree, sop, psi = config_problem(0)
    assert _check(tree, sop, psi, flavour) == 0


@pytest.mark.parametrize("flavour", [1, 2])
def test_emulated_tensor_core_sweep_bonds_36(flavour):
    # leaves of 40 points, bonds 36: mode products with 40 padded columns
    # (six level accumulators), hole products in 128-k chunks with four,
    # accumulations over 40 padded columns
    tree = balanced_tree(4, 40, 36)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(6),
                              omega=1.0)
    assert _check(tree, sop, random_wavefunction(tree, 6), flavour, tol=1e-10, noise_tol=1e-10) > 0


@pytest.mark.parametrize("flavour", [1, 2])
def test_emulated_tensor_core_sweep_cfg4(flavour):
    # bonds and leaves of 32: hole products and accumulations take the
    # digit arithmetic too (the GPU tolerance of the tensor-core plans)
    tree, sop, psi = config_problem(4)
    pv = PlanView(tree, sop, flavour | TENSOR, prec=1)
    assert len(pv.tables[52]) > 0 and len(pv.tables[57]) > 0
    _check(tree, sop, psi, flavour, tol=1e-10, noise_tol=1e-10)


@pytest.mark.parametrize("leaves,p,b,seed", [(7, 5, 4, 2), (5, 80, 12, 3)])
def test_emulated_tensor_core_sweep_random_trees(leaves, p, b, seed):
    # p = 80, bonds 12: the leaf products (k = 80) and the bonds below 32
    # stay on the FP32 pipe
    tree = balanced_tree(leaves, p, b)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(seed),
                              omega=1.0)
    _check(tree, sop, random_wavefunction(tree, seed), 2)


def test_emulated_tensor_core_forest():
    # five uneven trees in one compressed plan (bonds 4..24, leaves up to 32):
    # only the 32-point leaf products qualify for the digit arithmetic; each
    # tree's slice equals its own oracle sweep at the double-float tolerances
    from qutree_gb300.model import batched_problem, forest, forest_psi, forest_sop
    trees, sops, psis = batched_problem(5)
    f, node_off, mode_off = forest(trees)
    pv = PlanView(f, forest_sop(sops, mode_off), 2 | TENSOR, prec=1)
    pv.run(forest_psi(f, psis).flat())
    d = pv.dpsi()
    off = f.offsets()
    for k, (t, s, p) in enumerate(zip(trees, sops, psis)):
        r = O.derivative(t, s, p.flat())
        seg = d[off[node_off[k]]:off[node_off[k] + t.n_nodes]]
        err, noise = deriv_errors(t, seg, r.dpsi, r.rho)
        assert err <= TOL_DF and noise <= 1e-11
