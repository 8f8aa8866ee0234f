"""The 512-tree forest that bench.py times (uneven trees: 8..48 modes, p in
{8, 16, 32}, bonds 4..24, an own SOP per tree), every tree checked against
its own oracle sweep: energy, and the rho-weighted derivative of the tree's
slice of the forest derivative.  One plan and one graph per arithmetic.

The derivative's error grows with the condition number of the tree's
density matrices (cond up to 2e6 among these 512 trees, against 2e5 among
the first 24): rounding of rho of order u moves the regularised inverse by
u cond(rho).  Each tree is therefore held to max(tol, kappa cond(rho)), with
tol the tolerance of the other sweep tests for the arithmetic and kappa a
small multiple of its effective unit roundoff (largest err / cond measured
over the 512 trees: complex128 1.3e-17, double-float 3.8e-16 compressed and
1.6e-15 grouped, tensor-core double-float 5.8e-16, complex64 4.3e-9,
split-TF32 9.2e-9)."""
import numpy as np
import pytest

from forest_oracle import oracle_forest
from helpers import deriv_errors, rho_condition
from qutree_gb300 import qtgpu
from qutree_gb300.model import batched_problem, forest, forest_psi, forest_sop

pytestmark = pytest.mark.gpu
N_TREES = 512

# (flavour, energy tolerance, derivative tolerance, kappa)
CASES = [
    (qtgpu.QT_PLAN_COMPRESSED, 1e-12, 1e-12, 1e-16),
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64, 1e-11, 1e-11, 5e-15),
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC, 1e-10, 1e-10, 5e-15),
    (qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64, 1e-11, 1e-11, 5e-15),
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_C32, 2e-5, 2e-4, 5e-8),
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_TF32X3, 2e-5, 2e-4, 5e-8),
]


@pytest.fixture(scope="module")
def forest512():
    ref = oracle_forest(N_TREES)
    trees, sops, psis = batched_problem(N_TREES)
    f, node_off, mode_off = forest(trees)
    cond = [rho_condition(t, ref[k][2]) for k, t in enumerate(trees)]
    return trees, f, node_off, forest_sop(sops, mode_off), forest_psi(f, psis).flat(), ref, cond


@pytest.mark.parametrize("flavour,tol_e,tol,kappa", CASES)
def test_every_tree_of_the_bench_forest(forest512, flavour, tol_e, tol, kappa):
    trees, f, node_off, sop, flat, ref, cond = forest512
    hrep = qtgpu.HamiltonianRepresentation(sop, f, flavour=flavour)
    try:
        d = qtgpu.Derivative(hrep, flat)
        energies = hrep.energies()
    finally:
        hrep.close()
    assert len(energies) == N_TREES
    assert np.all(np.isfinite(energies))
    off = f.offsets()
    worst_e, worst = 0.0, (0.0, -1)
    for k, t in enumerate(trees):
        e, dref, rho = ref[k]
        worst_e = max(worst_e, abs(energies[k] - e) / max(1.0, abs(e)))
        seg = d[off[node_off[k]]:off[node_off[k] + t.n_nodes]]
        err, noise = deriv_errors(t, seg, dref, rho)
        ratio = max(err, noise) / max(tol, kappa * cond[k])
        worst = max(worst, (ratio, k))
    print(f"forest {N_TREES} flavour {flavour:#x}: dE {worst_e:.2e}, worst derivative error / bound "
          f"{worst[0]:.2f} (tree {worst[1]}, cond {cond[worst[1]]:.1e})")
    assert worst_e <= tol_e
    assert worst[0] <= 1.0
