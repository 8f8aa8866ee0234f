"""The 512-tree forest that bench.py times (uneven trees: 8..48 modes, p in
{8, 16, 32}, bonds 4..24, an own SOP per tree), every tree checked against
its own oracle sweep: energy, and the rho-weighted derivative of the tree's
slice of the forest derivative.  One plan and one graph per arithmetic; the
tolerances are those of the other sweep tests for each arithmetic."""
import numpy as np
import pytest

from forest_oracle import oracle_forest
from helpers import deriv_errors
from qutree_gb300 import qtgpu
from qutree_gb300.model import batched_problem, forest, forest_psi, forest_sop

pytestmark = pytest.mark.gpu
N_TREES = 512

# (flavour, energy and derivative tolerance, noise tolerance)
CASES = [
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64, 1e-11, 1e-11),
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC, 1e-10, 1e-10),
    (qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64, 1e-11, 1e-11),
    (qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_C32, 2e-4, 2e-4),
]


@pytest.fixture(scope="module")
def forest512():
    ref = oracle_forest(N_TREES)
    trees, sops, psis = batched_problem(N_TREES)
    f, node_off, mode_off = forest(trees)
    return trees, f, node_off, forest_sop(sops, mode_off), forest_psi(f, psis).flat(), ref


@pytest.mark.parametrize("flavour,tol,noise_tol", CASES)
def test_every_tree_of_the_bench_forest(forest512, flavour, tol, noise_tol):
    trees, f, node_off, sop, flat, ref = forest512
    hrep = qtgpu.HamiltonianRepresentation(sop, f, flavour=flavour)
    try:
        d = qtgpu.Derivative(hrep, flat)
        energies = hrep.energies()
    finally:
        hrep.close()
    assert len(energies) == N_TREES
    off = f.offsets()
    worst_e = worst_d = worst_n = 0.0
    for k, t in enumerate(trees):
        e, dref, rho = ref[k]
        worst_e = max(worst_e, abs(energies[k] - e) / max(1.0, abs(e)))
        seg = d[off[node_off[k]]:off[node_off[k] + t.n_nodes]]
        err, noise = deriv_errors(t, seg, dref, rho)
        worst_d, worst_n = max(worst_d, err), max(worst_n, noise)
    print(f"forest {N_TREES} flavour {flavour:#x}: dE {worst_e:.2e} dpsi {worst_d:.2e} noise {worst_n:.2e}")
    assert worst_e <= tol and worst_d <= tol and worst_n <= noise_tol
    assert np.all(np.isfinite(energies))
