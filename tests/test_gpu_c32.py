"""Complex64 arithmetic (QT_PREC_C32): every contraction in complex FP32 on
the FP32 pipe, checked against the complex128 oracle at tolerances stated
for FP32 (unit roundoff 2^-24 = 6e-8; reductions of up to a few thousand
products): energies and density matrices within TOL_C32 relative, the
rho-weighted derivative within DER_C32 relative to its largest entry.  The
complex64 variants of the batched forest and of the differentiation
workload run here too.  What these errors become along a long propagation
is measured by bench.py's precision study."""
import numpy as np
import pytest

import oracle as O
from helpers import deriv_errors, rel_err
from qutree_gb300 import qtgpu
from qutree_gb300.model import batched_problem, config_problem, forest, forest_psi, forest_sop

pytestmark = pytest.mark.gpu

TOL_C32 = 2e-5   # energy, density matrices, represent / mean-field matrices
DER_C32 = 2e-4   # rho-weighted derivative (projector cancellations)

PLANS = [qtgpu.QT_PLAN_REFERENCE, qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PLAN_COMPRESSED]


def _compare_c32(tree, sop, psi, flavour, phase=1.0):
    flat = psi.flat()
    r = O.derivative(tree, sop, flat, phase=phase)
    hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour)
    try:
        dpsi = qtgpu.Derivative(hrep, flat, phase)
        e = hrep.energy()
        de = abs(e - r.energy) / max(1.0, abs(r.energy))
        drho = rel_err(hrep.matrices(qtgpu.QT_MAT_RHO), r.rho)
        err, noise = deriv_errors(tree, dpsi, r.dpsi, r.rho)
        print(f"c32 flavour={flavour:#x}: dE {de:.2e} rho {drho:.2e} dpsi {err:.2e} noise {noise:.2e}")
        assert de <= TOL_C32
        assert drho <= TOL_C32
        if flavour & 0xFF != qtgpu.QT_PLAN_COMPRESSED:
            assert rel_err(hrep.matrices(qtgpu.QT_MAT_HMAT), r.hmat) <= TOL_C32
            assert rel_err(hrep.matrices(qtgpu.QT_MAT_HCON), r.hcon) <= TOL_C32
        assert err <= DER_C32 and noise <= DER_C32
        # fixed summation orders: a second sweep is bit-identical
        hrep.derivative(phase)
        assert np.array_equal(hrep.dpsi(), dpsi)
    finally:
        hrep.close()


@pytest.mark.parametrize("cfg", [0, 4])
@pytest.mark.parametrize("plan", PLANS)
@pytest.mark.parametrize("prec", [qtgpu.QT_PREC_C32, qtgpu.QT_PREC_TF32X3])
def test_c32_sweep(cfg, plan, prec):
    """Complex FP32 on the FP32 pipe, and with the mode products as
    split-TF32 on the tensor cores: both within the complex64 tolerances."""
    tree, sop, psi = config_problem(cfg)
    _compare_c32(tree, sop, psi, plan | prec, phase=np.exp(0.3j))


def test_tf32x3_full_size():
    """The 64-mode workload: split-TF32 tensor-core mode products against the
    complex128 plan on the same plan flavour."""
    tree, sop, psi = config_problem(1)
    out = {}
    for prec in (0, qtgpu.QT_PREC_C32, qtgpu.QT_PREC_TF32X3):
        h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED | prec)
        try:
            d = qtgpu.Derivative(h, psi.flat())
            out[prec] = (d, h.energy(), h.matrices(qtgpu.QT_MAT_RHO))
        finally:
            h.close()
    d0, e0, rho = out[0]
    for prec in (qtgpu.QT_PREC_C32, qtgpu.QT_PREC_TF32X3):
        d1, e1, _ = out[prec]
        err, noise = deriv_errors(tree, d1, d0, rho)
        print(f"64-mode prec={prec:#x}: dE {abs(e1 - e0) / abs(e0):.2e} dpsi {err:.2e} noise {noise:.2e}")
        assert abs(e1 - e0) <= TOL_C32 * abs(e0)
        assert err <= DER_C32 and noise <= DER_C32


@pytest.mark.parametrize("plan", [qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PLAN_COMPRESSED,
                                  qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_TF32X3])
def test_c32_forest_of_uneven_trees(plan):
    """The complex64 variant of the batched workload: 24 uneven trees in one
    plan, each tree's energy and derivative against its own oracle sweep."""
    trees, sops, psis = batched_problem(24)
    f, node_off, mode_off = forest(trees)
    prec = qtgpu.QT_PREC_C32 if not plan & qtgpu.QT_PREC_TF32X3 else 0
    hrep = qtgpu.HamiltonianRepresentation(forest_sop(sops, mode_off), f, flavour=plan | prec)
    try:
        d = qtgpu.Derivative(hrep, forest_psi(f, psis).flat())
        energies = hrep.energies()
        off = f.offsets()
        worst_e = worst_d = 0.0
        for k, (t, s, p) in enumerate(zip(trees, sops, psis)):
            r = O.derivative(t, s, p.flat())
            worst_e = max(worst_e, abs(energies[k] - r.energy) / max(1.0, abs(r.energy)))
            seg = d[off[node_off[k]]:off[node_off[k] + t.n_nodes]]
            err, noise = deriv_errors(t, seg, r.dpsi, r.rho)
            worst_d = max(worst_d, err, noise)
        print(f"c32 forest plan={plan}: dE {worst_e:.2e} dpsi {worst_d:.2e}")
        assert worst_e <= TOL_C32 and worst_d <= DER_C32
    finally:
        hrep.close()


@pytest.mark.parametrize("plan", [qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PLAN_COMPRESSED])
def test_c32_gradient_matches_finite_differences(plan):
    """The complex64 variant of the differentiation workload: the library's
    dE/dPhi^* in complex FP32 against central differences (h = 1e-6) of the
    exact (float64) energy along random directions; relative agreement
    within 1e-4 (FP32 rounding of the gradient itself)."""
    from tree_energy import fd_directional
    tree, sop, psi = config_problem(4)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=plan | qtgpu.QT_PLAN_GRADIENT | qtgpu.QT_PREC_C32)
    try:
        qtgpu.Derivative(h, psi.flat())
        g = h.gradient()
    finally:
        h.close()
    rng = np.random.default_rng(4321)
    worst = 0.0
    for _ in range(8):
        dirs = [rng.standard_normal(n.shape) + 1j * rng.standard_normal(n.shape) for n in tree.nodes]
        flat = np.concatenate([d.ravel(order="F") for d in dirs])
        analytic = 2.0 * np.vdot(g, flat).real
        fd = fd_directional(tree, sop, psi, dirs, h=1e-6)
        worst = max(worst, abs(analytic - fd) / max(1.0, abs(fd)))
    print(f"c32 gradient plan={plan}: worst FD deviation {worst:.2e}")
    assert worst <= 1e-4
