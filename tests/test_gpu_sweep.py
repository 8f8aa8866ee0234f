"""Full H.Psi sweeps on the GPU through the C ABI against the oracle, for
both plan flavours and both arithmetics (complex128 on the FP64 pipe and
double-float on the FP32 pipe).

Tolerances (complex128 plans; double-float plans 10x looser, see TOL_DF):
every contraction result (density matrices, represent and
mean-field matrices, energy) within 1e-12 relative; the derivative compared
after multiplying each non-top node back by its density matrix (undoing the
regularised inverse, whose condition number amplifies rounding noise),
within 1e-12 relative on every node whose derivative is not identically
zero; on nodes whose SPFs span their whole space the projector (1-P)
vanishes and |dPsi rho| must stay below 1e-11 (rounding noise); the raw
derivative within 1e-13 x cond(rho) when no such node exists."""
import numpy as np
import pytest

import oracle as O
from helpers import deriv_errors, rel_err, rho_condition, rho_weighted
from qutree_gb300 import qtgpu
from qutree_gb300.model import (MLO, OP_DENSE, SOP, HOBasis, OperatorTable, balanced_tree,
                                batched_problem, config_problem, coupled_oscillators, forest,
                                forest_psi, forest_sop, hartree_wavefunction, random_wavefunction)

pytestmark = pytest.mark.gpu
# complex128 (FP64 pipe): unit roundoff 2^-53
TOL = 1e-12
RAW = 1e-13
# double-float (FP32 pipe): unit roundoff ~2^-48, so reductions of a few
# thousand products with cancellation carry up to ~1e-12
TOL_DF = 1e-11
RAW_DF = 3e-12
NOISE = 1e-11  # |dPsi rho| on nodes where (1-P) = 0 (rounding noise of a cancellation)
# double-float with the mode products on the tensor cores:
# the digit arithmetic's error is relative to the row maxima of its operands
# (2^-49 of the row scale per value, plus the fp32 rounding of the last level
# accumulator when bonds exceed 32), so where the projector cancels large
# terms the derivative carries up to ~1e-10 of its scale
TOL_TC = 1e-10
RAW_TC = 3e-11
NOISE_TC = 1e-10


def _compare(tree, sop, psi, flavour, phase=1.0, eps=1e-10):
    df = bool(flavour & (qtgpu.QT_PREC_DF64 | qtgpu.QT_PREC_DF64_TC))
    TOL, RAW = (TOL_DF, RAW_DF) if df else (globals()["TOL"], globals()["RAW"])
    NOISE = globals()["NOISE"]
    if flavour & qtgpu.QT_PREC_DF64_TC:
        TOL, RAW, NOISE = TOL_TC, RAW_TC, NOISE_TC
    flat = psi.flat()
    r = O.derivative(tree, sop, flat, eps=eps, phase=phase)
    hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=flavour, eps=eps)
    try:
        dpsi = qtgpu.Derivative(hrep, flat, phase)
        e = hrep.energy()
        assert abs(e - r.energy) <= TOL * max(1.0, abs(r.energy))
        rho = hrep.matrices(qtgpu.QT_MAT_RHO)
        assert rel_err(rho, r.rho) <= TOL
        if flavour & 0xFF == qtgpu.QT_PLAN_COMPRESSED:  # no per-term matrices
            with pytest.raises(qtgpu.QtError, match="QT_ERR_STATE"):
                hrep.matrices(qtgpu.QT_MAT_HMAT)
        else:
            assert rel_err(hrep.matrices(qtgpu.QT_MAT_HMAT), r.hmat) <= TOL
            assert rel_err(hrep.matrices(qtgpu.QT_MAT_HCON), r.hcon) <= TOL
        err, noise = deriv_errors(tree, dpsi, r.dpsi, r.rho)
        assert err <= TOL
        assert noise <= NOISE
        cond = rho_condition(tree, r.rho)
        if noise == 0.0:  # no node whose derivative is pure rounding noise
            assert rel_err(dpsi, r.dpsi) <= RAW * max(cond, 10.0)
        ri = hrep.matrices(qtgpu.QT_MAT_RHOINV)
        assert rel_err(ri, r.rhoinv) <= RAW * max(cond, 10.0)
        # second call on the same graph reproduces bit for bit
        hrep.derivative(phase)
        assert np.array_equal(hrep.dpsi(), dpsi)
        return hrep.stats()
    finally:
        hrep.close()


FLAVOURS = [qtgpu.QT_PLAN_REFERENCE, qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PLAN_COMPRESSED,
            qtgpu.QT_PLAN_REFERENCE | qtgpu.QT_PREC_DF64, qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64,
            qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64]


@pytest.mark.parametrize("flavour", FLAVOURS)
def test_sweep_cfg0(flavour):
    tree, sop, psi = config_problem(0)
    _compare(tree, sop, psi, flavour)


# mode products and accumulations with k <= 64 on the tensor cores (seven
# digits per operand, exact digit products and level sums): TOL_TC
TC_FLAVOURS = [qtgpu.QT_PLAN_REFERENCE | qtgpu.QT_PREC_DF64_TC, qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64_TC,
               qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC]


@pytest.mark.parametrize("cfg", [0, 4])
@pytest.mark.parametrize("flavour", TC_FLAVOURS)
def test_sweep_tensor_core_mode_products(cfg, flavour):
    tree, sop, psi = config_problem(cfg)
    _compare(tree, sop, psi, flavour)


def test_tensor_core_mode_products_with_wide_leaves():
    """Leaves of 80 grid points: their mode products (k = 80 > 64) stay on
    the FP32 pipe beside the tensor-core ones of the same stages."""
    tree = balanced_tree(4, 80, 12)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(8),
                              omega=1.0)
    psi = random_wavefunction(tree, 8)
    for fl in TC_FLAVOURS:
        _compare(tree, sop, psi, fl, phase=np.exp(0.3j))


@pytest.mark.parametrize("flavour", FLAVOURS)
def test_sweep_cfg4(flavour):
    tree, sop, psi = config_problem(4)
    _compare(tree, sop, psi, flavour)


@pytest.mark.parametrize("leaves,p,b,seed", [(5, 4, 3, 1), (7, 5, 4, 2), (12, 3, 2, 3), (16, 16, 12, 4),
                                             (3, 8, 8, 5), (2, 6, 6, 6)])
def test_sweep_random_trees(leaves, p, b, seed):
    tree = balanced_tree(leaves, p, b)
    rng = np.random.default_rng(seed)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    psi = random_wavefunction(tree, seed)
    for fl in FLAVOURS:
        _compare(tree, sop, psi, fl, phase=np.exp(0.3j))


def test_sweep_known_answer_half_identity():
    # tests/test_SparseMatrixTree.cpp:54-87 on the GPU: represent = 0.5 I / 0.25 I,
    # mean field = diag(0.5, 0) / diag(1, 0) / 1 for the Hartree-product state.
    tree = balanced_tree(8, 2, 2)
    basis = HOBasis(2, omega=1.0, r0=0.0, wfr0=1.0, wfomega=0.0)
    psi = hartree_wavefunction(tree, 1993, lambda m: basis)
    ops = OperatorTable()
    x = ops.add("x", OP_DENSE, 0.5 * np.eye(2))
    sop = SOP(ops)
    sop.push_back(MLO([(0, x), (3, x)]), 1.0)
    hrep = qtgpu.HamiltonianRepresentation(sop, tree)
    try:
        qtgpu.Derivative(hrep, psi.flat())
        hmat = hrep.matrices(qtgpu.QT_MAT_HMAT)
        hc = hrep.matrices(qtgpu.QT_MAT_HCON)
        assert hmat.size == 5 * 4 + 1  # five 2x2 matrices and the top's 1x1
        hm = hmat[:20].reshape(5, 4)
        half = (0.5 * np.eye(2)).ravel(order="F")
        for k in range(4):
            assert np.abs(hm[k] - half).max() < 1e-12
        assert np.abs(hm[4] - 0.5 * half).max() < 1e-12
        assert hmat[20] == 0.0  # the top is not represented
        x1 = np.array([0.5, 0, 0, 0])
        for k in range(4):
            assert np.abs(hc[4 * k:4 * k + 4] - x1).max() < 1e-12
        assert np.abs(hc[16:20] - 2 * x1).max() < 1e-12
        assert abs(hc[20] - 1.0) < 1e-12
    finally:
        hrep.close()


def test_multi_factor_terms():
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
    for fl in FLAVOURS:
        _compare(tree, sop, psi, fl)


def test_nodes_without_terms():
    tree = balanced_tree(8, 4, 3)
    ops = OperatorTable()
    b = HOBasis(4, omega=1.0)
    kin = ops.add("k", OP_DENSE, b.kin)
    x = ops.add("x", 1, b.x.astype(complex))
    sop = SOP(ops)
    sop.push_back(MLO([(0, kin)]), 1.0)
    sop.push_back(MLO([(1, x), (2, x)]), 0.3)
    psi = random_wavefunction(tree, 21)
    for fl in FLAVOURS:
        _compare(tree, sop, psi, fl)


def test_errors_are_reported_not_fatal():
    tree, sop, psi = config_problem(0)
    hrep = qtgpu.HamiltonianRepresentation(sop, tree)
    try:
        with pytest.raises(qtgpu.QtError, match="QT_ERR_STATE"):
            hrep.dpsi()  # no sweep yet
        hrep.upload(psi)
        hrep.derivative()
        assert np.isfinite(hrep.energy())
    finally:
        hrep.close()


@pytest.mark.parametrize("flavour", [qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PREC_DF64,
                                     qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64,
                                     qtgpu.QT_PLAN_COMPRESSED | qtgpu.QT_PREC_DF64_TC])
def test_forest_of_uneven_trees(flavour):
    # 24 trees of 8..48 modes, p in {8,16,32}, random bonds 4..24, one plan and
    # one graph; every tree's slice and energy equal its own oracle sweep
    df = bool(flavour & (qtgpu.QT_PREC_DF64 | qtgpu.QT_PREC_DF64_TC))
    tol = TOL_DF if df else TOL
    noise_tol = NOISE
    if flavour & qtgpu.QT_PREC_DF64_TC:
        tol, noise_tol = TOL_TC, NOISE_TC
    trees, sops, psis = batched_problem(24)
    f, node_off, mode_off = forest(trees)
    hrep = qtgpu.HamiltonianRepresentation(forest_sop(sops, mode_off), f, flavour=flavour)
    try:
        d = qtgpu.Derivative(hrep, forest_psi(f, psis).flat())
        energies = hrep.energies()
        assert len(energies) == len(trees)
        off = f.offsets()
        for k, (t, s, p) in enumerate(zip(trees, sops, psis)):
            r = O.derivative(t, s, p.flat())
            assert abs(energies[k] - r.energy) <= tol * max(1.0, abs(r.energy))
            seg = d[off[node_off[k]]:off[node_off[k] + t.n_nodes]]
            err, noise = deriv_errors(t, seg, r.dpsi, r.rho)
            assert err <= tol and noise <= noise_tol
    finally:
        hrep.close()


def test_checkpoint_round_trip(tmp_path):
    # qt_psi_save writes QuTree's TTre format; qt_psi_load reads it back
    from qutree_gb300 import formats
    tree, sop, psi = config_problem(0)
    hrep = qtgpu.HamiltonianRepresentation(sop, tree)
    try:
        hrep.upload(psi)
        p = str(tmp_path / "gpu.ttre")
        hrep.save(p)
        back = formats.read_tensor_tree(p, tree)
        assert np.array_equal(back.flat(), psi.flat())
        other = psi.copy()
        other.tensors[-1] = other.tensors[-1] * (0.5 - 0.5j)
        q = str(tmp_path / "host.ttre")
        formats.write_tensor_tree(q, other)
        hrep.load(q)
        hrep.derivative()
        hrep2 = qtgpu.HamiltonianRepresentation(sop, tree)
        try:
            ref = qtgpu.Derivative(hrep2, other.flat())
        finally:
            hrep2.close()
        assert np.array_equal(hrep.dpsi(), ref)
        tree4, _, psi4 = config_problem(4)
        r = str(tmp_path / "wrong.ttre")
        formats.write_tensor_tree(r, psi4)
        with pytest.raises(qtgpu.QtError, match="QT_ERR_SHAPE"):
            hrep.load(r)
    finally:
        hrep.close()


@pytest.mark.parametrize("prec", [qtgpu.QT_PREC_DF64, qtgpu.QT_PREC_DF64_TC])
def test_non_finite_device_input_is_reported(prec):
    # a NaN in a Psi uploaded from device memory (no host-side check) reaches
    # the energy through either arithmetic of the mode products
    import torch
    tree, sop, psi = config_problem(0)
    flat = psi.flat().copy()
    flat[3] = np.nan
    dev = torch.from_numpy(flat.view(np.float64)).cuda()
    hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED | prec)
    try:
        hrep.upload_device(dev.data_ptr())
        hrep.derivative()
        with pytest.raises(qtgpu.QtError, match="QT_ERR_NUMERIC"):
            hrep.energy()
    finally:
        hrep.close()
