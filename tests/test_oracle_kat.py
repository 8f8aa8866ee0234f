"""The oracle against QuTree's own known-answer tests (CPU).

Each test restates one of the reference's gtest cases for the hot path
(file:line given per test) and runs it on the CPU oracle, pinning the
oracle to the reference's behaviour."""
import numpy as np
import pytest

import oracle as O
from qutree_gb300.model import (MLO, OP_DENSE, OP_DIAG, SOP, HOBasis, OperatorTable,
                                balanced_tree, hartree_wavefunction)

SMTEPS = 1e-7  # tests/test_SparseMatrixTree.cpp:10 (the checks below use 1e-12)


def _half_identity_problem():
    """SparseMatrixFactory (tests/test_SparseMatrixTree.cpp:12-39):
    balancedTree(8,2,2), Hartree-product state, MLO = 0.5*I on leaves 0, 3."""
    tree = balanced_tree(8, 2, 2)
    basis = HOBasis(2, omega=1.0, r0=0.0, wfr0=1.0, wfomega=0.0)
    psi = hartree_wavefunction(tree, 1993, lambda m: basis)
    ops = OperatorTable()
    x = ops.add("x", OP_DENSE, 0.5 * np.eye(2))
    sop = SOP(ops)
    sop.push_back(MLO([(0, x), (3, x)]), 1.0)
    return tree, sop, psi


def _sparse_mats(tree, sop, flat):
    offs = O.sparse_offsets(tree, sop)
    return offs


def test_sparse_tree_sizes():
    # TEST(SparseMatrixTree, TreeMarker) tests/test_SparseMatrixTree.cpp:41-46
    tree = balanced_tree(7, 4, 2)
    assert len(tree.sparse_tree([3, 4])) == 7
    # TEST_F(SparseMatrixFactory, TreeMarker_NoTail) :48-52
    tree8 = balanced_tree(8, 2, 2)
    assert len(tree8.sparse_tree([0, 3], tail=False)) == 5
    # TEST_F(SparseMatrixFactory, Constructor) :89-92
    assert len(tree8.sparse_tree([0, 3])) == 6


def test_represent_half_identity():
    # TEST_F(SparseMatrixFactory, Represent) tests/test_SparseMatrixTree.cpp:54-68
    tree, sop, psi = _half_identity_problem()
    r = O.derivative(tree, sop, psi.flat())
    offs = O.sparse_offsets(tree, sop)
    stree = tree.sparse_tree([0, 3])
    mats = [r.hmat[offs[(0, a)]:offs[(0, a)] + tree.nodes[a].d_up ** 2] for a in stree]
    half = (0.5 * np.eye(2)).ravel(order="F")
    for k in range(4):
        assert np.abs(mats[k] - half).max() < 1e-12
    assert np.abs(mats[4] - 0.5 * half).max() < 1e-12
    assert np.abs(mats[5]).max() == 0.0  # the top is not represented


def test_meanfield_half_identity():
    # TEST_F(SparseMatrixFactory, contraction) tests/test_SparseMatrixTree.cpp:70-87
    tree, sop, psi = _half_identity_problem()
    r = O.derivative(tree, sop, psi.flat())
    offs = O.sparse_offsets(tree, sop)
    stree = tree.sparse_tree([0, 3])
    mats = [r.hcon[offs[(0, a)]:offs[(0, a)] + tree.nodes[a].d_up ** 2] for a in stree]
    x = np.zeros(4, complex)
    x[0] = 0.5
    for k in range(4):
        assert np.abs(mats[k] - x).max() < 1e-12
    x[0] = 1.0
    assert np.abs(mats[4] - x).max() < 1e-12
    assert abs(mats[5][0] - 1.0) < 1e-12


def _kin_sop(tree):
    ops = OperatorTable()
    sop = SOP(ops)
    for m in range(tree.n_leaves):
        p = tree.leaf_dim(m)
        op = ops.add(("k", p), OP_DENSE, HOBasis(p).kin)
        sop.push_back(MLO([(m, op)]), 1.0)
    return sop


def test_density_hartree():
    # TEST(MatrixTreeFunctions, Density) tests/test_MatrixTree.cpp:69-89
    tree = balanced_tree(7, 5, 4)
    basis = HOBasis(5, omega=1.0, r0=0.0, wfr0=1.0, wfomega=0.0)
    psi = hartree_wavefunction(tree, 1923, lambda m: basis)
    r = O.derivative(tree, _kin_sop(tree), psi.flat())
    ro = 0
    for n in tree.nodes:
        d = n.d_up
        R = r.rho[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
        if n.is_top:
            continue
        expect = np.zeros((d, d))
        expect[0, 0] = 1.0
        assert np.abs(np.abs(R) - expect).max() < 1e-12


def test_spectral_decomposition_hartree():
    # TEST(MatrixTreeFunctions, SpectralDecompositionTree_Calc) tests/test_MatrixTree.cpp:91-104
    tree = balanced_tree(12, 2, 2)
    basis = HOBasis(2, omega=1.0, r0=0.0, wfr0=1.0, wfomega=0.0)
    psi = hartree_wavefunction(tree, 1993, lambda m: basis)
    r = O.derivative(tree, _kin_sop(tree), psi.flat())
    ro = 0
    for n in tree.nodes:
        d = n.d_up
        R = r.rho[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
        if n.is_top:
            continue
        w, _ = O.herm_eig(R)
        assert abs(w[1] - 1.0) < 1e-12


def test_regularised_inverse_identity():
    # TEST(MatrixTreeFunctions, SpectralDecompositionTree_Inverse) tests/test_MatrixTree.cpp:106-128
    rng = np.random.default_rng(1993)
    for d in (1, 2, 4, 7, 16):
        m = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
        H = m @ m.conj().T
        w, U = O.herm_eig(H)
        f = 1.0 / (w + 1e-10 * np.exp(-w / 1e-10))
        Hinv = (U * f) @ U.conj().T
        assert np.abs(Hinv @ H - np.eye(d)).max() < 1e-8


def test_herm_eig_against_numpy():
    rng = np.random.default_rng(7)
    for d in (1, 3, 8, 33, 64):
        a = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
        a = a + a.conj().T
        w, U = O.herm_eig(a)
        assert np.abs(w - np.linalg.eigvalsh(a)).max() < 1e-11 * max(1, np.abs(w).max())
        assert np.abs(U @ np.diag(w) @ U.conj().T - a).max() < 1e-11 * max(1, np.abs(w).max())
        assert np.all(U[0].real >= 0)  # phase convention
        inv = O.inverse(a)
        assert np.abs(inv @ a - np.eye(d)).max() < 1e-9


def _tensor_c():
    # TensorFactory::CreateTensorC (tests/test_Tensor.cpp:38-58)
    C = np.zeros((2, 2, 2), complex, order="F")
    C2 = np.zeros((2, 2, 2), complex, order="F")
    for b in range(2):
        for a in range(2):
            for c in range(2):
                C[b, a, c] = a * 1j
                C2[b, a, c] = c * 1j
    return C, C2


def test_hole_product_closed_form():
    # TEST_F(TensorFactory, HoleProduct) tests/test_Tensor.cpp:184-194
    C, _ = _tensor_c()
    for be in (O.LOOPS, O.BLAS):
        s = O.hole_product(C.ravel(order="F"), C.ravel(order="F"), 2, 2, 2, 2, backend=be)
        s = s.reshape((2, 2), order="F")
        for i in range(2):
            for j in range(2):
                assert abs(abs(s[i, j]) - 4.0 * i * j) < 1e-14


def test_dot_product_closed_form():
    # TEST_F(TensorFactory, DotProduct) tests/test_Tensor.cpp:196-206
    _, C2 = _tensor_c()
    for be in (O.LOOPS, O.BLAS):
        s = O.hole_product(C2.ravel(order="F"), C2.ravel(order="F"), 4, 2, 2, 1, backend=be)
        s = s.reshape((2, 2), order="F")
        for i in range(2):
            for j in range(2):
                assert abs(abs(s[i, j]) - 4.0 * i * j) < 1e-14


@pytest.fixture(params=["naive", "openblas"])
def blas(request):
    if request.param == "openblas":
        if O.attach_openblas(fast=False) is None:
            pytest.skip("no OpenBLAS found")
    else:
        O.detach_blas(fast=False)
    yield request.param
    O.detach_blas(fast=False)


def test_tensorblas_mode_products_agree(blas):
    # TensorBLASFactory matrixTensor tests (tests/test_TensorBLAS.cpp:60-119):
    # zgemm path == Fortran matvec path == loop path, every mode.
    rng = np.random.default_rng(129123)
    dim = 16
    A = rng.uniform(-1, 1, dim ** 3).astype(complex)
    S = rng.uniform(-1, 1, dim * dim).astype(complex)
    for mode in range(3):
        before, after = dim ** mode, dim ** (2 - mode)
        c1 = O.mode_product(S, A, before, dim, dim, after, backend=O.LOOPS)
        c2 = O.mode_product(S, A, before, dim, dim, after, backend=O.BLAS)
        ref = np.einsum("ja,bac->bjc", S.reshape((dim, dim), order="F"),
                        A.reshape((before, dim, after), order="F")).ravel(order="F")
        assert np.abs(c1 - ref).max() < 1e-12
        assert np.abs(c2 - ref).max() < 1e-12
    # rectangular (matrixTensor1): activeC != activeB
    h = rng.uniform(-1, 1, 5 * dim).astype(complex)
    c1 = O.mode_product(h, A, dim, dim, 5, dim, backend=O.LOOPS)
    ref = np.einsum("ja,bac->bjc", h.reshape((5, dim), order="F"),
                    A.reshape((dim, dim, dim), order="F")).ravel(order="F")
    assert np.abs(c1 - ref).max() < 1e-12


def test_tensorblas_contractions_agree(blas):
    # TEST_F(TensorBLASFactory, contraction) tests/test_TensorBLAS.cpp:123-137
    rng = np.random.default_rng(129124)
    dim = 16
    A = rng.uniform(-1, 1, dim ** 3).astype(complex)
    B = rng.uniform(-1, 1, dim ** 3).astype(complex)
    for mode in range(3):
        before, after = dim ** mode, dim ** (2 - mode)
        s1 = O.hole_product(A, B, before, dim, dim, after, backend=O.LOOPS)
        s2 = O.hole_product(A, B, before, dim, dim, after, backend=O.BLAS)
        ref = np.einsum("bic,bjc->ij", A.reshape((before, dim, after), order="F").conj(),
                        B.reshape((before, dim, after), order="F")).ravel(order="F")
        assert np.abs(s1 - ref).max() < 1e-11
        assert np.abs(s2 - ref).max() < 1e-11


def test_oracle_cmf_energy_converges_with_the_step():
    # fixed-step constant-mean-field propagation conserves the energy better
    # as dt shrinks (second-order scheme)
    from qutree_gb300.model import config_problem
    tree, sop, psi = config_problem(0)
    flat = psi.flat()
    e0 = O.derivative(tree, sop, flat).energy
    d = []
    for dt, n in ((2.0, 10), (1.0, 20)):
        y = O.cmf(tree, sop, flat, dt, n, 1)
        d.append(abs(O.derivative(tree, sop, y).energy - e0))
    assert d[1] < d[0] / 3.5
