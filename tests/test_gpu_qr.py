"""qrOrthogonal on the device (qt_qr_orthogonal) against the host
restatement (model.qr_orthogonal: numpy's Householder QR, LAPACK's gauge)
on seeded non-orthonormal wavefunctions.  The two gauges differ by a
unitary per node (the device reflectors map a column to
-e^{i arg x_0} |x| e_1, LAPACK's and Eigen's to a real multiple), and a
node's tensor is written in its children's gauge.  The comparison therefore
carries the relative gauge bottom-up: every child's D = Q_host^H Q_device is
applied along the child's index of its parent's device tensor before the
parent is compared.  Checked:
- every non-top node orthonormal (Q^H Q = I) within 1e-13;
- every non-top node's projector Q Q^H (in the host's gauge of its
  children) within 1e-12 of the host's, and its D unitary;
- the top node (in the host's gauge) within 1e-12 relative of the host's;
- the energy of the state (oracle sweep) within 1e-12 relative;
- on a tree small enough to expand, the dense state within 1e-12."""
import numpy as np
import pytest

import oracle as O
from qutree_gb300 import qtgpu
from qutree_gb300.model import (MLO, OP_DENSE, SOP, HOBasis, OperatorTable, TensorTree, Tree, _Build,
                                balanced_tree, config_problem, coupled_oscillators, mode_product, qr_orthogonal)

pytestmark = pytest.mark.gpu


def raw_wavefunction(tree, seed):
    """i.i.d. complex N(0,1) node tensors scaled to unit Frobenius norm (not orthonormal)."""
    rng = np.random.default_rng(seed)
    ts = []
    for n in tree.nodes:
        t = (rng.standard_normal(n.size) + 1j * rng.standard_normal(n.size)) / np.sqrt(2 * n.size)
        ts.append(t.reshape(n.shape, order="F"))
    return TensorTree(tree, ts)


def device_qr(tree, sop, psi):
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED)
    try:
        h.upload(psi.flat())
        h.qr_orthogonal()
        return TensorTree.from_flat(tree, h.psi())
    finally:
        h.close()


def dense(tree, psi):
    """The state as one vector (small trees): contract bottom-up."""
    vec = {}
    for n in tree.nodes:
        t = psi.tensors[n.address]
        if n.is_bottom:
            vec[n.address] = t.reshape((-1, n.d_up), order="F")
            continue
        m = t
        for k, c in enumerate(n.children):
            m = np.moveaxis(np.tensordot(vec[c], m, axes=([1], [k])), 0, k)
        # the children's physical indices now stand in place of their bonds
        vec[n.address] = m.reshape((-1, n.d_up), order="F")
    return vec[tree.top.address].ravel(order="F")


def check(tree, sop, psi0, tol=1e-12):
    ref = qr_orthogonal(psi0, rescale=False)
    got = device_qr(tree, sop, psi0)
    gauge = {}
    for n in tree.nodes:
        t = got.tensors[n.address]
        for k, c in enumerate(n.children):  # into the host's gauge of the children
            t = mode_product(gauge[c], t, k)
        if n.is_top:
            assert np.abs(t - ref.tensors[n.address]).max() <= tol * np.abs(ref.tensors[n.address]).max()
            continue
        q = t.reshape((-1, n.d_up), order="F")
        qh = ref.tensors[n.address].reshape((-1, n.d_up), order="F")
        qd = got.tensors[n.address].reshape((-1, n.d_up), order="F")
        assert np.abs(qd.conj().T @ qd - np.eye(n.d_up)).max() <= 1e-13
        assert np.abs(q @ q.conj().T - qh @ qh.conj().T).max() <= tol
        d = qh.conj().T @ q  # q = qh d
        assert np.abs(d.conj().T @ d - np.eye(n.d_up)).max() <= 1e-12
        gauge[n.address] = d
    e_got = O.derivative(tree, sop, got.flat(), want_mats=False).energy
    e_ref = O.derivative(tree, sop, ref.flat(), want_mats=False).energy
    assert abs(e_got - e_ref) <= tol * max(1.0, abs(e_ref))
    return got, ref


@pytest.mark.parametrize("cfg", [0, 4])
def test_qr_orthogonal_config(cfg):
    tree, sop, _ = config_problem(cfg)
    check(tree, sop, raw_wavefunction(tree, 40 + cfg))


def test_qr_orthogonal_ternary_tree():
    groups = [_Build([3, 3, 3, 3], [_Build([4, 3], leaf=True) for _ in range(3)]) for _ in range(3)]
    tree = Tree(_Build([3, 3, 3, 1], groups))
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=np.random.default_rng(3),
                              omega=1.0)
    check(tree, sop, raw_wavefunction(tree, 7))


def test_qr_orthogonal_keeps_the_dense_state():
    tree = balanced_tree(4, 4, 3)
    ops = OperatorTable()
    b = HOBasis(4, omega=1.0)
    sop = SOP(ops)
    sop.push_back(MLO([(0, ops.add("k", OP_DENSE, b.kin))]), 1.0)
    psi0 = raw_wavefunction(tree, 11)
    got, ref = check(tree, sop, psi0)
    v0, v1 = dense(tree, psi0), dense(tree, got)
    assert np.abs(v1 - v0).max() <= 1e-12 * np.abs(v0).max()


def test_qr_orthogonal_needs_a_wavefunction():
    tree, sop, _ = config_problem(0)
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_COMPRESSED)
    try:
        with pytest.raises(qtgpu.QtError, match="QT_ERR_STATE"):
            h.qr_orthogonal()
    finally:
        h.close()
