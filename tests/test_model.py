"""Host-side model builders: tree shapes, node order, leaf modes, DVR (CPU)."""
import numpy as np

from qutree_gb300.model import (HOBasis, balanced_tree, config_problem, config_tree_sop,
                                linear_bonds, mode_product, qr_orthogonal, random_wavefunction)


def test_node_order_and_modes_match_reference_linearisation():
    # balancedTree(8, ...): post-order walk, last child first
    # (Node::nextNode, src/TreeShape/Node.cpp:225-239); bottom node of mode k
    # is the k-th leaf in partition order (Tree::resetLeafModes).
    t = balanced_tree(8, 2, 2)
    shapes = [n.shape for n in t.nodes]
    assert len(shapes) == 15
    assert t.top.address == 14 and t.top.children == [13, 6]
    bottoms = [n for n in t.nodes if n.is_bottom]
    assert [n.address for n in bottoms] == [0, 1, 3, 4, 7, 8, 10, 11]
    assert [n.leaf_mode for n in bottoms] == [7, 6, 5, 4, 3, 2, 1, 0]
    for n in t.nodes:
        for k, c in enumerate(n.children):
            assert t.nodes[c].parent == n.address and t.nodes[c].child_idx == k
            assert c < n.address


def test_config_shapes():
    t, s = config_tree_sop(0)
    assert t.n_nodes == 15 and len(s) == 8 + 8 + 28
    assert sorted(set(n.shape for n in t.nodes)) == [(4, 4, 1), (4, 4, 4), (16, 4)]
    t, s = config_tree_sop(1)
    assert t.n_nodes == 127 and len(s) == 64 + 64 + 256
    assert linear_bonds(32, 64, 6) == [32, 38, 45, 51, 58, 64]
    assert max(n.size for n in t.nodes) == 58 * 58 * 64
    assert sum(n.size for n in t.nodes) * 16 / 1e6 > 60
    t, s = config_tree_sop(4)
    assert t.n_nodes == 31 and len(s) == 16 + 16 + 120
    t, s = config_tree_sop(3)
    assert max(n.size for n in t.nodes) == 86 * 86 * 96


def test_unbalanced_tree_and_clamping():
    t = balanced_tree(7, 5, 4)
    assert t.n_leaves == 7
    for n in t.nodes:
        if not n.is_bottom and not n.is_top:
            assert n.d_up <= int(np.prod(n.shape[:-1]))
    t = balanced_tree(48, 8, 24)
    assert t.n_leaves == 48 and t.top.d_up == 1


def test_ho_dvr():
    b = HOBasis(16, omega=1.0)
    # grid symmetric about r0 and ascending
    assert np.all(np.diff(b.x) > 0) and abs(b.x.sum()) < 1e-10
    assert np.allclose(b.kin, b.kin.T)
    # kinetic + harmonic potential has the HO ladder as lowest levels
    H = b.kin + np.diag(0.5 * b.x ** 2)
    w = np.linalg.eigvalsh(H)
    assert np.allclose(w[:5], np.arange(5) + 0.5, atol=1e-8)


def test_qr_orthogonal_preserves_state():
    t = balanced_tree(4, 3, 2)
    rng = np.random.default_rng(3)
    from qutree_gb300.model import TensorTree
    raw = TensorTree(t, [rng.standard_normal(n.shape) + 1j * rng.standard_normal(n.shape)
                         for n in t.nodes])
    q = qr_orthogonal(raw, rescale=False)
    qs = qr_orthogonal(raw)
    for n in t.nodes:
        if n.is_top:
            continue
        m = q.tensors[n.address].reshape((-1, n.d_up), order="F")
        assert np.allclose(m.conj().T @ m, np.eye(n.d_up), atol=1e-12)

    # state unchanged: contract both trees to the dense vector
    def dense(tt):
        vals = {}
        for n in t.nodes:
            phi = tt.tensors[n.address]
            if n.is_bottom:
                vals[n.address] = phi
            else:
                a, b = (vals[c] for c in n.children)
                vals[n.address] = np.einsum("xA,yB,ABj->xyj", a.reshape(-1, a.shape[-1]),
                                            b.reshape(-1, b.shape[-1]), phi).reshape(-1, n.d_up)
        return vals[t.top.address]

    assert np.allclose(dense(raw), dense(q), atol=1e-10)
    # the rescaled variant is the same state up to its norm
    a, b = dense(raw).ravel(), dense(qs).ravel()
    assert abs(abs(np.vdot(a, b)) / (np.linalg.norm(a) * np.linalg.norm(b)) - 1.0) < 1e-12


def test_random_wavefunction_is_normalised_and_seeded():
    t, s, psi = config_problem(0)
    _, _, psi2 = config_problem(0)
    assert np.array_equal(psi.flat(), psi2.flat())
    assert abs(np.linalg.norm(psi.tensors[-1]) - 1.0) < 1e-14
