"""The oracle against a dense-state evaluation of the same quantities (CPU).

An independent check of the restated sweep: on trees small enough to hold
Psi as a full array, energy, represent matrices, mean fields and the
projected H.Psi of every node are computed directly from their definitions
(tests/dense_reference.py) and compared with the oracle."""
import numpy as np
import pytest

import oracle as O
from dense_reference import Dense
from qutree_gb300.model import (balanced_tree, coupled_oscillators, random_wavefunction)

CASES = [
    # (leaves, p, bond, seed)
    (4, 4, 2, 11),
    (4, 5, 3, 12),
    (5, 3, 2, 13),   # unbalanced: a dangling bottom node is carried up
    (6, 3, 2, 14),
    (8, 3, 2, 15),
]


@pytest.mark.parametrize("leaves,p,b,seed", CASES)
def test_oracle_matches_dense(leaves, p, b, seed):
    tree = balanced_tree(leaves, p, b)
    rng = np.random.default_rng(seed)
    sop = coupled_oscillators(tree, n_pairs=None, coupling=0.2, quartic=0.1, rng=rng, omega=1.0)
    psi = random_wavefunction(tree, seed)
    r = O.derivative(tree, sop, psi.flat())
    D = Dense(tree, sop, psi)
    # energy
    assert abs(r.energy - D.energy()) < 1e-12 * max(1.0, abs(D.energy()))
    # represent and mean-field matrices of every active (term, node)
    offs = O.sparse_offsets(tree, sop)
    for (l, a), o in offs.items():
        n = tree.nodes[a]
        dd = n.d_up * n.d_up
        if not n.is_top:
            hm = r.hmat[o:o + dd].reshape((n.d_up, n.d_up), order="F")
            ref = D.hmat(l, a)
            assert np.abs(hm - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
        hc = r.hcon[o:o + dd].reshape((n.d_up, n.d_up), order="F")
        ref = D.hcon(l, a) if not n.is_top else np.eye(n.d_up)
        assert np.abs(hc - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    # derivative: dPsi x_last rho = -i (1-P) X  (non-top),  dPsi = -i X  (top)
    off = tree.offsets()
    ro = 0
    for n in tree.nodes:
        d = n.d_up
        R = r.rho[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
        dpsi = r.dpsi[off[n.address]:off[n.address + 1]].reshape((-1, d), order="F")
        # node-shaped arrays are indexed [a_1..a_k, j]; flatten column-major like the tensor
        Xf = np.asarray(D.x_node(n.address))
        Xf = Xf.reshape((-1, d), order="F")
        phi = psi.tensors[n.address].reshape((-1, d), order="F")
        if n.is_top:
            ref = -1j * Xf
            got = dpsi
        else:
            Pm = phi @ np.linalg.solve(phi.conj().T @ phi, phi.conj().T @ Xf)
            ref = -1j * (Xf - Pm)
            got = dpsi @ R.T
        scale = max(1e-300, np.abs(ref).max(), 1e-3 * np.abs(D.HPsi).max())
        assert np.abs(got - ref).max() / scale < 1e-11, (n.address, np.abs(got - ref).max() / scale)
