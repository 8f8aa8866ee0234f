"""<Psi|H|Psi> / <Psi|Psi> of a tree tensor network in any gauge (test
infrastructure): bottom-up matrix elements with overlap matrices for the
subtrees a term does not touch, so node tensors need not be orthonormal.
Used to check the energy gradient by finite differences."""
import numpy as np

from qutree_gb300.model import mode_product


def _contract(phi_bra, phi_ket, mats, last):
    """Phi_bra^dag (x_k mats[k]) Phi_ket over all indices but the last."""
    x = phi_ket
    for k, m in enumerate(mats):
        if m is not None:
            x = mode_product(m, x, k)
    d = phi_bra.shape[-1]
    return phi_bra.reshape(-1, d, order="F").conj().T @ x.reshape(-1, d, order="F")


def energy(tree, sop, tensors):
    S = {}
    for n in tree.nodes:
        phi = tensors[n.address]
        if n.is_bottom:
            S[n.address] = _contract(phi, phi, [None], True)
        else:
            S[n.address] = _contract(phi, phi, [S[c] for c in n.children], True)
    top = tree.top.address
    norm = S[top][0, 0].real
    sub = {n.address: tree.subtree_modes(n.address) for n in tree.nodes}
    cache = {}  # (node, restriction of the term to the node's subtree) -> matrix

    def rep(term, a):
        restr = tuple((m, o) for (m, o) in term.factors if m in sub[a])
        if not restr:
            return S[a]
        key = (a, tuple(sorted(restr, key=lambda mo: mo[0])))
        if key in cache:
            return cache[key]
        n = tree.nodes[a]
        phi = tensors[a]
        if n.is_bottom:
            op = np.eye(n.shape[0], dtype=complex)
            for (m, o) in term.factors:
                if m == n.leaf_mode:
                    op = sop.ops.dense(o) @ op
            val = _contract(phi, phi, [op], True)
        else:
            val = _contract(phi, phi, [rep(term, c) for c in n.children], True)
        cache[key] = val
        return val

    total = 0.0
    for l, term in enumerate(sop.terms):
        total += (sop.coeffs[l] * rep(term, top)[0, 0]).real
    return total / norm


def fd_directional(tree, sop, psi, direction, h=1e-6):
    """Central difference of the energy along a direction (list of tensors)."""
    plus = [t + h * d for t, d in zip(psi.tensors, direction)]
    minus = [t - h * d for t, d in zip(psi.tensors, direction)]
    return (energy(tree, sop, plus) - energy(tree, sop, minus)) / (2 * h)
