"""CPU restatement of QuTree's SCF / Krylov sweep with tail=false corrections.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU SCF
(qt_scf) and by bench.py's CPU-baseline leg; the product path never imports
this module.

Follows, routine by routine (numpy, complex128, no shortcuts):
  sparse trees without tail     src/TreeClasses/SparseTree.cpp:34-84
  active-neighbour counts       src/TreeClasses/HamiltonianRepresentation.cpp:117-134,
                                include/TreeOperators/ActiveCounter.h:17-33
  buildUp / representLayer      include/TreeClasses/HamiltonianRepresentation.h:89-104,
                                include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:17-54
  buildDown / contractionLayer  include/TreeClasses/HamiltonianRepresentation.h:106-127,
                                include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:146-190
  buildUpCorrection             src/TreeClasses/HamiltonianRepresentation.cpp:136-161
  buildDownCorrection           src/TreeClasses/HamiltonianRepresentation.cpp:163-203
  TreeFunctions::apply          include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:302-353
  applyHole                     include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:363-384
  SCF apply (effective H)       src/Applications/SCF.cpp:36-84
  solveKrylovSpace              src/Applications/SCF.cpp:138-195
  imaginaryTimePropagation      src/Applications/SCF.cpp:197-222
  diagonalizeKrylov             src/Applications/SCF.cpp:224-236
  sweep order, adjacentIndex    src/Applications/SCF.cpp:14-33,238-256
  scf driver                    src/Applications/SCF.cpp:267-341
  qr(Tensor, mode)              include/Core/Tensor_Implementation.h:863-869 (Householder, thin Q)

Parity of this restatement is pinned by independent checks in the tests
(with the wavefunction in canonical gauge toward the top, <Phi_top|H_eff|Phi_top>
equals the full tree energy; the SCF converges to the exact ground state of
small coupled-oscillator problems); QuTree has no SCF test of its own.
"""
from __future__ import annotations

import numpy as np

from qutree_gb300.model import OP_DENSE


def _mp(h, x, k):
    """C = h x_k x (matrixTensor)."""
    out = np.tensordot(h, x, axes=([1], [k]))
    return np.moveaxis(out, 0, k)


def _hole(a, b, k):
    """S(i, j) = sum over all indices but k of conj(a[.., i, ..]) b[.., j, ..] (contraction)."""
    am = np.moveaxis(a, k, -1).reshape(-1, a.shape[k])
    bm = np.moveaxis(b, k, -1).reshape(-1, b.shape[k])
    return am.conj().T @ bm


def _full(a, b):
    """fullContraction: trace of the dot product = sum conj(a) b."""
    return np.vdot(a.ravel(), b.ravel())


class SCFOracle:
    """HamiltonianRepresentation(H, tree, tree, tail=false) plus the SCF driver."""

    def __init__(self, tree, sop):
        self.tree, self.sop = tree, sop
        self.nodes = tree.nodes
        self.L = len(sop.terms)
        self.stree = [self._sparse_tree(l) for l in range(self.L)]
        self.nact = {n.address: [self._n_active(n, l) for l in range(self.L)] for n in self.nodes}
        self.hmat = [dict() for _ in range(self.L)]
        self.hcon = [dict() for _ in range(self.L)]
        zero = lambda n: np.zeros((n.shape[-1], n.shape[-1]), complex)
        for l in range(self.L):
            for a in self.stree[l]:
                n = self.nodes[a]
                self.hmat[l][a] = zero(n)
                self.hcon[l][a] = zero(n)
        self.hcorr = {n.address: zero(n) for n in self.nodes}
        self.hconcorr = {n.address: zero(n) for n in self.nodes}

    # -- sparse structure ----------------------------------------------------
    def _sparse_tree(self, l):
        modes = self.sop.terms[l].target_leaves()
        path = set()
        for m in modes:
            a = self.tree.leaf_node[m]
            while True:
                path.add(a)
                n = self.nodes[a]
                if n.parent < 0:
                    break
                a = n.parent
        order = sorted(path)
        # top-down, first node with more than one active child; keep it and below
        m = len(order) - 1
        while m > 0:
            n = self.nodes[order[m]]
            if sum(1 for c in n.children if c in path) > 1:
                break
            m -= 1
        m += 1
        return set(order[:m])

    def _n_active(self, n, l):
        if n.is_bottom:
            return 1 if n.leaf_mode in self.sop.terms[l].target_leaves() else 0
        k = sum(1 for c in n.children if c in self.stree[l])
        if n.parent < 0:
            return k
        return k + (1 if n.address in self.stree[l] else 0)

    # -- leaf operators ------------------------------------------------------
    def _leaf_apply(self, l, x, n):
        ops = self.sop.ops
        for (m, o) in self.sop.terms[l].factors:
            if m != n.leaf_mode:
                continue
            if ops.kind[o] == OP_DENSE:
                x = _mp(ops.dense(o), x, 0)
            else:
                x = ops.data[o][:, None] * x
        return x

    # -- building blocks -----------------------------------------------------
    def _apply_children(self, l, x, n, skip):
        for k, c in enumerate(n.children):
            if k == skip or c not in self.stree[l]:
                continue
            x = _mp(self.hmat[l][c], x, k)
        return x

    def build_up(self, psi, a):
        n = self.nodes[a]
        phi = psi[a]
        last = len(n.shape) - 1
        for l in range(self.L):
            if a not in self.stree[l]:
                continue
            if n.is_bottom:
                self.hmat[l][a] = _hole(phi, self._leaf_apply(l, phi, n), last)
            else:
                self.hmat[l][a] = _hole(phi, self._apply_children(l, phi, n, -1), last)
        self._build_up_correction(psi, a)

    def _build_up_correction(self, psi, a):
        n = self.nodes[a]
        phi = psi[a]
        last = len(n.shape) - 1
        corr = np.zeros((n.shape[-1], n.shape[-1]), complex)
        if not n.is_bottom:
            hA = np.zeros_like(phi)
            for k, c in enumerate(n.children):
                hA = hA + _mp(self.hcorr[c], phi, k)
            corr = _hole(phi, hA, last)
        if n.parent >= 0:
            for l in range(self.L):
                if self.nact[n.parent][l] != 1:
                    continue
                if a in self.stree[l]:
                    corr = corr + self.sop.coeffs[l] * self.hmat[l][a]
        self.hcorr[a] = corr

    def build_down(self, psi, a):
        n = self.nodes[a]
        if n.parent < 0:
            return
        p = self.nodes[n.parent]
        phi = psi[p.address]
        plast = len(p.shape) - 1
        for l in range(self.L):
            if a not in self.stree[l]:
                continue
            x = self._apply_children(l, phi, p, n.child_idx)
            if p.parent >= 0 and p.address in self.stree[l]:
                x = _mp(self.hcon[l][p.address], x, plast)
            self.hcon[l][a] = _hole(phi, x, n.child_idx)
        self._build_down_correction(psi, a)

    def _build_down_correction(self, psi, hole):
        h = self.nodes[hole]
        if h.parent < 0:
            return
        node = self.nodes[h.parent]
        phi = psi[node.address]
        last = len(node.shape) - 1
        hA = np.zeros_like(phi)
        for l in range(self.L):
            if self.nact[node.address][l] < 2 or hole in self.stree[l]:
                continue
            x = self._apply_children(l, phi, node, h.child_idx)
            if node.parent >= 0 and node.address in self.stree[l]:
                x = _mp(self.hcon[l][node.address], x, last)
            hA = hA + self.sop.coeffs[l] * x
        for k, c in enumerate(node.children):
            if k == h.child_idx:
                continue
            hA = hA + _mp(self.hcorr[c], phi, k)
        if node.parent >= 0:
            hA = hA + _mp(self.hconcorr[node.address], phi, last)
        self.hconcorr[hole] = _hole(phi, hA, h.child_idx)

    def initial_build(self, psi):
        """scf(): buildSCF(node, parent) for every non-top node, bottom-up."""
        for n in self.nodes:
            if n.parent >= 0:
                self.build_up(psi, n.address)

    # -- effective Hamiltonian at a node (SCF.cpp apply) -----------------------
    def apply(self, A, a):
        n = self.nodes[a]
        last = len(n.shape) - 1
        HA = np.zeros_like(A)
        for l in range(self.L):
            if n.is_bottom:
                if a in self.stree[l]:
                    HA = HA + self.sop.coeffs[l] * _mp(self.hcon[l][a], self._leaf_apply(l, A, n), last)
            elif self.nact[a][l] > 1:
                x = self._apply_children(l, A, n, -1)
                if n.parent >= 0 and a in self.stree[l]:
                    x = _mp(self.hcon[l][a], x, last)
                HA = HA + self.sop.coeffs[l] * x
        if not n.is_bottom:
            for k, c in enumerate(n.children):
                HA = HA + _mp(self.hcorr[c], A, k)
        if n.parent >= 0:
            HA = HA + _mp(self.hconcorr[a], A, last)
        return HA

    # -- Krylov ----------------------------------------------------------------
    def solve_krylov(self, psi_node, a, size, breakdown=None):
        """``breakdown``: None follows SCF.cpp (divide by any residual norm);
        a number ends the Lanczos space when the residual norm falls below it
        times the largest |alpha|, beta so far -- the rule qt_scf applies."""
        space = []
        x = psi_node.copy()
        x = x / np.sqrt(_full(x, x).real)
        space.append(x)
        alpha, beta = [], []
        hx = self.apply(x, a)
        alpha.append(_full(x, hx).real)
        x = hx - alpha[-1] * x
        for l in range(1, size):
            nrm = np.sqrt(_full(x, x).real)
            if breakdown is not None and nrm <= breakdown * max(np.abs(alpha).max(), max(beta, default=0.0)):
                size = l
                break
            beta.append(nrm)
            x = x / nrm
            space.append(x)
            hx = self.apply(x, a)
            alpha.append(_full(x, hx).real)
            x = hx - alpha[-1] * space[l] - beta[-1] * space[l - 1]
        T = np.diag(alpha).astype(complex)
        size = len(alpha)
        for l in range(size - 1):
            T[l + 1, l] = T[l, l + 1] = beta[l]
        E, U = np.linalg.eigh(T)
        return space, E, U

    @staticmethod
    def imaginary_time(space, E, U, beta):
        """The k = 0 term enters twice, as in SCF.cpp:208-214."""
        size = len(E)
        c = np.zeros(size, complex)
        for l in range(size):
            c[l] += U[l, 0] * np.conj(U[0, 0])
            for k in range(size):
                c[l] += U[l, k] * np.exp(-beta * (E[k] - E[0])) * np.conj(U[0, k])
        x = sum(c[l] * space[l] for l in range(size))
        return x / np.sqrt(_full(x, x).real)

    @staticmethod
    def ritz_ground(space, U):
        return sum(U[l, 0] * space[l] for l in range(len(space)))


def sweep_order(tree):
    """scf_sweep: depth-first from the top, returning to a node after each child."""
    out = []

    def add(a):
        out.append(a)
        n = tree.nodes[a]
        for c in n.children:
            add(c)
            out.append(a)

    add(tree.top.address)
    return out


def _adjacent(tree, frm, to):
    n = tree.nodes[frm]
    if to is None:
        return len(n.shape) - 1
    if to in n.children:
        return n.children.index(to)
    return len(n.shape) - 1


def _qr_mode(x, mode):
    """Thin Householder QR of x with `mode` as the column index (toMatrix / toTensor)."""
    xm = np.moveaxis(x, mode, -1)
    shp = xm.shape
    q, _ = np.linalg.qr(xm.reshape(-1, shp[-1]))
    return np.moveaxis(q.reshape(shp), -1, mode)


def scf(tree, sop, psi_tensors, n_iter=1, n_krylov=5, n_itp=0, beta=1.0, breakdown=None):
    """Run the SCF sweep; returns (lowest Ritz value of every Krylov solve,
    final node tensors).  ``breakdown``: see SCFOracle.solve_krylov."""
    psi = [np.array(t, dtype=complex, copy=True) for t in psi_tensors]
    rep = SCFOracle(tree, sop)
    rep.initial_build(psi)
    order = sweep_order(tree)
    energies = []
    for it in range(n_iter):
        for i, a in enumerate(order):
            n = tree.nodes[a]
            size = min(n_krylov, psi[a].size)
            space, E, U = rep.solve_krylov(psi[a], a, size, breakdown)
            energies.append(E[0])
            if it < n_itp:
                psi[a] = rep.imaginary_time(space, E, U, beta)
            else:
                psi[a] = rep.ritz_ground(space, U)
            nxt = order[i + 1] if i + 1 < len(order) else None
            out_idx = _adjacent(tree, a, nxt)
            w = psi[a]
            psi[a] = _qr_mode(w, out_idx)
            if nxt is None:
                break
            r = _hole(psi[a], w, out_idx)
            in_idx = _adjacent(tree, nxt, a)
            psi[nxt] = _mp(r, psi[nxt], in_idx)
            up = (n.parent == nxt) if n.parent >= 0 else False
            if up:
                rep.build_up(psi, a)
            else:
                rep.build_down(psi, nxt)
    return np.array(energies), psi
