"""Dense-state reference of the sweep quantities (test infrastructure).

For trees small enough to hold Psi as a full array, every sweep quantity has
a direct definition independent of the tree contraction order:
  V_n        the SPFs of node n as dense functions of its subtree's modes
  G_n        the single-hole functions of n (Psi = sum_j V_n[.., j] G_n[.., j])
  h_l[n]     = <V_n| O_l(inside n) |V_n>
  H_l[n]     = <G_n| O_l(outside n) |G_n>
  X_n[a, j]  = <chi_a g_j | H | Psi>   (chi_a: product of the children's SPFs)
  E          = <Psi|H|Psi> / <Psi|Psi>
The MCTDH derivative of a non-top node is -i rho^-1 (1-P) X_n, of the top -i X.
"""
from __future__ import annotations

import string

import numpy as np

LETTERS = string.ascii_letters


class Dense:
    def __init__(self, tree, sop, psi):
        self.tree, self.sop, self.psi = tree, sop, psi
        self.V, self.Vmodes = {}, {}
        for n in tree.nodes:
            self._spf(n)
        top = tree.top
        assert top.d_up == 1
        modes = self.Vmodes[top.address]
        full = self.V[top.address][..., 0]
        perm = [modes.index(m) for m in range(tree.n_leaves)]
        self.Psi = np.transpose(full, perm)  # axes = modes 0..f-1
        self.G, self.Gmodes = {}, {}
        for n in reversed(tree.nodes):
            self._hole(n)
        self.HPsi = self.apply_sop(self.Psi, range(len(sop)))

    # SPFs bottom-up
    def _spf(self, n):
        phi = self.psi.tensors[n.address]
        if n.is_bottom:
            self.V[n.address] = np.asarray(phi)
            self.Vmodes[n.address] = [n.leaf_mode]
            return
        ins, subs, modes, pos = [], [], [], 0
        core = "".join(LETTERS[26 + k] for k in range(len(n.children)))  # A, B, ...
        j = "Z"
        for k, c in enumerate(n.children):
            cm = self.Vmodes[c]
            lab = "".join(LETTERS[pos + i] for i in range(len(cm)))
            pos += len(cm)
            ins.append(self.V[c])
            subs.append(lab + core[k])
            modes += cm
        out = "".join(LETTERS[i] for i in range(pos)) + j
        expr = core + j + "," + ",".join(subs) + "->" + out
        self.V[n.address] = np.einsum(expr, phi, *ins)
        self.Vmodes[n.address] = modes

    # single-hole functions top-down
    def _hole(self, n):
        if n.is_top:
            self.G[n.address] = np.ones((1,), complex)
            self.Gmodes[n.address] = []
            return
        p = self.tree.nodes[n.parent]
        phi = self.psi.tensors[p.address]
        core = "".join(LETTERS[26 + k] for k in range(len(p.children)))
        j = "Z"
        ins, subs, modes, pos = [], [], [], 0
        for k, c in enumerate(p.children):
            if c == n.address:
                continue
            cm = self.Vmodes[c]
            lab = "".join(LETTERS[pos + i] for i in range(len(cm)))
            pos += len(cm)
            ins.append(self.V[c])
            subs.append(lab + core[k])
            modes += cm
        gm = self.Gmodes[p.address]
        glab = "".join(LETTERS[pos + i] for i in range(len(gm)))
        pos += len(gm)
        ins.append(self.G[p.address])
        subs.append(glab + j)
        modes += gm
        out = "".join(LETTERS[i] for i in range(pos)) + core[n.child_idx]
        expr = core + j + "," + ",".join(subs) + "->" + out
        self.G[n.address] = np.einsum(expr, phi, *ins)
        self.Gmodes[n.address] = modes

    # operators
    def op_on(self, arr, axis_of_mode, factors):
        for (m, o) in factors:
            if m not in axis_of_mode:
                continue
            ax = axis_of_mode[m]
            M = self.sop.ops.dense(o)
            arr = np.moveaxis(np.tensordot(M, arr, axes=([1], [ax])), 0, ax)
        return arr

    def apply_sop(self, psi_full, terms):
        out = np.zeros_like(psi_full)
        ax = {m: m for m in range(self.tree.n_leaves)}
        for l in terms:
            out += self.sop.coeffs[l] * self.op_on(psi_full, ax, self.sop.terms[l].factors)
        return out

    def energy(self):
        return (np.vdot(self.Psi, self.HPsi) / np.vdot(self.Psi, self.Psi)).real

    def hmat(self, l, a):
        V = self.V[a]
        modes = self.Vmodes[a]
        ax = {m: i for i, m in enumerate(modes)}
        inside = [(m, o) for (m, o) in self.sop.terms[l].factors if m in ax]
        OV = self.op_on(V, ax, inside)
        d = V.shape[-1]
        return V.reshape(-1, d).conj().T @ OV.reshape(-1, d)

    def hcon(self, l, a):
        G = self.G[a]
        modes = self.Gmodes[a]
        ax = {m: i for i, m in enumerate(modes)}
        outside = [(m, o) for (m, o) in self.sop.terms[l].factors if m in ax]
        OG = self.op_on(G, ax, outside)
        d = G.shape[-1]
        return G.reshape(-1, d).conj().T @ OG.reshape(-1, d)

    def x_node(self, a):
        """X_n[a_1..a_k, j] = <chi_a g_j | H Psi> as a node-shaped array."""
        n = self.tree.nodes[a]
        vm, gm = self.Vmodes[a], self.Gmodes[a]
        hp = np.transpose(self.HPsi, vm + gm)
        nin = len(vm)
        hp = hp.reshape(int(np.prod(hp.shape[:nin])), -1)
        y = hp @ self.G[a].reshape(-1, n.d_up).conj()  # (inside, j)
        if n.is_bottom:
            return y
        chi = None
        for c in n.children:
            Vc = self.V[c].reshape(-1, self.tree.nodes[c].d_up)
            chi = Vc if chi is None else np.einsum("xa,yb->xyab", chi, Vc).reshape(
                chi.shape[0] * Vc.shape[0], chi.shape[1] * Vc.shape[1])
        z = chi.conj().T @ y
        return z.reshape(tuple(n.shape))
