"""Host-side model of a tree tensor network: tree shape, leaf operators, SOP
Hamiltonian and the seeded wavefunction.

This module builds the *inputs* of the H.Psi sweep; it does no sweep
arithmetic.  Everything here mirrors QuTree's own input builders so that a
QuTree user finds the same objects:

* ``Tree`` / ``balanced_tree``   -- TreeFactory::balancedTree
  (src/TreeShape/TreeFactory.cpp:52-200) and the bottom-up node linearisation
  of Tree::linearizeNodes (src/TreeShape/Tree.cpp:92-114, Node::nextNode at
  src/TreeShape/Node.cpp:225-239) plus Tree::resetLeafModes
  (src/TreeShape/Tree.cpp:35-46).
* ``HOBasis``                     -- HO_Basis::initialize / InitXmat / InitKin
  (src/TreeShape/LeafTypes/HO_Basis.cpp:3-111): DVR grid and kinetic matrix.
* ``SOP`` / ``MLO``               -- SumOfProductsOperator / MultiLeafOperator
  (include/TreeOperators/SumOfProductsOperator.h:5-135,
  include/TreeOperators/MultiLeafOperator.h:11-196).
* ``random_wavefunction``         -- i.i.d. complex N(0,1) node tensors followed by
  qrOrthogonal (include/TreeClasses/TensorTree_Implementation.h:173-187).

Memory layout follows QuTree: a node tensor of shape (d_0, ..., d_{k-1}, d_up)
is column-major (first index fastest, include/Core/Tensor_Implementation.h:
154-165); node tensors are stored one after another in node-address order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

OP_DENSE = 0   # dense p x p complex matrix, column-major
OP_DIAG = 1    # diagonal: p complex numbers

# 4000 cm^-1 in atomic units, the oscillator frequency CoupledHO uses
# (contrib/Hamiltonians/Operators/CoupledHO/CoupledHO.cpp:17).
CM_PER_HARTREE = 219474.6313705
OMEGA_AU = 4000.0 / CM_PER_HARTREE


# --------------------------------------------------------------------------
# Tree shape
# --------------------------------------------------------------------------
@dataclass
class Node:
    address: int
    shape: tuple
    parent: int = -1
    children: list = field(default_factory=list)
    child_idx: int = -1          # position of this node among its parent's children
    leaf_mode: int = -1          # physical mode for bottom nodes, -1 otherwise
    height: int = 0              # 0 for bottom nodes, 1 + max(children) above

    @property
    def is_bottom(self) -> bool:
        return self.leaf_mode >= 0

    @property
    def is_top(self) -> bool:
        return self.parent < 0

    @property
    def size(self) -> int:
        return int(np.prod(self.shape))

    @property
    def order(self) -> int:
        return len(self.shape)

    @property
    def d_up(self) -> int:
        return self.shape[-1]


class _Build:
    """Mutable node used while the tree is assembled (children in order)."""

    def __init__(self, dims, children=None, leaf=False):
        self.dims = list(dims)
        self.children = children or []
        self.leaf = leaf
        self.mode = -1


class Tree:
    """Tree topology with nodes in QuTree's bottom-up address order."""

    def __init__(self, root: _Build):
        self.nodes: list[Node] = []
        self._linearize(root)
        # Tree::resetLeafModes: bottom nodes in address order get modes
        # n_leaves-1, n_leaves-2, ..., 0.
        bottoms = [n for n in self.nodes if n.leaf_mode >= 0]
        mode = len(bottoms) - 1
        for n in bottoms:
            n.leaf_mode = mode
            mode -= 1
        self.leaf_node = {n.leaf_mode: n.address for n in bottoms}
        for n in self.nodes:   # heights bottom-up
            n.height = 0 if n.is_bottom else 1 + max(self.nodes[c].height for c in n.children)

    def _linearize(self, root: _Build):
        # Node::nextNode is a post-order walk that visits children from the
        # last to the first; the counter of visited nodes is the address.
        def visit(b: _Build, parent_addr_slot):
            kids = []
            for c in reversed(b.children):
                kids.append(visit(c, None))
            addr = len(self.nodes)
            node = Node(address=addr, shape=tuple(b.dims),
                        leaf_mode=(0 if b.leaf else -1))
            self.nodes.append(node)
            kids = list(reversed(kids))   # back to child-index order
            node.children = kids
            for k, ka in enumerate(kids):
                self.nodes[ka].parent = addr
                self.nodes[ka].child_idx = k
            return addr

        visit(root, None)

    # -- queries ---------------------------------------------------------
    @property
    def n_nodes(self) -> int:
        return len(self.nodes)

    @property
    def n_leaves(self) -> int:
        return len(self.leaf_node)

    @property
    def top(self) -> Node:
        return self.nodes[-1]

    def leaf_dim(self, mode: int) -> int:
        return self.nodes[self.leaf_node[mode]].shape[0]

    def offsets(self, align: int = 1) -> np.ndarray:
        """Element offsets of the node tensors when stored back to back."""
        off = np.zeros(self.n_nodes + 1, dtype=np.int64)
        for n in self.nodes:
            sz = n.size
            if align > 1:
                sz = (sz + align - 1) // align * align
            off[n.address + 1] = off[n.address] + sz
        return off

    def descriptor(self):
        """Flat int32 arrays of the C ABI tree descriptor."""
        order = np.array([n.order for n in self.nodes], dtype=np.int32)
        dims = np.array([d for n in self.nodes for d in n.shape], dtype=np.int32)
        parent = np.array([n.parent for n in self.nodes], dtype=np.int32)
        child_idx = np.array([n.child_idx for n in self.nodes], dtype=np.int32)
        leaf_mode = np.array([n.leaf_mode for n in self.nodes], dtype=np.int32)
        return order, dims, parent, child_idx, leaf_mode

    def path_to_root(self, mode: int):
        a = self.leaf_node[mode]
        out = []
        while a >= 0:
            out.append(a)
            a = self.nodes[a].parent
        return out

    def sparse_tree(self, modes, tail: bool = True):
        """Addresses of the nodes on the leaf-to-root paths of ``modes`` in
        ascending order (SparseTree::SparseInitialize,
        src/TreeClasses/SparseTree.cpp:33-89).  Without ``tail`` the nodes
        above the highest branching point are cut off (top-down: stop at the
        first node with more than one active child, keep it)."""
        act = set()
        for m in modes:
            act |= set(self.path_to_root(m))
        nodes = sorted(act)
        if not tail:
            m = len(nodes) - 1
            while m > 0:
                nd = self.nodes[nodes[m]]
                if sum(1 for c in nd.children if c in act) > 1:
                    break
                m -= 1
            if m < len(nodes):
                m += 1
            nodes = nodes[:m]
        return nodes

    def subtree_modes(self, addr: int) -> set:
        n = self.nodes[addr]
        if n.is_bottom:
            return {n.leaf_mode}
        s = set()
        for c in n.children:
            s |= self.subtree_modes(c)
        return s


def _partition(nodes, n_partition, dim_node):
    """TreeFactory partition (src/TreeShape/TreeFactory.cpp:52-102)."""
    groups = []
    n_loop = len(nodes) // n_partition
    for k in range(n_loop):
        ch = nodes[k * n_partition:(k + 1) * n_partition]
        dims = [c.dims[-1] for c in ch]
        groups.append(_Build(dims + [min(int(np.prod(dims)), dim_node)], ch))
    n_rest = len(nodes) % n_partition
    if n_loop == 0 and n_rest > 0:
        ch = nodes[:n_rest]
        dims = [c.dims[-1] for c in ch]
        groups.append(_Build(dims + [min(int(np.prod(dims)), dim_node)], ch))
    else:
        groups.extend(nodes[n_loop * n_partition:])
    return groups


def balanced_tree(num_leaves: int, dim_leaves, dim_nodes: int, dim_inc: int = 0,
                  bonds=None) -> Tree:
    """Close-to-balanced binary tree, TreeFactory::balancedTree semantics.

    ``dim_leaves`` is an int or a per-leaf list.  By default the bond above an
    upper node at depth-from-bottom ``L`` is ``dim_nodes + L*dim_inc``
    (src/TreeShape/TreeFactory.cpp:175-196).  ``bonds`` overrides that with an
    explicit list indexed by the height of the lower node (bottom = 0), or a
    callable ``bonds(height, leaf_dim_or_None) -> int``.  Every bond is clamped
    to the product of the node's child dims (TreeFactory.cpp:69,117,189), and
    nodes that do not contract are expanded away (expandNodes, :126-141).
    """
    if isinstance(dim_leaves, (int, np.integer)):
        dim_leaves = [int(dim_leaves)] * num_leaves

    def bond(height, p):
        if bonds is None:
            return dim_nodes if height == 0 else dim_nodes + height * dim_inc
        if callable(bonds):
            return int(bonds(height, p))
        return int(bonds[min(height, len(bonds) - 1)])

    leaves = []
    for k in range(num_leaves):
        p = dim_leaves[k]
        b = _Build([p, min(bond(0, p), p)], leaf=True)
        leaves.append(b)
    nodes = leaves
    count = 0
    while len(nodes) > 1:
        nodes = _partition(nodes, 2, 1 << 30)
        count += 1
        if count > 100:
            raise RuntimeError("balanced_tree: partitioning did not converge")
    root = nodes[0]

    # bond dims by height (distance to the bottom layer), clamped to lastBefore
    def set_dims(b: _Build) -> int:
        if b.leaf:
            return 0
        hs = [set_dims(c) for c in b.children]
        h = 1 + max(hs)
        for k, c in enumerate(b.children):
            b.dims[k] = c.dims[-1]
        lb = int(np.prod(b.dims[:-1]))
        b.dims[-1] = min(bond(h, None), lb)
        return h

    set_dims(root)
    root.dims[-1] = 1

    # expandNodes: a non-bottom, non-top node whose bond equals the product of
    # its children's dims performs no contraction; splice its children into
    # its parent.
    def expand(b: _Build):
        changed = True
        while changed:
            changed = False
            new_children = []
            for c in b.children:
                if (not c.leaf) and int(np.prod(c.dims[:-1])) == c.dims[-1]:
                    new_children.extend(c.children)
                    changed = True
                else:
                    new_children.append(c)
            b.children = new_children
        b.dims = [c.dims[-1] for c in b.children] + [b.dims[-1]]
        for c in b.children:
            if not c.leaf:
                expand(c)

    expand(root)
    return Tree(root)


# --------------------------------------------------------------------------
# Leaf operators: harmonic-oscillator DVR
# --------------------------------------------------------------------------
def _symmetric_eig_phase(a: np.ndarray):
    """Ascending eigenpairs with QuTree's phase convention (first row >= 0),
    Matrix::rDiag (include/Core/Matrix_Implementation.h:251-274)."""
    w, v = np.linalg.eigh(a)
    for i in range(v.shape[1]):
        if v[0, i] < 0:
            v[:, i] *= -1
    return w, v


class HOBasis:
    """Harmonic-oscillator DVR of dimension p (HO_Basis::initialize)."""

    def __init__(self, p: int, omega: float = 1.0, r0: float = 0.0,
                 wfr0: float = 1.0, wfomega: float = 0.0):
        self.p, self.omega, self.r0 = p, omega, r0
        self.wfr0, self.wfomega = wfr0, wfomega
        x = np.zeros((p, p))
        for n in range(p):
            if n + 1 < p:
                x[n + 1, n] = math.sqrt(n + 1.0)
            if n - 1 >= 0:
                x[n - 1, n] = math.sqrt(n * 1.0)
        x *= math.sqrt(1.0 / (2.0 * omega))
        self.x, self.trafo = _symmetric_eig_phase(x)
        self.x = self.x + r0
        kin = np.zeros((p, p))
        for i in range(p):
            for j in range(p):
                v = 0.0
                if i == j + 2:
                    v = math.sqrt((j + 1.0) * (j + 2.0))
                if i == j:
                    v = -(2 * j + 1.0)
                if i == j - 2:
                    v = math.sqrt(j * (j - 1.0))
                kin[j, i] = v * (-omega / 2.0) * 0.5
        # unitarySimilarityTrafo(A, B) = B^T A B
        self.kin = self.trafo.T @ kin @ self.trafo

    def init_spf(self, d_up: int) -> np.ndarray:
        """HO_Basis::initSPF (src/TreeShape/LeafTypes/HO_Basis.cpp:35-57)."""
        phi = np.zeros((self.p, d_up), dtype=np.complex128)
        for i in range(self.p):
            w = self.trafo[0, i] / math.exp(-0.5 * self.omega * (self.x[i] - self.r0) ** 2)
            phi[i, 0] = w * math.exp(-0.5 * self.wfomega * (self.x[i] - self.wfr0) ** 2)
        for n in range(1, d_up):
            phi[:, n] = self.x * phi[:, n - 1]
        return gram_schmidt(phi)


def gram_schmidt(a: np.ndarray) -> np.ndarray:
    """Column Gram-Schmidt with re-orthogonalisation (gramSchmidt,
    include/Core/Tensor_Implementation.h:805-853) on a (lastBefore, d_up)
    matrix view."""
    a = np.array(a, dtype=np.complex128, copy=True)
    for n in range(a.shape[1]):
        for _ in range(15):
            acc = 0.0
            for m in range(n):
                ov = np.vdot(a[:, m], a[:, n])
                acc += abs(ov)
                a[:, n] -= ov * a[:, m]
            nrm = np.vdot(a[:, n], a[:, n])
            if abs(nrm) != 0:
                a[:, n] /= math.sqrt(nrm.real)
            if acc <= 1e-12:
                break
    return a


# --------------------------------------------------------------------------
# Potential (CDVR)
# --------------------------------------------------------------------------
class PolyPotential:
    """Potential of a Hamiltonian with hasV, applied by CDVR: V(x) =
    sum_t c_t prod_(g, p) x_g^p (a polynomial stands in for the reference's
    Potential::evaluate callback, include/TreeOperators/Potential.h:9-18).
    Evaluation: terms in order, each product left to right, as the device
    kernel does."""

    def __init__(self, n_modes: int, terms):
        self.f = n_modes
        self.terms = [(float(c), [(int(g), int(p)) for g, p in fac]) for c, fac in terms]

    def __call__(self, X: np.ndarray) -> np.ndarray:
        v = np.zeros(X.shape[:-1])
        for c, fac in self.terms:
            t = np.full(X.shape[:-1], c)
            for g, p in fac:
                for _ in range(p):
                    t = t * X[..., g]
            v = v + t
        return v

    def descriptor(self):
        """(coeff[n_terms], ptr[n_terms+1], mode[], power[]) for qt_cdvr_upload."""
        coeff = np.array([c for c, _ in self.terms], dtype=np.float64)
        ptr = np.zeros(len(self.terms) + 1, dtype=np.int32)
        modes, pows = [], []
        for t, (_, fac) in enumerate(self.terms):
            for g, p in fac:
                modes.append(g)
                pows.append(p)
            ptr[t + 1] = len(modes)
        return coeff, ptr, np.array(modes, dtype=np.int32), np.array(pows, dtype=np.int32)

    @classmethod
    def cdvr_model(cls, f: int, coupling: bool = True):
        """contrib/Hamiltonians/PESs/CDVRModelV/CDVRModelV.cpp:7-28:
        sum_i omega^2/2 x_i^2 + lambda^2 sum_i x_i x_(i+1 mod f)."""
        cm = 219474.6313705
        lam, om = 2000.0 / cm, 4000.0 / cm
        terms = [(0.5 * om * om, [(i, 2)]) for i in range(f)]
        if coupling:
            terms += [(lam * lam, [(i, 1), ((i + 1) % f, 1)]) for i in range(f)]
        return cls(f, terms)


# --------------------------------------------------------------------------
# Sum-of-products operator
# --------------------------------------------------------------------------
class OperatorTable:
    """Flat table of leaf operators (dense p x p or diagonal), deduplicated by
    object identity of the caller's key."""

    def __init__(self):
        self.kind: list[int] = []
        self.dim: list[int] = []
        self.data: list[np.ndarray] = []
        self._keys: dict = {}

    def add(self, key, kind: int, arr: np.ndarray) -> int:
        if key is not None and key in self._keys:
            return self._keys[key]
        arr = np.asarray(arr, dtype=np.complex128)
        if kind == OP_DENSE:
            assert arr.ndim == 2 and arr.shape[0] == arr.shape[1]
            flat = arr.ravel(order="F")
            dim = arr.shape[0]
        else:
            assert arr.ndim == 1
            flat = arr
            dim = arr.shape[0]
        idx = len(self.kind)
        self.kind.append(kind)
        self.dim.append(dim)
        self.data.append(flat)
        if key is not None:
            self._keys[key] = idx
        return idx

    def descriptor(self):
        kind = np.array(self.kind, dtype=np.int32)
        dim = np.array(self.dim, dtype=np.int32)
        off = np.zeros(len(self.kind), dtype=np.int64)
        acc = 0
        for i, d in enumerate(self.data):
            off[i] = acc
            acc += d.size
        data = (np.concatenate(self.data) if self.data else np.zeros(0, np.complex128))
        return kind, dim, off, np.ascontiguousarray(data.astype(np.complex128))

    def dense(self, op: int) -> np.ndarray:
        """Operator as a dense complex matrix (for checks)."""
        if self.kind[op] == OP_DENSE:
            p = self.dim[op]
            return self.data[op].reshape((p, p), order="F")
        return np.diag(self.data[op])


class MLO:
    """Product of leaf operators: factors (mode, op) applied in list order."""

    def __init__(self, factors=None):
        self.factors: list[tuple[int, int]] = list(factors or [])

    def push_back(self, op: int, mode: int):
        self.factors.append((mode, op))

    def target_leaves(self):
        seen = []
        for m, _ in self.factors:
            if m not in seen:
                seen.append(m)
        return seen


class SOP:
    """Sum of products: H = sum_l coeff_l * MLO_l."""

    def __init__(self, ops: OperatorTable):
        self.ops = ops
        self.terms: list[MLO] = []
        self.coeffs: list[complex] = []

    def push_back(self, mlo: MLO, coeff):
        self.terms.append(mlo)
        self.coeffs.append(complex(coeff))

    def __len__(self):
        return len(self.terms)

    def descriptor(self):
        coeff = np.array(self.coeffs, dtype=np.complex128)
        ptr = np.zeros(len(self.terms) + 1, dtype=np.int32)
        modes, opids = [], []
        for l, t in enumerate(self.terms):
            for m, o in t.factors:
                modes.append(m)
                opids.append(o)
            ptr[l + 1] = len(modes)
        return (coeff, ptr, np.array(modes, dtype=np.int32),
                np.array(opids, dtype=np.int32))


def coupled_oscillators(tree: Tree, n_pairs=None, coupling=0.1, quartic=0.0,
                        rng=None, omega=OMEGA_AU, pairs_per_mode=None,
                        include_q2=True) -> SOP:
    """Seeded coupled-oscillator SOP, structured like CoupledHO
    (contrib/Hamiltonians/Operators/CoupledHO/CoupledHO.cpp:7-66).

    Per mode: one kinetic term (dense real DVR matrix) and one on-site term
    (diagonal: 1/2 w^2 q^2, plus ``quartic * w^3 * q^4`` when ``quartic`` is
    non-zero).  Couplings: ``c_ij * w^2 * q_i q_j`` with c_ij ~ U(-coupling,
    coupling), over all pairs (``n_pairs=None``), ``n_pairs`` pairs drawn
    uniformly without replacement, or ``pairs_per_mode`` random partners per
    mode.  Coefficients carry w^2 so that the coupling strength is relative
    to the harmonic force constant.
    """
    rng = rng if rng is not None else np.random.default_rng(0)
    ops = OperatorTable()
    sop = SOP(ops)
    f = tree.n_leaves
    kin, onsite, xop = {}, {}, {}
    for k in range(f):
        p = tree.leaf_dim(k)
        if p not in kin:
            b = HOBasis(p, omega=omega)
            kin[p] = ops.add(("kin", p), OP_DENSE, b.kin.astype(np.complex128))
            v = 0.5 * omega * omega * b.x ** 2
            if quartic:
                v = v + quartic * omega ** 3 * b.x ** 4
            onsite[p] = ops.add(("v", p), OP_DIAG, v.astype(np.complex128))
            xop[p] = ops.add(("x", p), OP_DIAG, b.x.astype(np.complex128))
    for k in range(f):
        p = tree.leaf_dim(k)
        sop.push_back(MLO([(k, kin[p])]), 1.0)
        if include_q2:
            sop.push_back(MLO([(k, onsite[p])]), 1.0)
    all_pairs = [(i, j) for i in range(f) for j in range(i + 1, f)]
    if pairs_per_mode is not None:
        chosen = set()
        for i in range(f):
            npm = int(rng.integers(pairs_per_mode[0], pairs_per_mode[1] + 1))
            partners = rng.permutation([j for j in range(f) if j != i])[:npm]
            for j in partners:
                chosen.add((min(i, int(j)), max(i, int(j))))
        pairs = sorted(chosen)
    elif n_pairs is None or n_pairs >= len(all_pairs):
        pairs = all_pairs
    else:
        sel = rng.choice(len(all_pairs), size=n_pairs, replace=False)
        pairs = [all_pairs[s] for s in sorted(sel)]
    for (i, j) in pairs:
        c = rng.uniform(-coupling, coupling) * omega * omega
        sop.push_back(MLO([(i, xop[tree.leaf_dim(i)]), (j, xop[tree.leaf_dim(j)])]), c)
    return sop


# --------------------------------------------------------------------------
# Wavefunction
# --------------------------------------------------------------------------
def mode_product(h: np.ndarray, phi: np.ndarray, k: int) -> np.ndarray:
    """C = h x_k phi: C[..., a', ...] = sum_a h[a', a] phi[..., a, ...]."""
    out = np.tensordot(h, phi, axes=([1], [k]))
    return np.moveaxis(out, 0, k)


def hole_product(a: np.ndarray, b: np.ndarray, k: int) -> np.ndarray:
    """S[i, j] = sum_{all but k} conj(a[..i..]) b[..j..]."""
    axes = [x for x in range(a.ndim) if x != k]
    return np.tensordot(a.conj(), b, axes=(axes, axes))


class TensorTree:
    """Node tensors of a tree, each an ndarray in Fortran (column-major) order."""

    def __init__(self, tree: Tree, tensors):
        self.tree = tree
        self.tensors = [np.asfortranarray(t, dtype=np.complex128) for t in tensors]

    def flat(self, align: int = 1) -> np.ndarray:
        off = self.tree.offsets(align)
        out = np.zeros(int(off[-1]), dtype=np.complex128)
        for n, t in zip(self.tree.nodes, self.tensors):
            out[off[n.address]:off[n.address] + n.size] = t.ravel(order="F")
        return out

    @staticmethod
    def from_flat(tree: Tree, flat: np.ndarray, align: int = 1) -> "TensorTree":
        off = tree.offsets(align)
        ts = []
        for n in tree.nodes:
            ts.append(flat[off[n.address]:off[n.address] + n.size].reshape(n.shape, order="F"))
        return TensorTree(tree, ts)

    def copy(self) -> "TensorTree":
        return TensorTree(self.tree, [t.copy() for t in self.tensors])


def qr_orthogonal(psi: TensorTree, rescale: bool = True) -> TensorTree:
    """qrOrthogonal (include/TreeClasses/TensorTree_Implementation.h:173-187):
    bottom-up, replace each non-top node by the Q of its (lastBefore x d_up)
    matrix and push R = Q^dagger Phi into the parent (R divided by its
    Frobenius norm when ``rescale``)."""
    tree = psi.tree
    out = psi.copy()
    for n in tree.nodes:
        if n.is_top:
            continue
        phi = out.tensors[n.address]
        mat = phi.reshape((-1, n.d_up), order="F")
        q, _ = np.linalg.qr(mat)
        s = q.conj().T @ mat
        if rescale:
            # keeps every tensor O(1): without it the norms of R multiply up
            # the layers (squared per level) and overflow double precision on
            # deep trees; only the state's norm changes, its direction not
            s = s / np.linalg.norm(s)
        out.tensors[n.address] = np.asfortranarray(q.reshape(n.shape, order="F"))
        out.tensors[n.parent] = np.asfortranarray(
            mode_product(s, out.tensors[n.parent], n.child_idx))
    return out


def random_wavefunction(tree: Tree, seed: int, normalize_top: bool = True) -> TensorTree:
    """Node tensors with i.i.d. complex N(0,1) entries (re and im), drawn from
    a PCG64 stream seeded with ``seed`` node by node in address order, then
    QR-orthonormalised bottom-up and the top normalised."""
    rng = np.random.default_rng(seed)
    ts = []
    for n in tree.nodes:
        re = rng.standard_normal(n.size)
        im = rng.standard_normal(n.size)
        ts.append((re + 1j * im).reshape(n.shape, order="F"))
    psi = qr_orthogonal(TensorTree(tree, ts))
    if normalize_top:
        t = psi.tensors[-1]
        psi.tensors[-1] = t / np.linalg.norm(t)
    return psi


def hartree_wavefunction(tree: Tree, gen_seed: int, basis_of_leaf) -> TensorTree:
    """Hartree-product start state used by QuTree's own tests:
    TensorTree(gen, tree, delta_lowest=true)
    (include/TreeClasses/TensorTree_Implementation.h:24-66).  Bottom nodes
    get HO initSPF; upper nodes uniform(-1,1) fill, first column set to e_0,
    Gram-Schmidt.  The random stream is numpy's MT19937 seeded with
    ``gen_seed`` (values differ from libstdc++'s stream; the structural
    results the tests check do not depend on them)."""
    rng = np.random.Generator(np.random.MT19937(gen_seed))
    ts = []
    for n in tree.nodes:
        if n.is_bottom:
            b = basis_of_leaf(n.leaf_mode)
            ts.append(b.init_spf(n.d_up))
        else:
            a = rng.uniform(-1.0, 1.0, n.size).astype(np.complex128).reshape(
                (-1, n.d_up), order="F")
            a[:, 0] = 0.0
            a[0, 0] = 1.0
            ts.append(gram_schmidt(a).reshape(n.shape, order="F"))
    return TensorTree(tree, ts)


# --------------------------------------------------------------------------
# The benchmark configurations
# --------------------------------------------------------------------------
def linear_bonds(lo: int, hi: int, n_heights: int):
    """Bond dims growing linearly from ``lo`` (bottom edges) to ``hi`` (edges
    below the top), rounded: 32..64 over 6 heights gives 32,38,45,51,58,64."""
    return [int(round(lo + (hi - lo) * h / (n_heights - 1))) for h in range(n_heights)]


def config_tree_sop(cfg: int, seed_base: int = 20261203):
    """(tree, sop) of configuration ``cfg`` (0: 8 modes p16 b4; 1: 64 modes p32
    b32..64; 3: 64 modes p32 b48..96; 4: 16 modes p32 b32)."""
    rng = np.random.default_rng(seed_base + cfg + 1000)
    if cfg == 0:
        tree = balanced_tree(8, 16, 4)
        sop = coupled_oscillators(tree, n_pairs=None, coupling=0.1, rng=rng)
    elif cfg == 1:
        tree = balanced_tree(64, 32, 32, bonds=linear_bonds(32, 64, 6))
        sop = coupled_oscillators(tree, n_pairs=256, coupling=0.05, quartic=0.05, rng=rng)
    elif cfg == 3:
        bonds = [32, 58, 67, 77, 86, 96]
        tree = balanced_tree(64, 32, 32, bonds=bonds)
        sop = coupled_oscillators(tree, n_pairs=256, coupling=0.05, quartic=0.05, rng=rng)
    elif cfg == 4:
        tree = balanced_tree(16, 32, 32)
        sop = coupled_oscillators(tree, n_pairs=None, coupling=0.1, rng=rng)
    else:
        raise ValueError(f"unknown config {cfg}")
    return tree, sop


def config_problem(cfg: int, seed_base: int = 20261203):
    tree, sop = config_tree_sop(cfg, seed_base)
    psi = random_wavefunction(tree, seed_base + cfg)
    return tree, sop, psi


def cdvr_problem(n_modes: int = 16, p: int = 16, bond: int = 12, seed: int = 20261203,
                 coupling: bool = True):
    """Hamiltonian with a CDVR potential: HO-DVR leaves (omega = 4000 cm^-1 in
    atomic units, as the coupled-oscillator configs use), the kinetic energy
    of every mode as the SOP part and contrib's CDVRModelV as the potential,
    on a balanced binary tree.  Returns (tree, sop, psi, leaf_x, potential)."""
    tree = balanced_tree(n_modes, p, bond)
    basis = HOBasis(p, omega=4000.0 / 219474.6313705)
    ops = OperatorTable()
    kin = ops.add("kin", OP_DENSE, basis.kin.astype(np.complex128))
    sop = SOP(ops)
    for m in range(n_modes):
        ml = MLO()
        ml.push_back(kin, m)
        sop.push_back(ml, 1.0)
    psi = random_wavefunction(tree, seed)
    leaf_x = {m: basis.x.copy() for m in range(n_modes)}
    return tree, sop, psi, leaf_x, PolyPotential.cdvr_model(n_modes, coupling)


# --------------------------------------------------------------------------
# Forests: many independent trees in one sweep
# --------------------------------------------------------------------------
def balance_bonds(tree: Tree) -> Tree:
    """Clamp bonds so every density matrix can have full rank: top-down, a
    child's bond may not exceed its parent's bond times the product of its
    siblings' bonds (with a bond-1 top, both children of a binary top get the
    same bond).  Shapes are edited in place; returns the tree."""
    changed = True
    while changed:
        changed = False
        for p in reversed(tree.nodes):
            if p.is_bottom:
                continue
            dims = list(p.shape)
            for k, c in enumerate(p.children):
                cap = dims[-1]
                for j in range(len(p.children)):
                    if j != k:
                        cap *= dims[j]
                if dims[k] > cap:
                    dims[k] = cap
                    cn = tree.nodes[c]
                    cn.shape = tuple(list(cn.shape[:-1]) + [cap])
                    changed = True
            p.shape = tuple(dims)
    return tree


def forest(trees):
    """Concatenate independent trees into one forest descriptor: node
    addresses and leaf modes are offset tree by tree (every tree's nodes
    precede its root).  Returns (forest, node_offsets, mode_offsets)."""
    f = Tree.__new__(Tree)
    f.nodes = []
    f.leaf_node = {}
    node_off, mode_off = [], []
    na = nm = 0
    for t in trees:
        node_off.append(na)
        mode_off.append(nm)
        for n in t.nodes:
            m = Node(address=n.address + na, shape=n.shape,
                     parent=(n.parent + na) if n.parent >= 0 else -1,
                     children=[c + na for c in n.children], child_idx=n.child_idx,
                     leaf_mode=(n.leaf_mode + nm) if n.leaf_mode >= 0 else -1, height=n.height)
            f.nodes.append(m)
            if m.leaf_mode >= 0:
                f.leaf_node[m.leaf_mode] = m.address
        na += t.n_nodes
        nm += t.n_leaves
    f.tops = [n.address for n in f.nodes if n.parent < 0]
    return f, node_off, mode_off


def forest_sop(sops, mode_off):
    """One SOP over a forest: every term keeps its own tree's leaves (modes
    offset), operators pooled into one table."""
    ops = OperatorTable()
    out = SOP(ops)
    for sop, mo in zip(sops, mode_off):
        remap = {}
        for l, term in enumerate(sop.terms):
            fac = []
            for (m, o) in term.factors:
                if o not in remap:
                    remap[o] = ops.add(None, sop.ops.kind[o], sop.ops.dense(o) if sop.ops.kind[o] == OP_DENSE
                                       else sop.ops.data[o])
                fac.append((m + mo, remap[o]))
            out.push_back(MLO(fac), sop.coeffs[l])
    return out


def forest_psi(f, psis):
    return TensorTree(f, [t for p in psis for t in p.tensors])


def batched_problem(n_trees: int, seed_base: int = 20261203, modes=(8, 16, 32, 48),
                    pdims=(8, 16, 32), bond_range=(4, 24), couplings=(2, 6)):
    """The many-tree batch: every tree draws its mode count, physical
    dimension and per-edge bonds (uniform in bond_range, clamped to the
    product of the child dims and to p at the bottom), and carries its own
    seeded coupled-oscillator SOP with couplings[0]..couplings[1] random
    partners per mode.  Bonds are then balanced (``balance_bonds``) so that
    no density matrix is rank deficient by construction.  Returns
    (trees, sops, psis)."""
    trees, sops, psis = [], [], []
    for t in range(n_trees):
        rng = np.random.default_rng(seed_base + 2 + 7919 * t)
        f = int(rng.choice(modes))
        p = int(rng.choice(pdims))
        edge_rng = np.random.default_rng(seed_base + 3 + 7919 * t)
        tree = balance_bonds(balanced_tree(
            f, p, bond_range[1],
            bonds=lambda h, pp: int(edge_rng.integers(bond_range[0], bond_range[1] + 1))))
        sop = coupled_oscillators(tree, coupling=0.1, rng=rng, pairs_per_mode=couplings)
        psi = random_wavefunction(tree, seed_base + 4 + 7919 * t)
        trees.append(tree)
        sops.append(sop)
        psis.append(psi)
    return trees, sops, psis
