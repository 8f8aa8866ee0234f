"""CPU restatement of QuTree's CDVR potential path (Hamiltonians with a
non-SOP potential, ``H.hasV``).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU CDVR
stages and by bench.py's CPU-baseline leg; the product path never imports
this module.

Follows, routine by routine (numpy, complex128):
  CDVR::Update                       src/DVR/CDVR.cpp:150-175
  XMatrixTrees (x represent, holes)  include/DVR/XMatrixTrees.h:22-84
  Regularize (seeded noise + GS)     src/DVR/XMatrixTrees.cpp:6-19
  SparseTree without tail / inverse  src/TreeClasses/SparseTree.cpp:33-108
  contraction with hole weights      include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:144-240,296-353
  TDDVR::update, LayerGrid, setGrids src/DVR/TDDVR.cpp:12-110
  weighted simultaneous diagonalisation  oracle/cdvr_wsd.cpp (C, fixed operation order)
  MatrixTensorTree                   src/DVR/MatrixTensorTree.cpp:12-75
  orthogonal                         include/TreeClasses/TensorTree_Implementation.h:142-171
  sqrt / inverse of matrix trees     src/TreeClasses/SpectralDecompositionTree.cpp:98-125,
                                     include/Core/Matrix_Implementation.h:636-668
  GridTransformation                 src/DVR/TDDVR.cpp:186-205,236-270
  UpdateNodeDVR / UpdateEdgeDVR      src/DVR/CDVR.cpp:21-88
  fillX / fillXNode / fillXEdge      src/DVR/cdvr_functions.cpp:25-65
  calculateDeltaVs (local, E, F)     src/DVR/cdvr_functions.cpp:67-215
  doubleHoleContraction              include/Core/Tensor_Extension_Implementation.h:215-239
  CDVR::apply                        src/DVR/CDVR.cpp:90-123
  cdvr_functions::apply              src/DVR/cdvr_functions.cpp:217-275
  Apply (+= cdvr_.apply)             src/TreeClasses/HamiltonianRepresentation.cpp:30-32

Two behaviours of the reference are kept on purpose:
  * the X-matrix holes live on every node except the leaf's own bottom node
    (tail=false, inverse tree) while the hole grids live only on nodes whose
    subtree does not hold the leaf (tail=true, inverse tree); setGrids hands
    the hole diagonals out by rank, so on an upper node whose subtree holds
    low-numbered modes a hole grid receives the diagonal of another mode's
    matrix.  ``aligned=True`` gives every hole grid its own mode's diagonal
    instead (not the reference's behaviour).
  * the X-matrix holes are built on a copy of Psi with seeded noise
    (std::mt19937(23949), std::normal_distribution, amplitude 1e-4 on the
    real parts) and Gram-Schmidt, restated here from the published
    Mersenne-Twister and Marsaglia polar methods as libstdc++ applies them.
The reference's Potential is any C++ function of the coordinates; this
restatement (like the device path) takes polynomial potentials
V(x) = sum_t c_t prod_(g,p) x_g^p, which covers contrib's CDVRModelV.
Parity of this restatement is pinned by independent checks in the tests
(complete single-particle bases give the exact DVR potential energy; a
constant potential gives E = c); QuTree has no CDVR test of its own.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

from qutree_gb300.model import PolyPotential, TensorTree, gram_schmidt, hole_product, mode_product  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")


# --------------------------------------------------------------------------
# weighted simultaneous diagonalisation (C, bit-fixed operation order)
# --------------------------------------------------------------------------
def build_wsd(quiet: bool = True) -> str:
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libcdvr_wsd.so")
    src = os.path.join(HERE, "cdvr_wsd.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o",
           out + ".tmp", src]
    subprocess.check_call(cmd, stdout=subprocess.DEVNULL if quiet else None)
    os.replace(out + ".tmp", out)
    return out


_wsd = None


def _wsd_lib():
    global _wsd
    if _wsd is None:
        L = ctypes.CDLL(build_wsd())
        L.orc_layer_grid.restype = ctypes.c_int
        L.orc_layer_grid.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p]
        _wsd = L
    return _wsd


def layer_grid_multi(xs, W, eps: float = 1e-5):
    """LayerGrid with several matrices (src/DVR/TDDVR.cpp:72-88): returns
    (trafo = T^dagger, [grid_k], (sweeps, converged))."""
    n, d = len(xs), W.shape[0]
    X = np.zeros((n, d, d), dtype=np.complex128)
    for k, x in enumerate(xs):
        X[k] = np.asarray(x).T  # column-major per matrix
    X = np.ascontiguousarray(X)
    Wc = np.ascontiguousarray(np.asarray(W, dtype=np.complex128).T)
    T = np.zeros((d, d), dtype=np.complex128)
    g = np.zeros((n, d))
    info = np.zeros(2, dtype=np.int32)
    rc = _wsd_lib().orc_layer_grid(n, d, X.ctypes.data, Wc.ctypes.data, eps, T.ctypes.data,
                                   g.ctypes.data, info.ctypes.data)
    if rc != 0:
        raise RuntimeError("orc_layer_grid failed")
    return T.T.copy(), [g[k].copy() for k in range(n)], (int(info[0]), int(info[1]))


def layer_grid_single(x):
    """LayerGrid with one matrix (src/DVR/TDDVR.cpp:68-71): diagonalize,
    trafo = U^dagger, grid = ascending eigenvalues."""
    w, U = np.linalg.eigh(0.5 * (x + x.conj().T))
    return U.conj().T.copy(), [w.copy()]


# --------------------------------------------------------------------------
# seeded noise of Regularize (std::mt19937 + std::normal_distribution)
# --------------------------------------------------------------------------
def regularize_noise(tree, eps: float = 1e-4, seed: int = 23949):
    """Per node (address order) the real noise eps * N(0,1) that Regularize
    (src/DVR/XMatrixTrees.cpp:6-19) adds element by element.  Uniform
    deviates: generate_canonical<double, 53> from two 32-bit outputs,
    (g0 + g1 2^32) / 2^64; normals: Marsaglia's polar method, the second
    variate of each pair returned first and the first one saved."""
    total = sum(n.size for n in tree.nodes)
    mt = np.random.MT19937()
    mt._legacy_seeding(seed)
    # at most 4/pi pairs per normal pair on average; draw generously
    raw = mt.random_raw(int(4 * total + 4096)).astype(np.float64)
    pos = 0

    def canon():
        nonlocal pos, raw
        if pos + 2 > raw.size:
            raw = np.concatenate([raw, mt.random_raw(4096).astype(np.float64)])
        s = raw[pos] + raw[pos + 1] * 4294967296.0
        pos += 2
        r = s / 18446744073709551616.0
        return r if r < 1.0 else math.nextafter(1.0, 0.0)

    saved = None
    out = []
    for n in tree.nodes:
        v = np.zeros(n.size)
        for i in range(n.size):
            if saved is not None:
                z, saved = saved, None
            else:
                while True:
                    x = 2.0 * canon() - 1.0
                    y = 2.0 * canon() - 1.0
                    r2 = x * x + y * y
                    if not (r2 > 1.0 or r2 == 0.0):
                        break
                mult = math.sqrt(-2 * math.log(r2) / r2)
                saved = x * mult
                z = y * mult
            v[i] = eps * z
        out.append(v)
    return out


# --------------------------------------------------------------------------
# tree helpers
# --------------------------------------------------------------------------
def density(tree, ts):
    """TreeFunctions::contraction(Rho, Psi, tree, orthogonal=true)
    (include/TreeClasses/MatrixTreeFunctions_Implementation.h:58-102)."""
    rho = [None] * tree.n_nodes
    for n in reversed(tree.nodes):
        if n.is_top:
            rho[n.address] = np.eye(n.d_up, dtype=np.complex128)
        else:
            p = tree.nodes[n.parent]
            ket = mode_product(rho[p.address], ts[p.address], p.order - 1)
            rho[n.address] = hole_product(ts[p.address], ket, n.child_idx)
    return rho


def spectral(m, fn):
    """U f(lambda) U^dagger of a Hermitian matrix (toMatrix of a spectral
    decomposition with a function applied to the eigenvalues)."""
    w, U = np.linalg.eigh(0.5 * (m + m.conj().T))
    return (U * fn(w)) @ U.conj().T


def sqrt_ev(w):
    return np.sqrt(np.maximum(w, 0.0))


def reg_inverse(eps):
    """inverse(Vector, eps) (include/Core/Vector_Implementation.h:266-280)."""
    return lambda w: 1.0 / (w + eps * np.exp(-w / eps))


def _as_mat(t):
    """(lastBefore, last) view of a node tensor."""
    return t.reshape((-1, t.shape[-1]), order="F")


def double_hole(A, B, k1, k2):
    """doubleHoleContraction: C[a, b, c, e] = sum over all other indices of
    conj(A[.. a@k1 .. b@k2 ..]) B[.. c@k1 .. e@k2 ..]."""
    Am = np.moveaxis(A, (k1, k2), (0, 1)).reshape(A.shape[k1], A.shape[k2], -1)
    Bm = np.moveaxis(B, (k1, k2), (0, 1)).reshape(B.shape[k1], B.shape[k2], -1)
    return np.einsum("abr,cer->abce", Am.conj(), Bm)


def orthogonal(tree, ts):
    """orthogonal(Psi, tree) (include/TreeClasses/TensorTree_Implementation.h:142-171)."""
    ts = [t.copy() for t in ts]
    for n in tree.nodes:
        if n.is_top:
            continue
        phi = ts[n.address]
        S = hole_product(phi, phi, n.order - 1)
        w, U = np.linalg.eigh(0.5 * (S + S.conj().T))
        SW = ((U * np.sqrt(np.maximum(w, 0.0))) @ U.conj().T).T
        p = n.parent
        ts[p] = mode_product(SW, ts[p], n.child_idx)
        ts[n.address] = gram_schmidt(_as_mat(phi)).reshape(n.shape, order="F")
    return ts


# --------------------------------------------------------------------------
# CDVR
# --------------------------------------------------------------------------
class CDVROracle:
    """CDVR(tree) with Update(Psi, V, tree) and apply(Phi, rho_x, node)."""

    def __init__(self, tree, leaf_x, potential: PolyPotential, aligned: bool = False,
                 use_orthogonal: bool = True):
        self.tree = tree
        self.f = tree.n_leaves
        self.leaf_x = {m: np.asarray(leaf_x[m], dtype=np.float64) for m in range(self.f)}
        self.V = potential
        self.aligned = aligned
        self.use_orthogonal = use_orthogonal
        self.sub = {n.address: sorted(tree.subtree_modes(n.address)) for n in tree.nodes}
        self.noise = regularize_noise(tree)

    # -- X matrices ----------------------------------------------------------
    def x_mats(self, ts):
        """represent(mats_, Xsop, Psi, Psi) on the leaf-to-root paths (tail=true)."""
        tree = self.tree
        mats = [dict() for _ in range(self.f)]
        for l in range(self.f):
            prev = None
            for a in tree.path_to_root(l):
                n = tree.nodes[a]
                if n.is_top:
                    break
                phi = ts[a]
                if n.is_bottom:
                    t = self.leaf_x[l].reshape((-1,) + (1,) * (n.order - 1)) * phi
                else:
                    c = tree.nodes[prev]
                    t = mode_product(mats[l][prev], phi, c.child_idx)
                mats[l][a] = hole_product(phi, t, n.order - 1)
                prev = a
        return mats

    def chi(self, ts):
        """Regularize(Psi, tree, sqrt(1e-8)): noise on the real parts, then gramSchmidt."""
        out = []
        for n, t, z in zip(self.tree.nodes, ts, self.noise):
            a = t.ravel(order="F") + z
            a = a.reshape((-1, n.d_up), order="F")
            out.append(gram_schmidt(a).reshape(n.shape, order="F"))
        return out

    def x_holes(self, mats, chi):
        """contraction(holes_, Chi, Chi, mats_, rho, tree) on the inverse trees
        of the tail-free leaf trees, then UnweightContractions."""
        tree = self.tree
        holes = [dict() for _ in range(self.f)]
        for l in range(self.f):
            bottom = tree.leaf_node[l]
            path = set(tree.path_to_root(l))
            for n in reversed(tree.nodes):
                a = n.address
                if a == bottom:
                    continue
                if n.is_top:
                    holes[l][a] = np.eye(n.d_up, dtype=np.complex128)
                    continue
                p = tree.nodes[n.parent]
                t = chi[p.address]
                for k, c in enumerate(p.children):
                    if k == n.child_idx or c not in path:
                        continue
                    t = mode_product(mats[l][c], t, k)
                if not p.is_top:
                    t = mode_product(holes[l][p.address], t, p.order - 1)
                holes[l][a] = hole_product(chi[p.address], t, n.child_idx)
        rho_chi = density(tree, chi)
        for l in range(self.f):
            for a in list(holes[l].keys()):
                n = tree.nodes[a]
                if n.is_top:
                    continue
                rs = spectral(rho_chi[a], sqrt_ev)
                isq = spectral(rs, reg_inverse(1e-8))
                holes[l][a] = isq @ holes[l][a] @ isq
        return holes

    # -- grids ---------------------------------------------------------------
    def grid_problems(self, a):
        """(modes of the X list, modes of the active grid trees) for the node
        grid and the hole grid of node a."""
        tree = self.tree
        sub = self.sub[a]
        g_list = list(sub)
        h_list = [l for l in range(self.f) if tree.leaf_node[l] != a]
        h_grids = [l for l in range(self.f) if l not in sub]
        return g_list, h_list, h_grids

    def grids(self, mats, holes, rho, wsd=None):
        """TDDVR::update's two updateGrids.  ``wsd(kind, node, xs, W)``, when
        given, replaces the several-matrix solve (kind "grid" or "hole"); the
        parity tests pass one that runs this module's solver on the device's
        own inputs, because the solver's accept / reject steps make its
        result discontinuous in its inputs."""
        tree = self.tree
        self.trafo, self.htrafo = {}, {}
        self.grid, self.hgrid = {}, {}  # (mode, node) -> vector
        self.wsd_info = {}
        for n in tree.nodes:
            a = n.address
            if n.is_top:
                self.trafo[a] = np.eye(n.d_up, dtype=np.complex128)
                self.htrafo[a] = np.eye(n.d_up, dtype=np.complex128)
                continue
            g_list, h_list, h_grids = self.grid_problems(a)
            for kind, xs_modes, src in (("grid", g_list, mats), ("hole", h_list, holes)):
                xs = [src[l][a] for l in xs_modes]
                if len(xs) == 1:
                    T, diag = layer_grid_single(xs[0])
                    info = None
                elif wsd is not None:
                    T, diag, info = wsd(kind, a, xs, rho[a])
                else:
                    T, diag, info = layer_grid_multi(xs, rho[a])
                self.wsd_info[(kind, a)] = info
                if kind == "grid":
                    self.trafo[a] = T
                    for j, l in enumerate(xs_modes):
                        self.grid[(l, a)] = diag[j]
                else:
                    self.htrafo[a] = T
                    for r, l in enumerate(h_grids):
                        j = xs_modes.index(l) if self.aligned else r
                        self.hgrid[(l, a)] = diag[j]

    # -- potential on node and edge grids -------------------------------------
    def coords_node(self, a):
        """Per mode: (tensor index, grid vector) of fillXNode."""
        tree = self.tree
        n = tree.nodes[a]
        src = {}
        if n.is_bottom:
            src[n.leaf_mode] = (0, self.leaf_x[n.leaf_mode])
        else:
            for k, c in enumerate(n.children):
                for l in self.sub[c]:
                    src[l] = (k, self.grid[(l, c)])
        if not n.is_top:
            for l in range(self.f):
                if l not in self.sub[a]:
                    src[l] = (n.order - 1, self.hgrid[(l, a)])
        return src

    def coords_edge(self, a):
        src = {}
        for l in range(self.f):
            if l in self.sub[a]:
                src[l] = (0, self.grid[(l, a)])
            else:
                src[l] = (1, self.hgrid[(l, a)])
        return src

    def _eval(self, shape, src):
        X = np.zeros(tuple(shape) + (self.f,))
        for l in range(self.f):
            k, g = src[l]
            sh = [1] * len(shape)
            sh[k] = len(g)
            X[..., l] = np.broadcast_to(np.asarray(g).reshape(sh), shape)
        return self.V(X)

    # -- update --------------------------------------------------------------
    def update(self, psi: TensorTree, rho=None, wsd=None):
        """CDVR::Update (src/DVR/CDVR.cpp:150-175)."""
        tree = self.tree
        ts = psi.tensors
        if rho is None:
            rho = density(tree, ts)
        self.rho = rho
        mats = self.x_mats(ts)
        chi = self.chi(ts)
        holes = self.x_holes(mats, chi)
        self.mats, self.holes = mats, holes
        self.grids(mats, holes, rho, wsd)
        # MatrixTensorTree(Psi, tree, true)
        nodes = orthogonal(tree, ts) if self.use_orthogonal else [t.copy() for t in ts]
        rhoN = density(tree, nodes)
        edges = {}
        for n in tree.nodes:
            if n.is_top:
                continue
            B = spectral(rhoN[n.address], sqrt_ev)
            nodes[n.address] = mode_product(B, nodes[n.address], n.order - 1)
            edges[n.address] = spectral(B, reg_inverse(1e-7))
        # GridTransformation
        for n in tree.nodes:
            a = n.address
            t = nodes[a]
            if not n.is_bottom:
                for k, c in enumerate(n.children):
                    t = mode_product(self.trafo[c], t, k)
            if not n.is_top:
                t = mode_product(self.htrafo[a], t, n.order - 1)
            nodes[a] = t
        for a in edges:
            edges[a] = self.trafo[a].conj() @ edges[a] @ self.htrafo[a].conj().T
        self.at, self.edges = nodes, edges
        # potential on node and edge grids
        self.vnode = {n.address: self._eval(n.shape, self.coords_node(n.address))
                      for n in tree.nodes}
        self.vedge = {a: self._eval((tree.nodes[a].d_up,) * 2, self.coords_edge(a)) for a in edges}
        # bottom-up and top-down normalised coefficients
        self.cup, self.cdown = {}, {}
        for n in tree.nodes:
            a = n.address
            if n.is_top:
                self.cup[a] = nodes[a]
                continue
            self.cup[a] = mode_product(edges[a], nodes[a], n.order - 1)
            self.cdown[a] = mode_product(edges[a].T, nodes[n.parent], n.child_idx)
        self.delta_vs()

    def delta_vs(self):
        """calculateDeltaVs (src/DVR/cdvr_functions.cpp:199-215)."""
        tree = self.tree
        self.dv = {}
        for n in tree.nodes:
            if n.is_top:
                continue
            a = n.address
            d = n.d_up
            cu = _as_mat(self.cup[a])
            vn = _as_mat(self.vnode[a].astype(np.complex128))
            T = np.einsum("bl,bi,bm->lim", cu.conj(), vn, cu)
            dv = np.zeros((d, d, d, d), dtype=np.complex128)
            for i0 in range(d):
                dv[:, i0, :, i0] = T[:, i0, :]
            for l0 in range(d):
                for l1 in range(d):
                    dv[l0, l1, l0, l1] -= self.vedge[a][l0, l1]
            if not n.is_bottom:
                last = n.order - 1
                for k, c in enumerate(n.children):
                    D = double_hole(self.cdown[c], self.cup[a], k, last)
                    F = double_hole(self.cup[a], self.cdown[c], k, last)
                    E = np.einsum("abxy,yjxi->abij", self.dv[c], D)
                    dv += np.einsum("xayb,xyij->abij", F, E)
            self.dv[a] = dv

    # -- apply ---------------------------------------------------------------
    def apply(self, phi, a, rho_a):
        """CDVR::apply (src/DVR/CDVR.cpp:90-123) with cdvr_functions::apply."""
        n = self.tree.nodes[a]
        last = n.order - 1
        sq = None
        if not n.is_top:
            sq = spectral(rho_a, lambda w: (lambda g: g + 1e-6 * np.exp(-g / 1e-6))(sqrt_ev(w)))
            phi = mode_product(sq, phi, last)
        if not n.is_bottom:
            for k, c in enumerate(n.children):
                phi = mode_product(self.trafo[c], phi, k)
        if not n.is_top:
            phi = mode_product(self.htrafo[a], phi, last)
        v = self.vnode[a] * phi
        if not n.is_bottom:
            for k, c in enumerate(n.children):
                x = hole_product(self.cdown[c], phi, k)
                y = np.einsum("abxy,yx->ab", self.dv[c], x)
                v = v + mode_product(y, self.cdown[c], k)
        if not n.is_bottom:
            for k, c in enumerate(n.children):
                v = mode_product(self.trafo[c].conj().T, v, k)
        if not n.is_top:
            v = mode_product(self.htrafo[a].conj().T, v, last)
            v = mode_product(sq.conj().T, v, last)
        return v


# --------------------------------------------------------------------------
# the sweep with the CDVR term
# --------------------------------------------------------------------------
def rho_list(tree, flat_rho):
    out, off = [], 0
    for n in tree.nodes:
        d = n.d_up
        out.append(flat_rho[off:off + d * d].reshape((d, d), order="F"))
        off += d * d
    return out


def derivative(tree, sop, psi_flat, cdvr: CDVROracle, eps=1e-10, phase=1.0, wsd=None):
    """Derivative() of a Hamiltonian with SOP part ``sop`` and potential
    ``cdvr.V``: the oracle's SOP sweep plus, per node, the CDVR term of Apply
    taken through the same projector and inverse density
    (src/TreeClasses/HamiltonianRepresentation.cpp:6-81)."""
    import oracle as orc
    res = orc.derivative(tree, sop, psi_flat, eps=eps, phase=phase)
    rho = rho_list(tree, res.rho)
    rhoinv = rho_list(tree, res.rhoinv)
    psi = TensorTree.from_flat(tree, np.asarray(psi_flat))
    cdvr.update(psi, rho, wsd=wsd)
    alpha = -1j * complex(phase)
    dpsi = TensorTree.from_flat(tree, res.dpsi.copy())
    h00 = res.h00
    vphi = {}
    for n in tree.nodes:
        a = n.address
        phi = psi.tensors[a]
        v = cdvr.apply(phi, a, rho[a])
        vphi[a] = v
        if n.is_top:
            dpsi.tensors[a] = dpsi.tensors[a] + alpha * v
            h00 = h00 + np.vdot(phi.ravel(order="F"), v.ravel(order="F"))
        else:
            P = _as_mat(phi)
            X = _as_mat(v)
            S = P.conj().T @ P
            D = P.conj().T @ X
            Y = X - P @ np.linalg.solve(S, D)
            dpsi.tensors[a] = dpsi.tensors[a] + (alpha * Y @ rhoinv[a].T).reshape(n.shape, order="F")
    res.dpsi = dpsi.flat()
    res.h00 = h00
    res.vphi = vphi
    return res
