"""CDVR potential path on the CPU: the oracle pinned by independent checks,
and the planned CDVR stages (run by the numpy plan interpreter) against the
oracle."""
import os
import subprocess

import numpy as np
import pytest

import cdvr as C
from helpers import cdvr_device_wsd
from plan_emulator import B_MATS, PlanView
from qutree_gb300.model import (MLO, OP_DENSE, SOP, HOBasis, OperatorTable, PolyPotential, Tree,
                                _Build, random_wavefunction)


def binary4(p, d1, d2):
    leaves = [_Build([p, d1], leaf=True) for _ in range(4)]
    m0 = _Build([d1, d1, d2], children=leaves[:2])
    m1 = _Build([d1, d1, d2], children=leaves[2:])
    return Tree(_Build([d2, d2, 1], children=[m0, m1]))


def binary8(p, d1, d2, d3):
    def pair(a, b, d):
        return _Build([a.dims[-1], b.dims[-1], d], children=[a, b])
    lv = [_Build([p, d1], leaf=True) for _ in range(8)]
    l1 = [pair(lv[2 * i], lv[2 * i + 1], d2) for i in range(4)]
    l2 = [pair(l1[0], l1[1], d3), pair(l1[2], l1[3], d3)]
    return Tree(_Build([d3, d3, 1], children=l2))


def uneven6(p):
    """Six modes: a node with three children, a branch one layer deeper
    than the other; bonds no larger than the density matrices' ranks allow."""
    lv = [_Build([p, 3], leaf=True) for _ in range(6)]
    n3 = _Build([3, 3, 3, 4], children=lv[0:3])
    n2 = _Build([3, 3, 4], children=lv[3:5])
    n2b = _Build([4, 3, 4], children=[n2, lv[5]])
    return Tree(_Build([4, 4, 1], children=[n3, n2b]))


def two_leaf(p):
    leaves = [_Build([p, p], leaf=True) for _ in range(2)]
    return Tree(_Build([p, p, 1], children=leaves))


def kinetic_sop(tree, basis):
    ops = OperatorTable()
    kin = ops.add("kin", OP_DENSE, basis.kin.astype(complex))
    sop = SOP(ops)
    for m in range(tree.n_leaves):
        ml = MLO()
        ml.push_back(kin, m)
        sop.push_back(ml, 1.0)
    return sop


def full_state(tree, psi):
    """Dense wavefunction in the leaf DVR basis (modes in axis order)."""
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"

    def rec(a):
        n = tree.nodes[a]
        if n.is_bottom:
            return psi.tensors[a], [n.leaf_mode]
        parts = [rec(c) for c in n.children]
        ops, subs, out, modes, nxt = [psi.tensors[a]], [letters[:n.order]], "", [], n.order
        for k, (ct, cm) in enumerate(parts):
            s = letters[nxt:nxt + ct.ndim - 1] + letters[k]
            nxt += ct.ndim - 1
            ops.append(ct)
            subs.append(s)
            out += s[:-1]
            modes += cm
        out += letters[n.order - 1]
        return np.einsum(",".join(subs) + "->" + out, *ops), modes
    t, modes = rec(tree.top.address)
    return t[..., 0], modes


def dvr_energy(tree, psi, V, xs):
    t, modes = full_state(tree, psi)
    grids = np.meshgrid(*[xs[m] for m in modes], indexing="ij")
    X = np.zeros(t.shape + (tree.n_leaves,))
    for i, m in enumerate(modes):
        X[..., m] = grids[i]
    w = np.abs(t) ** 2
    return float(np.sum(w * V(X)) / np.sum(w))


def cdvr_energy(tree, psi, V, xs, aligned=False):
    orc = C.CDVROracle(tree, xs, V, aligned=aligned)
    rho = C.density(tree, psi.tensors)
    orc.update(psi, rho)
    top = tree.top.address
    v = orc.apply(psi.tensors[top], top, rho[top])
    phi = psi.tensors[top].ravel(order="F")
    return float(np.vdot(phi, v.ravel(order="F")).real / np.vdot(phi, phi).real)


# --------------------------------------------------------------------------
# the oracle, pinned
# --------------------------------------------------------------------------
def test_noise_is_libstdcxx_normal_sequence(tmp_path):
    """Regularize's noise: std::mt19937(23949) with std::normal_distribution,
    compared with the C++ standard library itself."""
    src = tmp_path / "n.cpp"
    src.write_text('#include <random>\n#include <cstdio>\nint main(){std::mt19937 g(23949);'
                   'std::normal_distribution<double> d;for(int i=0;i<999;++i)printf("%.17g\\n",d(g));}\n')
    exe = tmp_path / "n"
    subprocess.check_call(["g++", "-O2", "-o", str(exe), str(src)])
    ref = np.array([float(x) for x in subprocess.check_output([str(exe)]).split()])
    tree = binary4(5, 4, 3)  # 4*20 + 2*48 + 9 = 185 numbers
    tree2 = binary8(6, 5, 6, 7)
    got = np.concatenate(C.regularize_noise(tree2, eps=1.0))[:999]
    assert np.array_equal(got, ref)
    got1 = np.concatenate(C.regularize_noise(tree, eps=1.0))
    assert np.array_equal(got1, ref[:got1.size])


@pytest.mark.parametrize("aligned", [False, True])
def test_two_modes_complete_basis_is_exact(aligned):
    """With complete single-particle bases on two modes every grid is a
    single-matrix eigenproblem and CDVR gives the DVR potential energy."""
    p = 6
    tree = two_leaf(p)
    xs = {m: HOBasis(p).x for m in range(2)}
    V = PolyPotential.cdvr_model(2)
    for seed in (1, 2, 3):
        psi = random_wavefunction(tree, seed)
        e = cdvr_energy(tree, psi, V, xs, aligned)
        assert abs(e - dvr_energy(tree, psi, V, xs)) <= 1e-12 * abs(e)


def test_constant_potential_gives_constant_energy():
    tree = binary4(5, 4, 3)
    xs = {m: HOBasis(5).x for m in range(4)}
    V = PolyPotential(4, [(0.37, [])])
    psi = random_wavefunction(tree, 4)
    assert abs(cdvr_energy(tree, psi, V, xs) - 0.37) < 1e-12


def test_aligned_hole_grids_closer_to_exact_on_complete_tree():
    """Two layers, complete bases: CDVR is close to the DVR energy; the
    reference's rank-ordered hole grids are further off than per-mode ones."""
    p = 3
    tree = binary4(p, p, p * p)
    xs = {m: HOBasis(p).x for m in range(4)}
    V = PolyPotential.cdvr_model(4)
    psi = random_wavefunction(tree, 11)
    ex = dvr_energy(tree, psi, V, xs)
    e_al = cdvr_energy(tree, psi, V, xs, aligned=True)
    e_ref = cdvr_energy(tree, psi, V, xs, aligned=False)
    assert abs(e_al - ex) < 1e-3 * abs(ex)
    assert abs(e_al - ex) < abs(e_ref - ex)


def test_wsd_of_commuting_matrices_finds_their_eigenvalues():
    rng = np.random.default_rng(3)
    d, n = 5, 3
    U, _ = np.linalg.qr(rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)))
    D = [np.sort(rng.standard_normal(d)) for _ in range(n)]
    xs = [U @ np.diag(x) @ U.conj().T for x in D]
    W = np.diag(np.linspace(0.4, 0.1, d)).astype(complex)
    W = U @ W @ U.conj().T
    T, grids, (sweeps, conv) = C.layer_grid_multi(xs, W)
    assert conv == 1
    # T x_k T^dagger is diagonal up to the iteration's tolerance
    for x, g in zip(xs, grids):
        y = T @ x @ T.conj().T
        assert np.abs(y - np.diag(np.diag(y))).max() < 1e-3
        assert np.allclose(np.sort(g), np.sort(np.diag(y).real), atol=1e-3)


# --------------------------------------------------------------------------
# planned CDVR stages against the oracle
# --------------------------------------------------------------------------
CASES = [("binary4", lambda: binary4(5, 4, 3), 5), ("binary8", lambda: binary8(6, 4, 5, 4), 6),
         ("uneven6", lambda: uneven6(5), 5)]


@pytest.mark.parametrize("name,mk,p", CASES)
@pytest.mark.parametrize("flavour", [0, 1])
@pytest.mark.parametrize("aligned", [False, True])
def test_emulated_cdvr_sweep_matches_oracle(name, mk, p, flavour, aligned):
    tree = mk()
    basis = HOBasis(p)
    f = tree.n_leaves
    xs = {m: basis.x for m in range(f)}
    sop = kinetic_sop(tree, basis)
    V = PolyPotential.cdvr_model(f)
    V.terms.append((0.01, [(0, 1), (f // 2, 1), (f - 1, 2)]))  # a three-mode term
    psi = random_wavefunction(tree, 7)
    pv = PlanView(tree, sop, flavour=flavour, cdvr=(xs, V, aligned))
    pv.run(psi.flat())
    h00, s00 = pv.energy_parts()
    wsd = emulated_wsd(pv, tree)
    res = C.derivative(tree, sop, psi.flat(), C.CDVROracle(tree, xs, V, aligned=aligned), wsd=wsd)
    assert wsd.calls  # the several-matrix solve ran on the emulated inputs
    assert abs(h00 - res.h00) <= 1e-12 * abs(res.h00)
    scale = np.abs(res.dpsi).max()
    assert np.abs(pv.dpsi() - res.dpsi).max() <= 1e-10 * scale


def emulated_wsd(pv, tree):
    mats = pv.bufs[B_MATS]
    rho = [mats[o:o + n.d_up ** 2].reshape((n.d_up, n.d_up), order="F")
           for o, n in zip(pv.tables[11], tree.nodes)]
    return cdvr_device_wsd(tree, pv.cdvr_arena(), pv.tables[39], rho)


def test_emulated_cdvr_grids_match_oracle():
    tree = binary8(6, 4, 5, 4)
    xs = {m: HOBasis(6).x for m in range(8)}
    V = PolyPotential.cdvr_model(8)
    psi = random_wavefunction(tree, 9)
    pv = PlanView(tree, kinetic_sop(tree, HOBasis(6)), cdvr=(xs, V, False))
    pv.run(psi.flat())
    arena = pv.cdvr_arena()
    orc = C.CDVROracle(tree, xs, V)
    orc.update(psi, wsd=emulated_wsd(pv, tree))
    lay = pv.tables[38]
    for n in tree.nodes:
        if n.is_top:
            continue
        a, d = n.address, n.d_up
        g_off, h_off, ng, nh = lay[a][2], lay[a][3], lay[a][4], lay[a][5]
        for j, m in enumerate(sorted(tree.subtree_modes(a))):
            np.testing.assert_allclose(arena[g_off + j * d:g_off + (j + 1) * d].real, orc.grid[(m, a)],
                                       atol=1e-10)
        vn = arena[lay[a][6]:lay[a][6] + n.size].real
        np.testing.assert_allclose(vn, orc.vnode[a].ravel(order="F"), rtol=1e-10, atol=1e-14)


def test_cdvr_plan_rejections():
    tree = binary4(5, 4, 3)
    basis = HOBasis(5)
    xs = {m: basis.x for m in range(4)}
    sop = kinetic_sop(tree, basis)
    V = PolyPotential.cdvr_model(4)
    with pytest.raises(ValueError, match="reference or grouped"):
        PlanView(tree, sop, flavour=2, cdvr=(xs, V, False))
    with pytest.raises(ValueError, match="complex128"):
        PlanView(tree, sop, flavour=0, prec=1, cdvr=(xs, V, False))
    with pytest.raises(ValueError, match="gradient"):
        PlanView(tree, sop, flavour=0 | 0x1000, cdvr=(xs, V, False))
    bad = {m: basis.x[:4] for m in range(4)}
    with pytest.raises(ValueError, match="leaf dimension"):
        PlanView(tree, sop, flavour=0, cdvr=(bad, V, False))


def test_wsd_eigensolve_matches_a_dense_eigensolver():
    # the optimiser's 3x3 eigenproblem (rfoBuildHessian's H: h22 = 0) as the
    # restatement solves it -- power-of-two scaling, binary32 Newton start,
    # binary64 Newton with binary32 step quotients -- against numpy's eigh:
    # the top eigenvector's ratios v0/v2, v1/v2 and v0^2 + v1^2 over twelve
    # decades of scale (top eigenvalue separated, v2 not small)
    import ctypes
    lib = ctypes.CDLL(C.build_wsd())
    f = lib.orc_eig3_top
    dp = ctypes.POINTER(ctypes.c_double)
    f.argtypes = [ctypes.c_void_p, dp, dp, dp]
    rng = np.random.default_rng(0)
    worst, checked = 0.0, 0
    for _ in range(3000):
        sc = 10.0 ** rng.uniform(-12, 6)
        a = 10.0 ** rng.uniform(-6, 0)
        pre = rng.normal(size=3) * sc
        g = rng.normal(size=2) * np.sqrt(sc)
        H = np.zeros((3, 3))
        H[0, 0], H[1, 1] = pre[0] * a * a, pre[2] * a * a
        H[0, 1] = H[1, 0] = pre[1] * a * a
        H[0, 2] = H[2, 0] = g[0] * a
        H[1, 2] = H[2, 1] = g[1] * a
        Hc = np.ascontiguousarray(H.T.reshape(-1))
        u0, u1, t2 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        f(Hc.ctypes.data, ctypes.byref(u0), ctypes.byref(u1), ctypes.byref(t2))
        w, V = np.linalg.eigh(H)
        v = V[:, -1]
        if abs(v[2]) < 1e-3 * np.abs(v).max() or abs(w[-1] - w[-2]) < 1e-6 * np.abs(w).max():
            continue
        checked += 1
        worst = max(worst, abs(u0.value - v[0] / v[2]) / (1 + abs(v[0] / v[2])),
                    abs(u1.value - v[1] / v[2]) / (1 + abs(v[1] / v[2])), abs(t2.value - (v[0] ** 2 + v[1] ** 2)))
    assert checked > 2000 and worst < 1e-11
