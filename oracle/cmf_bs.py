"""CPU restatement of QuTree's adaptive constant-mean-field integrator:
CMFIntegrator::Integrate / CMFstep / Error (src/Applications/CMFIntegrator.cpp:
25-218) with one Bulirsch-Stoer integrator per node (include/Util/
BS_integrator.h:11-268), the node error of LayerInterface::Error
(src/TreeClasses/LayerInterface.cpp:5-31) and the re-orthonormalisation
orthogonal() after accepted steps (include/TreeClasses/TensorTree_Implementation.h:
142-169, gramSchmidt of include/Core/Tensor_Implementation.h:805-850).

TEST INFRASTRUCTURE ONLY: the checker of qutree_gb300/cmf.py.  The product
path never imports it.

Sequential, as the reference runs it: node after node, each node's
integrator from its own step size.  The frozen-matrix derivatives come from a
session object with build(psi), deriv_node(n, phi) (node n's
LayerDerivative with the matrices of the last build) and rho() --
oracle.Frozen for the CPU oracle.
"""
from __future__ import annotations

import math

import numpy as np


class BSIntegrator:
    """BS_integrator (include/Util/BS_integrator.h): modified-midpoint steps
    of the sequence 2, 4, 6, 8, 12, 16, ... with rational extrapolation in
    h^2 (rzextr) over at most `maxuse` estimates and step-size control."""

    def __init__(self, dim: int):
        self.dim = dim
        self.maxuse, self.max_ = 7, 11
        self.shrink, self.grow = 0.95, 1.2
        seq = [2, 4, 6]
        for i in range(3, self.max_):
            seq.append(seq[i - 2] * 2)
        self.sequence = seq
        self.yvec = [np.zeros(dim, np.complex128) for _ in range(5)]
        self.ytab = [np.zeros(dim, np.complex128) for _ in range(self.maxuse)]
        self.xtab = [0.0] * self.max_

    def integrate(self, y, x, xend, dx, eps, ddx, err):
        """Integrate from x to xend; returns (y, x, dx)."""
        while xend - x > dx * 1e-6:
            if x + dx > xend:
                dx = xend - x + 1e-10
            y, x, dx = self.bsstep(y, x, dx, eps, ddx, err)
        return y, x, dx

    def clearmemory(self):
        for a in self.yvec:
            a[:] = 0
        for a in self.ytab:
            a[:] = 0
        self.xtab = [0.0] * self.max_

    def bsstep(self, y, x, dx, eps, ddx, err):
        self.clearmemory()
        yv = self.yvec
        yv[0][:] = y
        yv[3][:] = y
        yv[4][:] = ddx(x, y)
        h = dx
        end = False
        while not end:
            i = 0
            while not (end or i >= self.max_):
                self.mmid(x, h / (1.0 * self.sequence[i]), self.sequence[i], ddx)
                x_est = (h / (1.0 * self.sequence[i])) ** 2
                self.rzextr(i, x_est, yv[0], yv[1], yv[2])
                yv[0][:] = yv[1]
                yv[1] += yv[2]
                error = err(yv[0], yv[1])
                if error < eps:
                    x += h
                    if i == self.maxuse - 1:
                        dx = h * self.shrink
                    elif i == self.maxuse - 2:
                        dx = h * self.grow
                    else:
                        dx = (h * self.sequence[self.maxuse - 2]) / (1.0 * self.sequence[i])
                    end = True
                i += 1
            if not end:
                h = h / 4.0
                k = 0
                while k < (self.max_ - self.maxuse) / 2.0:
                    h /= 2.0
                    k += 1
                if dx + h == dx:
                    raise RuntimeError("BS integrator: step size underflow")
        return yv[0].copy(), x, dx

    def mmid(self, xstart, h, step, ddx):
        yv = self.yvec
        yv[0][:] = yv[3]
        yv[1][:] = yv[3] + h * yv[4]
        x = xstart + h
        yv[2][:] = ddx(x, yv[1])
        for _ in range(1, step):
            yv[2][:] = yv[0] + 2 * h * yv[2]
            yv[0][:] = yv[1]
            yv[1][:] = yv[2]
            x += h
            yv[2][:] = ddx(x, yv[1])
        yv[0][:] = (yv[0] + yv[1] + h * yv[2]) / 2.0

    def rzextr(self, i_est, x_est, yest, ysav, dy):
        self.xtab[i_est] = x_est
        if i_est == 0:
            ysav[:] = yest
            dy[:] = yest
            self.ytab[0][:] = yest
            return
        mi = i_est + 1 if i_est < self.maxuse else self.maxuse
        fx = [0.0] * self.maxuse
        for k in range(1, mi):
            fx[k] = self.xtab[i_est - k] / x_est
        yy = yest.copy()
        v = self.ytab[0].copy()
        c = yy.copy()
        self.ytab[0][:] = yy
        ddy = np.zeros_like(yy)
        for k in range(1, mi):
            bi = fx[k] * v
            b = bi - c
            nz = np.abs(b) != 0
            q = np.divide(c - v, b, out=np.zeros_like(b), where=nz)
            ddy = np.where(nz, c * q, v)
            c = np.where(nz, bi * q, c)
            v = self.ytab[k].copy()
            self.ytab[k][:] = ddy
            yy = yy + ddy
        dy[:] = ddy
        ysav[:] = yy


def layer_error(phi, chi, rho_n, d, top):
    """LayerInterface::Error: the rho-weighted node difference, relative."""
    diff = (phi - chi).reshape((-1, d), order="F")
    if top:
        delta = float(np.sum((np.conj(diff) * diff).real))
        P = phi.reshape((-1, d), order="F")
        norm = abs(np.trace(P.conj().T @ P))
    else:
        G = diff.conj().T @ diff  # G[n, m] = sum_i conj(D[i, n]) D[i, m]
        delta = float(np.sum(rho_n * G).real)
        norm = abs(np.trace(rho_n))
    return math.sqrt(abs(delta / norm))


def gram_schmidt(A):
    """gramSchmidt (include/Core/Tensor_Implementation.h:805-850) on the
    columns of A (lastBefore x lastDimension), in place."""
    n_col = A.shape[1]
    for n in range(n_col):
        it, accum = 0, 1.0
        while accum > 1e-12 and it < 15:
            it += 1
            accum = 0.0
            for m in range(n):
                ov = np.vdot(A[:, m], A[:, n])
                accum += abs(ov)
                A[:, n] -= ov * A[:, m]
            nrm = np.vdot(A[:, n], A[:, n])
            if abs(nrm) != 0:
                A[:, n] /= math.sqrt(nrm.real)


def orthogonal(tree, psi):
    """orthogonal(TensorTree&, const Tree&): bottom-up, S^(1/2) of each
    non-top node into its parent, then Gram-Schmidt of the node."""
    off = tree.offsets()
    for node in tree.nodes:
        if node.is_top:
            continue
        a = node.address
        d = node.d_up
        Phi = psi[off[a]:off[a + 1]].reshape((-1, d), order="F")
        S = Phi.conj().T @ Phi
        w, U = np.linalg.eigh(S)
        root = np.sqrt(np.maximum(w, 0.0))
        SW = (U * root) @ U.conj().T  # S^(1/2)
        SW = SW.T                     # SW(j, k) = sum_l U(k, l) sqrt(w_l) conj(U(j, l))
        p = tree.nodes[node.parent]
        pa = p.address
        shape = list(p.shape)
        k = node.child_idx
        B = psi[off[pa]:off[pa + 1]].reshape(shape, order="F")
        B = np.moveaxis(np.tensordot(SW, B, axes=([1], [k])), 0, k)  # matrixTensor(SW, B, k)
        psi[off[pa]:off[pa + 1]] = B.reshape(-1, order="F")
        A = Phi.copy()
        gram_schmidt(A)
        psi[off[a]:off[a + 1]] = A.reshape(-1, order="F")


def rho_blocks(tree, rho_flat):
    out, ro = {}, 0
    for n in tree.nodes:
        d = n.d_up
        out[n.address] = rho_flat[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
    return out


def cmf_integrate(tree, frozen, psi, t0, t_end, dt, out, acc_root, acc_leaf):
    """CMFIntegrator::Integrate from t0 to t_end with initial step dt and
    output interval `out`; returns (psi, dt, stats)."""
    off = tree.offsets()
    nodes = tree.nodes
    tconst, max_increase = 0.25, 2.25
    bs = {n.address: BSIntegrator(int(off[n.address + 1] - off[n.address])) for n in nodes}
    dt_bs = {n.address: dt / 2.0 for n in nodes}
    psi = np.array(psi, dtype=np.complex128, copy=True)
    time = t0
    t_next = time + out
    frozen.build(psi)
    calc_mat = False
    err = 0.0
    stats = {"accepted": 0, "refused": 0, "builds": 1}

    def cmf_step(Y, t_a, t_b):
        rho = rho_blocks(tree, frozen.rho())
        for n in nodes:
            a = n.address
            sl = slice(off[a], off[a + 1])
            d = n.d_up

            def ddx(x, phi, a=a):
                return frozen.deriv_node(a, phi)

            def errf(p1, p2, a=a, d=d, top=n.is_top):
                return layer_error(p1, p2, rho[a], d, top)

            y, _, dt_bs[a] = bs[a].integrate(Y[sl].copy(), t_a, t_b, dt_bs[a], acc_leaf, ddx, errf)
            Y[sl] = y

    while time + 1e-6 < t_end:
        dtmax = min(t_end - time, t_next - time)
        if dt > dtmax:
            dt = dtmax
        elif 2 * dt > dtmax:
            dt = min(dt, dtmax * 0.6)
        psi0 = psi.copy()
        if calc_mat:
            frozen.build(psi)
            stats["builds"] += 1
            calc_mat = False
        ts = dt * tconst
        cmf_step(psi, time, time + ts)
        psi2 = psi.copy()
        cmf_step(psi2, time + ts, time + 2 * ts)
        frozen.build(psi2)
        cmf_step(psi, time + dt * tconst, time + dt * (1 - tconst))
        psi2 = psi0.copy()
        cmf_step(psi2, time, time + dt)
        frozen.build(psi2)
        stats["builds"] += 2
        cmf_step(psi, time + dt * (1 - tconst), time + dt)
        rho = rho_blocks(tree, frozen.rho())
        e2 = 0.0
        for n in nodes:
            a = n.address
            sl = slice(off[a], off[a + 1])
            e2 += layer_error(psi[sl], psi2[sl], rho[a], n.d_up, n.is_top) ** 2
        err = math.sqrt(e2) * 0.25
        if err > acc_root:
            psi = psi0
            calc_mat = True
            dt *= (acc_root / err) ** (1.0 / 3.0) * 0.8
            stats["refused"] += 1
        else:
            time += dt
            orthogonal(tree, psi)
            if time + 1e-10 >= t_next:
                t_next = time + out
            fac = max_increase if err == 0 else min((acc_root / err) ** (1.0 / 3.0), max_increase)
            dt = dt * fac
            stats["accepted"] += 1
    return psi, dt, stats
