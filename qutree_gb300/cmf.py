"""Adaptive constant-mean-field propagation on the device: QuTree's
CMFIntegrator (src/Applications/CMFIntegrator.cpp:11-218) with a
Bulirsch-Stoer integrator per node (include/Util/BS_integrator.h:11-268).

The reference integrates node after node, each with its own step size, and
evaluates LayerInterface::Derivative one node at a time.  With the mean
fields frozen, node p's derivative depends on node p's tensor only, so here
every node's Bulirsch-Stoer step control runs as a coroutine (a generator
that yields the node tensor it needs the derivative of) and ONE device call
-- qt_layer_derivatives on a wavefunction holding every waiting node's
tensor in its slot -- serves all nodes of a round.  The matrices come from
qt_build on the device; step control, extrapolation and the
re-orthonormalisation (orthogonal(), include/TreeClasses/
TensorTree_Implementation.h:142-169) run on the host in complex128.

Names follow the reference: CMFIntegrator.integrate = Integrate, cmf_step =
CMFstep, error = Error, layer_error = LayerInterface::Error.
"""
from __future__ import annotations

import math

import numpy as np

from . import qtgpu

# BS_integrator's control parameters (BS_integrator::Initialize)
_MAXUSE, _MAX = 7, 11
_SHRINK, _GROW = 0.95, 1.2


def _sequence():
    seq = [2, 4, 6]
    for i in range(3, _MAX):
        seq.append(seq[i - 2] * 2)
    return seq


_SEQ = _sequence()


def layer_error(phi, chi, rho_n, d, top):
    """LayerInterface::Error (src/TreeClasses/LayerInterface.cpp:5-31): the
    difference of two node tensors weighted by the node's density matrix,
    relative to its trace (the top node: plain norm, relative to |Phi|^2)."""
    diff = (phi - chi).reshape((-1, d), order="F")
    if top:
        delta = float(np.sum((np.conj(diff) * diff).real))
        P = phi.reshape((-1, d), order="F")
        norm = abs(np.trace(P.conj().T @ P))
    else:
        G = diff.conj().T @ diff
        delta = float(np.sum(rho_n * G).real)
        norm = abs(np.trace(rho_n))
    return math.sqrt(abs(delta / norm))


def _rzextr(state, i_est, x_est, yest):
    """Rational extrapolation to h -> 0 (BS_integrator::rzextr); returns
    (ysav, dy)."""
    xtab, ytab = state
    xtab[i_est] = x_est
    if i_est == 0:
        ytab[0][:] = yest
        return yest.copy(), yest.copy()
    mi = i_est + 1 if i_est < _MAXUSE else _MAXUSE
    fx = [0.0] + [xtab[i_est - k] / x_est for k in range(1, mi)]
    yy = yest.copy()
    v = ytab[0].copy()
    c = yest.copy()
    ytab[0][:] = yest
    ddy = np.zeros_like(yest)
    for k in range(1, mi):
        bi = fx[k] * v
        b = bi - c
        nz = np.abs(b) != 0
        q = np.divide(c - v, b, out=np.zeros_like(b), where=nz)
        ddy = np.where(nz, c * q, v)
        c = np.where(nz, bi * q, c)
        v = ytab[k].copy()
        ytab[k][:] = ddy
        yy = yy + ddy
    return yy, ddy


def _bs_node(y, x, xend, dx, eps, err):
    """BS_integrator::Integrate of one node as a coroutine: yields the node
    tensor whose derivative it needs, receives that derivative; returns
    (y, dx) at xend."""
    n = y.size
    while xend - x > dx * 1e-6:
        if x + dx > xend:
            dx = xend - x + 1e-10
        # bsstep
        xtab = [0.0] * _MAX
        ytab = [np.zeros(n, np.complex128) for _ in range(_MAXUSE)]
        y3 = y.copy()
        y4 = yield y3
        h = dx
        end = False
        while not end:
            i = 0
            while not (end or i >= _MAX):
                # modified midpoint (mmid) with `step` substeps of hh
                step = _SEQ[i]
                hh = h / (1.0 * step)
                y0 = y3.copy()
                y1 = y3 + hh * y4
                y2 = yield y1
                for _ in range(1, step):
                    y2 = y0 + 2 * hh * y2
                    y0 = y1
                    y1 = y2
                    y2 = yield y1
                y0 = (y0 + y1 + hh * y2) / 2.0
                ysav, dy = _rzextr((xtab, ytab), i, hh ** 2, y0)
                y_est, y_hi = ysav, ysav + dy
                if err(y_est, y_hi) < eps:
                    x += h
                    if i == _MAXUSE - 1:
                        dx = h * _SHRINK
                    elif i == _MAXUSE - 2:
                        dx = h * _GROW
                    else:
                        dx = (h * _SEQ[_MAXUSE - 2]) / (1.0 * _SEQ[i])
                    end = True
                    y = y_est
                i += 1
            if not end:
                h = h / 4.0
                k = 0
                while k < (_MAX - _MAXUSE) / 2.0:
                    h /= 2.0
                    k += 1
                if dx + h == dx:
                    raise RuntimeError("CMF integrator: Bulirsch-Stoer step size underflow")
    return y, dx


def _gram_schmidt(A):
    """gramSchmidt (include/Core/Tensor_Implementation.h:805-850), columns."""
    for n in range(A.shape[1]):
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


class CMFIntegrator:
    """CMFIntegrator on a HamiltonianRepresentation (any plan whose context
    supports qt_build / qt_layer_derivatives, complex128 or double-float)."""

    def __init__(self, hrep, phase: complex = 1.0):
        self.h = hrep
        self.tree = hrep.tree
        self.phase = complex(phase)
        self.tconst = 0.25
        self.max_increase = 2.25
        off = self.tree.offsets()
        self.off = off
        self.slices = {n.address: slice(int(off[n.address]), int(off[n.address + 1])) for n in self.tree.nodes}
        self.dt_bs = {}
        self.rho = {}
        self.stats = {"accepted": 0, "refused": 0, "builds": 0, "derivative_rounds": 0}

    # -- device ---------------------------------------------------------------
    def build(self, psi):
        """HamiltonianRepresentation::build at psi (on the device)."""
        self.h.upload(psi)
        self.h.build()
        flat = self.h.matrices(qtgpu.QT_MAT_RHO)
        ro = 0
        for n in self.tree.nodes:
            d = n.d_up
            self.rho[n.address] = flat[ro:ro + d * d].reshape((d, d), order="F")
            ro += d * d
        self.stats["builds"] += 1

    def _derivatives(self, full):
        self.h.upload(full)
        self.h.layer_derivatives(self.phase)
        self.stats["derivative_rounds"] += 1
        return self.h.dpsi()

    # -- CMFstep ----------------------------------------------------------------
    def cmf_step(self, Y, t_a, t_b, acc_leaf):
        """Every node's tensor in Y from t_a to t_b with the current matrices
        (CMFIntegrator::CMFstep); the nodes' Bulirsch-Stoer integrators run
        side by side, one device derivative call per round."""
        gens, pending = {}, {}
        for n in self.tree.nodes:
            a = n.address

            def err(p1, p2, a=a, d=n.d_up, top=n.is_top):
                return layer_error(p1, p2, self.rho[a], d, top)

            g = _bs_node(Y[self.slices[a]].copy(), t_a, t_b, self.dt_bs[a], acc_leaf, err)
            try:
                pending[a] = next(g)
                gens[a] = g
            except StopIteration as stop:
                Y[self.slices[a]], self.dt_bs[a] = stop.value
        base = Y.copy()
        while pending:
            full = base.copy()
            for a, phi in pending.items():
                full[self.slices[a]] = phi
            d = self._derivatives(full)
            nxt = {}
            for a in pending:
                try:
                    nxt[a] = gens[a].send(d[self.slices[a]].copy())
                except StopIteration as stop:
                    Y[self.slices[a]], self.dt_bs[a] = stop.value
            pending = nxt

    def error(self, psi, chi):
        """CMFIntegrator::Error: the nodes' errors added in quadrature."""
        e2 = 0.0
        for n in self.tree.nodes:
            sl = self.slices[n.address]
            e2 += layer_error(psi[sl], chi[sl], self.rho[n.address], n.d_up, n.is_top) ** 2
        return math.sqrt(e2)

    def orthogonal(self, psi):
        """orthogonal(): bottom-up, S^(1/2) of each non-top node into its
        parent (matrixTensor), then Gram-Schmidt of the node."""
        for n in self.tree.nodes:
            if n.is_top:
                continue
            sl = self.slices[n.address]
            d = n.d_up
            Phi = psi[sl].reshape((-1, d), order="F").copy()
            w, U = np.linalg.eigh(Phi.conj().T @ Phi)
            SW = ((U * np.sqrt(np.maximum(w, 0.0))) @ U.conj().T).T
            p = self.tree.nodes[n.parent]
            psl = self.slices[p.address]
            B = psi[psl].reshape(list(p.shape), order="F")
            k = n.child_idx
            B = np.moveaxis(np.tensordot(SW, B, axes=([1], [k])), 0, k)
            psi[psl] = B.reshape(-1, order="F")
            _gram_schmidt(Phi)
            psi[sl] = Phi.reshape(-1, order="F")

    # -- Integrate ----------------------------------------------------------------
    def integrate(self, psi, t0: float, t_end: float, dt: float, out: float | None = None,
                  acc_root: float = 1e-5, acc_leaf: float = 1e-6):
        """CMFIntegrator::Integrate from t0 to t_end (initial step dt, output
        times every `out`, default t_end - t0): CMF steps of dt/4, dt/2, dt/4
        with matrices at t, t + dt/2 and t + dt, the error against one step
        of dt, step-size control (0.8 (acc/err)^(1/3), growth at most 2.25),
        orthogonal() after accepted steps.  Returns (psi, dt): the
        wavefunction at t_end (also left on the device) and the next step."""
        tree = self.tree
        out = (t_end - t0) if out is None else out
        flat = psi if isinstance(psi, np.ndarray) else psi.flat()
        psi = np.array(flat, dtype=np.complex128, copy=True)
        self.dt_bs = {n.address: dt / 2.0 for n in tree.nodes}
        time = t0
        t_next = time + out
        self.build(psi)
        calc_mat = False
        tc = self.tconst
        while time + 1e-6 < t_end:
            dtmax = min(t_end - time, t_next - time)
            if dt > dtmax:
                dt = dtmax
            elif 2 * dt > dtmax:
                dt = min(dt, dtmax * 0.6)
            psi0 = psi.copy()
            if calc_mat:
                self.build(psi)
                calc_mat = False
            ts = dt * tc
            self.cmf_step(psi, time, time + ts, acc_leaf)
            psi2 = psi.copy()
            self.cmf_step(psi2, time + ts, time + 2 * ts, acc_leaf)
            self.build(psi2)
            self.cmf_step(psi, time + dt * tc, time + dt * (1 - tc), acc_leaf)
            psi2 = psi0.copy()
            self.cmf_step(psi2, time, time + dt, acc_leaf)
            self.build(psi2)
            self.cmf_step(psi, time + dt * (1 - tc), time + dt, acc_leaf)
            err = self.error(psi, psi2) * 0.25
            if err > acc_root:
                psi = psi0
                calc_mat = True
                dt *= (acc_root / err) ** (1.0 / 3.0) * 0.8
                self.stats["refused"] += 1
            else:
                time += dt
                self.orthogonal(psi)
                if time + 1e-10 >= t_next:
                    t_next = time + out
                fac = self.max_increase if err == 0 else min((acc_root / err) ** (1.0 / 3.0), self.max_increase)
                dt = dt * fac
                self.stats["accepted"] += 1
        self.h.upload(psi)
        return psi, dt
