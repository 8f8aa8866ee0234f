"""numpy interpreter of the sweep plan (test infrastructure).

Loads the host-only planner library (libqtplan.so, built from the same
qt_plan.cpp the GPU library uses), builds the plan of a (tree, SOP) pair and
executes its stages one by one with numpy: the mode products, hole products,
accumulations, mean-field sums, density inverses and projector pieces the GPU
kernels perform.  Comparing the result with the oracle checks the planner's
schedule (ordering, buffer reuse, slot sharing, term grouping) without a GPU;
the GPU tests then check the kernels against the same oracle.
"""
from __future__ import annotations

import ctypes

import numpy as np

from qutree_gb300 import build as qbuild

_P = np.ctypeslib.ndpointer
_i32 = _P(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = _P(dtype=np.int64, flags="C_CONTIGUOUS")
_lib = None

B_PSI, B_HPHI, B_DPSI, B_MATS, B_OPS, B_SCR, B_PARAM, B_PSI64, B_DPSI64, B_GRAD, B_GRAD64, B_KEEP = range(12)
ST_MP, ST_HP, ST_ACC, ST_LIN, ST_EIG, ST_PROJ, ST_CVT, ST_GRAD = range(8)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(qbuild.build_plan_lib())
        L.qtp_build.restype = ctypes.c_void_p
        L.qtp_build.argtypes = [ctypes.c_int, _i32, _i32, _i32, _i32, _i32, ctypes.c_int, _i32, _i32,
                                _i64, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, _i32, _i32,
                                _i32, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_char_p,
                                ctypes.c_int]
        L.qtp_free.argtypes = [ctypes.c_void_p]
        L.qtp_size.restype = ctypes.c_int64
        L.qtp_size.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.qtp_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.qtp_stage_name.restype = ctypes.c_char_p
        L.qtp_stage_name.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib = L
    return _lib


def repack_ops(kind, dim, off, data):
    """The device operator table layout: each operator 16-element aligned."""
    cur = 0
    offs, chunks = [], []
    for k, d, o in zip(kind, dim, off):
        n = d * d if k == 0 else d
        offs.append(cur)
        chunks.append((cur, data[o:o + n]))
        cur = (cur + n + 15) // 16 * 16
    out = np.zeros(max(cur, 16), np.complex128)
    for c, v in chunks:
        out[c:c + v.size] = v
    return out


class PlanView:
    def __init__(self, tree, sop, flavour=0, budget=1 << 28, prec=0):
        L = lib()
        order, dims, parent, child_idx, leaf_mode = tree.descriptor()
        kind, odim, ooff, odata = sop.ops.descriptor()
        coeff, ptr, modes, opids = sop.descriptor()
        self.ops = repack_ops(kind, odim, ooff, odata)
        odata = np.ascontiguousarray(odata)
        coeff = np.ascontiguousarray(coeff)
        err = ctypes.create_string_buffer(512)
        h = L.qtp_build(tree.n_nodes, order, dims, parent, child_idx, leaf_mode, len(kind), kind,
                        odim, ooff, odata.ctypes.data, len(sop), coeff.ctypes.data, ptr, modes,
                        opids, flavour, prec, budget, err, 512)
        if not h:
            raise ValueError(err.value.decode())
        self.h = h
        self.tree, self.sop = tree, sop
        self.tables = {}
        widths = {0: 5, 1: 11, 2: 9, 3: 9, 4: 4, 5: 5, 6: 2, 7: 7, 8: 13, 10: 2, 13: 4, 18: 6, 19: 14}
        for what in list(range(14)) + [18, 19]:
            n = int(L.qtp_size(h, what))
            a = np.zeros(max(n, 1), np.int64)
            if n:
                L.qtp_get(h, what, a.ctypes.data)
            a = a[:n]
            if what in widths:
                a = a.reshape(-1, widths[what])
            self.tables[what] = a
        for what in (15, 16, 17):
            n = int(L.qtp_size(h, what))
            a = np.zeros(max(n, 1))
            if n:
                L.qtp_get(h, what, a.ctypes.data)
            self.tables[what] = a[:n]
        self.mp_alpha = self.tables[15].reshape(-1, 2) @ np.array([1, 1j]) if len(self.tables[15]) else np.zeros(0)
        self.lin_c = self.tables[16].reshape(-1, 2) @ np.array([1, 1j]) if len(self.tables[16]) else np.zeros(0)
        self.stage_names = [L.qtp_stage_name(h, i).decode() for i in range(len(self.tables[0]))]
        L.qtp_free(h)
        self.pairs = self.tables[13]  # rows (term, node, hslot, cslot), terms ascending
        s = self.tables[9]
        self.psi_arena, self.mats_size, self.scratch_size, self.ops_size = map(int, s[:4])
        self.energy_off, self.stop_off = int(s[4]), int(s[5])
        self.prec = int(s[6])
        self.keep_size, self.main_end = int(s[7]), int(s[8])
        st = self.tables[17]
        self.stats = dict(ref_flops=st[0], exec_flops=st[1], launches=int(st[2]),
                          rep_chains=int(st[3]), mf_chains=int(st[4]), app_chains=int(st[5]))

    # -- interpreter -------------------------------------------------------
    def run(self, psi_flat, phase=1.0, eps=1e-10, frozen_after=False):
        """Run the sweep (stages [0, main_end)).  ``frozen_after``: then run
        the frozen-matrix derivative stages on the same Psi as well."""
        psi0 = np.asarray(psi_flat, np.complex128).copy()
        bufs = [psi0,
                np.zeros(self.psi_arena, np.complex128),
                np.zeros(self.psi_arena, np.complex128),
                np.zeros(max(self.mats_size, 16), np.complex128),
                self.ops.copy(),
                np.zeros(max(self.scratch_size, 16), np.complex128),
                np.zeros(16, np.complex128), None, None,
                np.zeros(self.psi_arena, np.complex128), None,
                np.zeros(max(self.keep_size, 16), np.complex128)]
        if self.prec == 1:
            # separate caller-facing complex128 arrays; conversions are copies here
            bufs[B_PSI] = np.zeros_like(psi0)
            bufs[B_PSI64] = psi0
            bufs[B_DPSI64] = np.zeros_like(psi0)
            bufs[B_GRAD64] = np.zeros_like(psi0)
        else:
            bufs[B_PSI64] = bufs[B_PSI]
            bufs[B_DPSI64] = bufs[B_DPSI]
            bufs[B_GRAD64] = bufs[B_GRAD]
        bufs[B_PARAM][0] = -1j * complex(phase)
        for off, d in self.tables[10]:
            bufs[B_MATS][off:off + d * d] = np.eye(d).ravel(order="F")

        def view(buf, off, n):
            return bufs[buf][off:off + n]

        T = self.tables
        stages = list(T[0][:self.main_end])
        if frozen_after:
            stages += list(T[0][self.main_end:]) if len(T[0]) > self.main_end else []
        for kind, t0, nt, _, _ in stages:
            for t in range(t0, t0 + nt):
                if kind == ST_MP:
                    ib, io, ob, oo, hb, ho, bef, ain, aout, aft, diag = T[1][t]
                    x = view(ib, io, bef * ain * aft).reshape((bef, ain, aft), order="F")
                    if diag:
                        h = view(hb, ho, ain)
                        y = x * h[None, :, None]
                    else:
                        h = view(hb, ho, aout * ain).reshape((aout, ain), order="F")
                        y = np.einsum("ja,bac->bjc", h, x)
                    view(ob, oo, bef * aout * aft)[:] = (self.mp_alpha[t] * y).ravel(order="F")
                elif kind == ST_HP:
                    ab, ao, bb, bo, sb, so, bef, a, aft = T[2][t]
                    A = view(ab, ao, bef * a * aft).reshape((bef, a, aft), order="F")
                    B = view(bb, bo, bef * a * aft).reshape((bef, a, aft), order="F")
                    S = np.einsum("bic,bjc->ij", A.conj(), B)
                    view(sb, so, a * a)[:] = S.ravel(order="F")
                elif kind == ST_ACC:
                    ob, oo, ap, aoff, rows, d, first, count, add = T[3][t]
                    acc = np.zeros((rows, d), np.complex128)
                    for s in range(first, first + count):
                        hb, ho, xb, xo = T[4][s]
                        X = view(xb, xo, rows * d).reshape((rows, d), order="F")
                        if hb < 0:
                            acc += X
                        else:
                            H = view(hb, ho, d * d).reshape((d, d), order="F")
                            acc += X @ H.T
                    alpha = bufs[B_MATS][aoff] if ap == 2 else (bufs[B_PARAM][0] if ap else 1.0)
                    out = view(ob, oo, rows * d)
                    v = (alpha * acc).ravel(order="F")
                    out[:] = out + v if add else v
                elif kind == ST_LIN:
                    ob, oo, d, first, count = T[5][t]
                    acc = np.zeros(d * d, np.complex128)
                    for s in range(first, first + count):
                        mb, mo = T[6][s]
                        acc += self.lin_c[s] * view(mb, mo, d * d)
                    view(ob, oo, d * d)[:] = acc
                elif kind == ST_EIG:
                    rb, ro, ib, io, ub, uo, d = T[7][t]
                    R = view(rb, ro, d * d).reshape((d, d), order="F")
                    R = 0.5 * (R + R.conj().T)
                    w, U = np.linalg.eigh(R)
                    f = 1.0 / (w + eps * np.exp(-w / eps))
                    view(ib, io, d * d)[:] = ((U * f) @ U.conj().T).ravel(order="F")
                elif kind == ST_CVT:
                    sb, so, db, do, n, _ = T[18][t]
                    view(db, do, n)[:] = view(sb, so, n)
                elif kind == ST_GRAD:
                    r = T[19][t]
                    d = r[12]
                    E = (view(r[6], r[7], 1)[0] / view(r[8], r[9], 1)[0]).real
                    eo = view(r[0], r[1], d * d) if r[0] >= 0 else np.zeros(d * d, complex)
                    view(r[4], r[5], d * d)[:] = eo - E * view(r[2], r[3], d * d)
                    if r[13]:
                        view(r[10], r[11], 1)[0] = 1.0 / view(r[8], r[9], 1)[0].real
                elif kind == ST_PROJ:
                    r = T[8][t]
                    d = r[12]
                    m = lambda k: view(r[2 * k], r[2 * k + 1], d * d).reshape((d, d), order="F")
                    S, D, Ri = m(0), m(1), m(2)
                    Sinv = np.linalg.inv(S)
                    Pm = Sinv @ D
                    M2 = -(Ri @ Pm.T)
                    view(r[6], r[7], d * d)[:] = Sinv.ravel(order="F")
                    view(r[8], r[9], d * d)[:] = Pm.ravel(order="F")
                    view(r[10], r[11], d * d)[:] = M2.ravel(order="F")
        self.bufs = bufs
        return bufs

    def dpsi(self):
        return self.bufs[B_DPSI64].copy()

    def gradient(self):
        return self.bufs[B_GRAD64].copy()

    def energy_parts(self):
        m = self.bufs[B_MATS]
        return m[self.energy_off], m[self.stop_off]

    def sparse(self, which):
        """hmat (which=0) or hcon (which=1) in the oracle's sparse layout."""
        out = []
        for l, a, hs, cs in self.pairs:
            dd = self.tree.nodes[a].d_up ** 2
            s2 = hs if which == 0 else cs
            out.append(self.bufs[B_MATS][s2:s2 + dd] if s2 >= 0 else np.zeros(dd, np.complex128))
        return np.concatenate(out)
