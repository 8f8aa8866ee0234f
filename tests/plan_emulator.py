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

B_PSI, B_HPHI, B_DPSI, B_MATS, B_OPS, B_SCR, B_PARAM, B_PSI64, B_DPSI64, B_GRAD, B_GRAD64, B_KEEP, B_HPW, B_KRY, B_CDVR = range(15)
(ST_MP, ST_HP, ST_ACC, ST_LIN, ST_EIG, ST_PROJ, ST_CVT, ST_GRAD, ST_MM,
 ST_TC, ST_GS, ST_EIGF, ST_WSD, ST_VPOT, ST_DVL, ST_EW) = range(16)


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
        L.qtp_build_cdvr.restype = ctypes.c_void_p
        L.qtp_build_cdvr.argtypes = L.qtp_build.argtypes + [
            ctypes.c_int, _i32, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, _i32, _i32, _i32, ctypes.c_int]
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
    def __init__(self, tree, sop, flavour=0, budget=1 << 28, prec=0, cdvr=None):
        """cdvr: optional (leaf_x dict mode -> grid, PolyPotential, aligned) of a
        Hamiltonian with a CDVR potential."""
        L = lib()
        order, dims, parent, child_idx, leaf_mode = tree.descriptor()
        kind, odim, ooff, odata = sop.ops.descriptor()
        coeff, ptr, modes, opids = sop.descriptor()
        self.ops = repack_ops(kind, odim, ooff, odata)
        odata = np.ascontiguousarray(odata)
        coeff = np.ascontiguousarray(coeff)
        err = ctypes.create_string_buffer(512)
        args = (tree.n_nodes, order, dims, parent, child_idx, leaf_mode, len(kind), kind,
                odim, ooff, odata.ctypes.data, len(sop), coeff.ctypes.data, ptr, modes,
                opids, flavour, prec, budget, err, 512)
        self.potential = None
        if cdvr is None:
            h = L.qtp_build(*args)
        else:
            leaf_x, pot, aligned = cdvr
            self.potential = pot
            f = len(leaf_x)
            ldim = np.array([len(leaf_x[m]) for m in range(f)], dtype=np.int32)
            lx = np.ascontiguousarray(np.concatenate([np.asarray(leaf_x[m], float) for m in range(f)]))
            pc, pp, pm, pw = pot.descriptor()
            pc = np.ascontiguousarray(pc)
            h = L.qtp_build_cdvr(*args, f, ldim, lx.ctypes.data, len(pc), pc.ctypes.data, pp, pm, pw,
                                 1 if aligned else 0)
        if not h:
            raise ValueError(err.value.decode())
        self.h = h
        self.tree, self.sop = tree, sop
        self.tensor = bool(flavour & 0x8000)  # mode products with the tensor-core digit arithmetic
        self.tables = {}
        widths = {0: 5, 1: 11, 2: 9, 3: 9, 4: 4, 5: 5, 6: 2, 7: 7, 8: 13, 10: 2, 13: 4, 18: 6, 19: 14,
                  20: 6, 22: 6, 23: 4, 24: 27, 25: 8, 26: 12, 27: 11, 28: 2, 29: 11, 33: 3, 34: 10,
                  35: 8, 36: 2, 38: 14, 39: 5, 40: 2, 41: 4, 42: 2, 43: 2, 44: 5, 45: 3, 46: 4, 47: 3, 49: 3, 50: 2, 51: 2,
                  52: 16, 53: 4, 54: 2, 55: 4, 57: 4, 58: 2, 59: 5}
        for what in list(range(14)) + [18, 19, 20, 21, 22, 23] + list(range(24, 30)) + list(range(33, 61)):
            n = int(L.qtp_size(h, what))
            a = np.zeros(max(n, 1), np.int64)
            if n:
                L.qtp_get(h, what, a.ctypes.data)
            a = a[:n]
            if what in widths:
                a = a.reshape(-1, widths[what])
            self.tables[what] = a
        for what in (15, 16, 17, 30, 31, 32):
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
        ci = self.tables[37]
        self.cdvr = bool(ci[0]) if len(ci) else False
        self.cdvr_size = int(ci[1]) if len(ci) else 0
        self.tc_alpha = self.tables[30].reshape(-1, 2) @ np.array([1, 1j]) if len(self.tables[30]) else np.zeros(0)

    # -- interpreter -------------------------------------------------------
    def run(self, psi_flat, phase=1.0, eps=1e-10, frozen_after=False):
        """Run the sweep (stages [0, main_end)).  ``frozen_after``: then run
        the frozen-matrix derivative stages on the same Psi as well."""
        self.init(psi_flat, phase)
        T = self.tables
        stages = list(range(self.main_end))
        if frozen_after:
            stages += list(range(self.main_end, len(T[0])))
        self.exec(stages, eps)
        return self.bufs

    def init(self, psi_flat, phase=1.0):
        """Fresh buffers with Psi loaded (identities set, matrices zero)."""
        psi0 = np.asarray(psi_flat, np.complex128).copy()
        bufs = [psi0,
                np.zeros(self.psi_arena, np.complex128),
                np.zeros(self.psi_arena, np.complex128),
                np.zeros(max(self.mats_size, 16), np.complex128),
                self.ops.copy(),
                np.zeros(max(self.scratch_size, 16), np.complex128),
                np.zeros(16, np.complex128), None, None,
                np.zeros(self.psi_arena, np.complex128), None,
                np.zeros(max(self.keep_size, 16), np.complex128), np.zeros(16, np.complex128),
                np.zeros(max(int(self.tables[21][2]) if len(self.tables[21]) else 16, 16), np.complex128)]
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
        cd = np.zeros(max(self.cdvr_size, 16), np.complex128)
        vals = self.tables[32].reshape(-1, 2) @ np.array([1, 1j]) if len(self.tables[32]) else []
        pos = 0
        for off, cnt in self.tables[36]:
            cd[off:off + cnt] = vals[pos:pos + cnt]
            pos += cnt
        bufs.append(cd)
        bufs[B_PARAM][0] = -1j * complex(phase)
        for off, d in self.tables[10]:
            bufs[B_MATS][off:off + d * d] = np.eye(d).ravel(order="F")
        self.bufs = bufs

    def exec(self, stage_ids, eps=1e-10):
        """Execute the given stages on the current buffers."""
        bufs = self.bufs

        def view(buf, off, n):
            return bufs[buf][off:off + n]

        T = self.tables
        for si in stage_ids:
            kind, t0, nt, _, _ = T[0][si]
            for t in range(t0, t0 + nt):
                if kind == ST_MP:
                    ib, io, ob, oo, hb, ho, bef, ain, aout, aft, diag = T[1][t]
                    x = view(ib, io, bef * ain * aft).reshape((bef, ain, aft), order="F")
                    if diag:
                        h = view(hb, ho, ain)
                        y = x * h[None, :, None]
                    else:
                        h = view(hb, ho, aout * ain).reshape((aout, ain), order="F")
                        if self.tensor and 32 <= ain <= 64 and 32 <= aout <= 64:
                            y = oz_mode_product(h, x)
                        else:
                            y = np.einsum("ja,bac->bjc", h, x)
                    view(ob, oo, bef * aout * aft)[:] = (self.mp_alpha[t] * y).ravel(order="F")
                elif kind == ST_HP:
                    ab, ao, bb, bo, sb, so, bef, a, aft = T[2][t]
                    A = view(ab, ao, bef * a * aft).reshape((bef, a, aft), order="F")
                    B = view(bb, bo, bef * a * aft).reshape((bef, a, aft), order="F")
                    if self.tensor and self.prec == 1 and hp_tc_eligible(bef, a, aft):
                        S = oz_hole_product(A, B)
                    else:
                        S = np.einsum("bic,bjc->ij", A.conj(), B)
                    view(sb, so, a * a)[:] = S.ravel(order="F")
                elif kind == ST_ACC:
                    ob, oo, ap, aoff, rows, d, first, count, add = T[3][t]
                    alpha = bufs[B_MATS][aoff] if ap == 2 else (bufs[B_PARAM][0] if ap else 1.0)
                    tc = self.tensor and self.prec == 1 and acc_tc_eligible(rows, d)
                    acc = np.zeros((rows, d), np.complex128)
                    for s in range(first, first + count):
                        hb, ho, xb, xo = T[4][s]
                        X = view(xb, xo, rows * d).reshape((rows, d), order="F")
                        H = np.eye(d) if hb < 0 else view(hb, ho, d * d).reshape((d, d), order="F")
                        if tc:  # alpha H_t in the digit arithmetic, term by term
                            acc += oz_mode_product(alpha * H, X[:, :, None])[:, :, 0]
                        elif hb < 0:
                            acc += X
                        else:
                            acc += X @ H.T
                    out = view(ob, oo, rows * d)
                    v = (acc if tc else alpha * acc).ravel(order="F")
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
                elif kind == ST_MM:
                    ob, oo, d, first, count, trans = T[22][t]
                    acc = np.zeros((d, d), np.complex128)
                    for s_ in range(first, first + count):
                        ab, ao, bb, bo = T[23][s_]
                        A = view(ab, ao, d * d).reshape((d, d), order="F")
                        B = view(bb, bo, d * d).reshape((d, d), order="F")
                        acc += A @ (B.T if trans else B)
                    view(ob, oo, d * d)[:] = acc.ravel(order="F")
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
                elif kind >= ST_TC:
                    self._cdvr_task(kind, t, view, eps)
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

    # -- CDVR tasks --------------------------------------------------------
    def _cdvr_task(self, kind, t, view, eps):
        T = self.tables
        bufs = self.bufs
        if kind == ST_TC:
            r = T[24][t]
            ab, ao, bb, bo, cb, co = r[:6]
            M0, M1, N0, N1, K0, K1, cjA, cjB, add = r[6:15]
            am0, am1, ak0, ak1, bk0, bk1, bn0, bn1, cm0, cm1, cn0, cn1 = r[15:27]

            def ix(e0, s0, e1, s1):
                return (np.arange(e0)[:, None] * s0 + np.arange(e1)[None, :] * s1).ravel(order="F")
            mA, kA = ix(M0, am0, M1, am1), ix(K0, ak0, K1, ak1)
            kB, nB = ix(K0, bk0, K1, bk1), ix(N0, bn0, N1, bn1)
            mC, nC = ix(M0, cm0, M1, cm1), ix(N0, cn0, N1, cn1)
            A = bufs[ab][ao + mA[:, None] + kA[None, :]]
            B = bufs[bb][bo + kB[:, None] + nB[None, :]]
            if cjA:
                A = A.conj()
            if cjB:
                B = B.conj()
            res = self.tc_alpha[t] * (A @ B)
            idx = co + mC[:, None] + nC[None, :]
            if add:
                bufs[cb][idx] += res
            else:
                bufs[cb][idx] = res
        elif kind == ST_GS:
            from qutree_gb300.model import gram_schmidt
            ib, io, nb, no, ob, oo, rows, cols = T[25][t]
            a = (view(ib, io, rows * cols) + view(nb, no, rows * cols)).reshape((rows, cols), order="F")
            view(ob, oo, rows * cols)[:] = gram_schmidt(a).ravel(order="F")
        elif kind == ST_EIGF:
            r = T[26][t]
            d, fn = r[10], r[11]
            e = T[31][t]
            A = view(r[0], r[1], d * d).reshape((d, d), order="F")
            A = 0.5 * (A + A.conj().T)
            w, U = np.linalg.eigh(A)
            if fn == 4:
                view(r[2], r[3], d * d)[:] = U.conj().T.ravel(order="F")
                view(r[8], r[9], d)[:] = w
            else:
                g = np.sqrt(np.maximum(w, 0.0))
                f = {0: lambda: 1.0 / (w + e * np.exp(-w / e)), 1: lambda: g,
                     2: lambda: 1.0 / (g + e * np.exp(-g / e)), 3: lambda: g + e * np.exp(-g / e)}[fn]()
                view(r[2], r[3], d * d)[:] = ((U * f) @ U.conj().T).ravel(order="F")
        elif kind == ST_WSD:
            import cdvr as ocdvr
            r = T[27][t]
            d, n, first = r[8], r[9], r[10]
            W = view(r[0], r[1], d * d).reshape((d, d), order="F")
            xs = []
            for q in range(first, first + n):
                xb, xo = T[28][q]
                xs.append(view(xb, xo, d * d).reshape((d, d), order="F"))
            Tr, grids, _ = ocdvr.layer_grid_multi(xs, W)
            view(r[2], r[3], d * d)[:] = Tr.ravel(order="F")
            view(r[4], r[5], n * d)[:] = np.concatenate(grids)
        elif kind == ST_VPOT:
            r = T[29][t]
            ob, oo, n, order, first = r[:5]
            dims = tuple(int(x) for x in r[5:5 + order])
            f = self.potential.f
            X = np.zeros(dims + (f,))
            for g in range(f):
                gb, go, index = T[33][first + g]
                vals = view(gb, go, dims[index]).real
                sh = [1] * order
                sh[index] = dims[index]
                X[..., g] = np.broadcast_to(vals.reshape(sh), dims)
            view(ob, oo, n)[:] = self.potential(X).ravel(order="F")
        elif kind == ST_DVL:
            cb, co, vb, vo, eb, eo, db, do, bef, d = T[34][t]
            cu = view(cb, co, bef * d).reshape((bef, d), order="F")
            vn = view(vb, vo, bef * d).reshape((bef, d), order="F")
            ve = view(eb, eo, d * d).reshape((d, d), order="F")
            Tl = np.einsum("bl,bi,bm->lim", cu.conj(), vn, cu)
            dv = np.zeros((d, d, d, d), np.complex128)
            for i0 in range(d):
                dv[:, i0, :, i0] = Tl[:, i0, :]
            for l0 in range(d):
                for l1 in range(d):
                    dv[l0, l1, l0, l1] -= ve[l0, l1]
            view(db, do, d ** 4)[:] = dv.ravel(order="F")
        elif kind == ST_EW:
            vb, vo, ib, io, ob, oo, n, add = T[35][t]
            res = view(vb, vo, n) * view(ib, io, n)
            out = view(ob, oo, n)
            out[:] = out + res if add else res

    def cdvr_arena(self):
        return self.bufs[B_CDVR].copy()

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


# --------------------------------------------------------------------------
# SCF sweep on the emulated plan (the host logic qt_scf runs around the GPU
# stages): Lanczos on the effective Hamiltonian of each node, Cholesky-QR
# (twice) toward the next node, R into the next node, buildUp / buildDown.
# --------------------------------------------------------------------------
OZ_DIGITS = 7


def _oz_split(r, sigma):
    """Error-free split: (x, r - x) with x = fl(fl(r + sigma) - sigma), r
    rounded to the nearest multiple of ulp(sigma) (float32, as the device)."""
    x = ((r + sigma).astype(np.float32) - sigma).astype(np.float32)
    return x, (r - x).astype(np.float32)


def _oz_sigma_digits(hi, lo, eb):
    """Digits of the double-float values hi + lo (float32 arrays) of rows
    whose largest biased exponent of hi parts is eb (broadcast): the row is
    scaled by 2^(126 - eb) and cut by the splits of sigma_s = 1.5 * 2^(16 - 7s),
    the low part joining from s = 3, as qt_umma.cu.  Returns the integers q_s
    (float64 arrays, digit first) with hi + lo ~ 2^E sum_s q_s 2^(-7(s+1))."""
    sc = np.exp2((126 - eb).astype(np.float64)).astype(np.float32)
    rh = (hi * sc).astype(np.float32)
    rl = (lo * sc).astype(np.float32)
    out = []
    for s in range(OZ_DIGITS):
        sigma = np.float32(1.5 * 2.0 ** (16 - 7 * s))
        x, rh = _oz_split(rh, sigma)
        if s >= 3:
            xl, rl = _oz_split(rl, sigma)
            x = (x + xl).astype(np.float32)
        out.append(x.astype(np.float64) * 2.0 ** (7 * (s + 1)))
    return out


def _oz_digits(v):
    """Digits of the rows of a complex matrix v (rows x k): the value split
    into double-float parts, seven signed digits per real part against the
    row's largest exponent.  Returns (E per row, re digits, im digits),
    digits as float64 arrays (digit, row, k)."""
    parts = []
    for comp in (v.real, v.imag):
        hi = comp.astype(np.float32)
        lo = (comp - hi.astype(np.float64)).astype(np.float32)
        parts.append((hi, lo))
    ex = np.maximum.reduce([(p[0].view(np.uint32) >> 23) & 0xFF for p in parts])
    eb = np.maximum(ex.max(axis=1, initial=0), 1).astype(np.int64)[:, None]
    out = []
    for hi, lo in parts:
        out.append(np.stack(_oz_sigma_digits(hi, lo, eb)))
    return (eb[:, 0] - 126).astype(np.float64), out[0], out[1]


def oz_mode_product(h, x):
    """out[b, j, c] = sum_a h(j, a) x[b, a, c] with the digit arithmetic of
    the tensor-core mode products with the fewest level accumulators (64
    output columns): the level sums L = 0, 1, 2 are exact (float64 holds them
    exactly), the levels 3..6 share one sum rounded to float32 as the
    device's fourth accumulator is, and everything is scaled by
    2^(E_r + F_j)."""
    bef, ain, aft = x.shape
    X = np.moveaxis(x, 1, -1).reshape(-1, ain)  # one row per (b, c)
    Ex, xr, xi = _oz_digits(X)
    Fh, hr, hi = _oz_digits(h)
    re = np.zeros((X.shape[0], h.shape[0]))
    im = np.zeros_like(re)
    r3 = np.zeros_like(re)
    i3 = np.zeros_like(re)
    for L in range(OZ_DIGITS):
        sr = np.zeros_like(re)
        si = np.zeros_like(re)
        for s in range(L + 1):
            u = L - s
            sr += xr[s] @ hr[u].T - xi[s] @ hi[u].T
            si += xr[s] @ hi[u].T + xi[s] @ hr[u].T
        if L < 3:
            re += sr * 2.0 ** (-7 * (L + 2))
            im += si * 2.0 ** (-7 * (L + 2))
        else:
            r3 += sr * 2.0 ** (-7 * (L - 3))
            i3 += si * 2.0 ** (-7 * (L - 3))
    re += r3.astype(np.float32).astype(np.float64) * 2.0 ** (-35)
    im += i3.astype(np.float32).astype(np.float64) * 2.0 ** (-35)
    scale = np.exp2(Ex[:, None] + Fh[None, :])
    y = (re + 1j * im) * scale
    return np.moveaxis(y.reshape(bef, aft, -1), -1, 1)


HP_CHUNK = 64


def acc_tc_eligible(rows, d):
    """The accumulations the planner puts on the tensor cores (qt_internal.h)."""
    return 32 <= d <= 64 and rows >= 64


def hp_tc_eligible(before, a, after):
    """The hole products the planner puts on the tensor cores (qt_internal.h)."""
    return 32 <= a <= 64 and before * after >= 2 * HP_CHUNK


def hp_tc_kc(a):
    """Reduction length of a tensor-core hole-product chunk (qt_internal.h)."""
    return 2 * HP_CHUNK if (a + 7) // 8 * 8 > 32 else HP_CHUNK


def oz_hole_product(A, B):
    """S(i, j) = sum_k conj(A[b, i, c]) B[b, j, c], k = b + before c, with
    the digit arithmetic of the tensor-core hole products: the reduction in
    chunks of hp_tc_kc(a) k, every chunk with its own exponents per row of B (per j)
    and of A (per i); complex products as Re = Br Ar + Bi Ai and
    Im = Bi Ar - Br Ai; levels 0..2 exact, levels 3..6 in one float32 sum
    (the fewest accumulators), each chunk scaled by 2^(E_j + F_i) and the
    chunks summed."""
    bef, a, aft = A.shape
    XA = np.transpose(A, (2, 0, 1)).reshape(-1, a)  # row k = c * before + b
    XB = np.transpose(B, (2, 0, 1)).reshape(-1, B.shape[1])
    K = XA.shape[0]
    S = np.zeros((B.shape[1], a), np.complex128)  # rows j, columns i
    kc = hp_tc_kc(a)
    for k0 in range(0, K, kc):
        Eb, br, bi = _oz_digits(XB[k0:k0 + kc].T)
        Fa, ar, ai = _oz_digits(XA[k0:k0 + kc].T)
        re = np.zeros((br.shape[1], ar.shape[1]))
        im = np.zeros_like(re)
        r3 = np.zeros_like(re)
        i3 = np.zeros_like(re)
        for L in range(OZ_DIGITS):
            sr = np.zeros_like(re)
            si = np.zeros_like(re)
            for s in range(L + 1):
                u = L - s
                sr += br[s] @ ar[u].T + bi[s] @ ai[u].T
                si += bi[s] @ ar[u].T - br[s] @ ai[u].T
            if L < 3:
                re += sr * 2.0 ** (-7 * (L + 2))
                im += si * 2.0 ** (-7 * (L + 2))
            else:
                r3 += sr * 2.0 ** (-7 * (L - 3))
                i3 += si * 2.0 ** (-7 * (L - 3))
        re += r3.astype(np.float32).astype(np.float64) * 2.0 ** (-35)
        im += i3.astype(np.float32).astype(np.float64) * 2.0 ** (-35)
        S += (re + 1j * im) * np.exp2(Eb[:, None] + Fa[None, :])
    return S.T


def _mp(h, x, k):
    return np.moveaxis(np.tensordot(h, x, axes=([1], [k])), 0, k)


def _hole(a, b, k):
    am = np.moveaxis(a, k, -1).reshape(-1, a.shape[k])
    bm = np.moveaxis(b, k, -1).reshape(-1, b.shape[k])
    return am.conj().T @ bm


def chol_qr(x, mode, cond_limit=1e-6):
    """Q with orthonormal columns along `mode`: Cholesky-QR applied twice,
    Householder QR when the Gram matrix is (near) singular -- the rule qt_scf
    follows."""
    q = x
    for _ in range(2):
        s = _hole(q, q, mode)
        try:
            L = np.linalg.cholesky(s)
        except np.linalg.LinAlgError:
            L = None
        dg = np.abs(np.diag(L)) if L is not None else None
        if L is None or dg.min() <= cond_limit * dg.max():
            xm = np.moveaxis(x, mode, -1)
            shp = xm.shape
            qh, _ = np.linalg.qr(xm.reshape(-1, shp[-1]))
            return np.moveaxis(qh.reshape(shp), -1, mode)
        r = L.conj().T  # s = r^dag r, r upper triangular
        q = _mp(np.linalg.inv(r).T, q, mode)
    return q


def scf_emulated(pv, tree, psi_flat, n_iter=1, n_krylov=5, n_itp=0, beta=1.0):
    from scf import sweep_order  # oracle module: the reference's sweep order
    pv.init(psi_flat)
    if pv.prec == 1:  # the conversion qt_scf runs first (a copy here)
        pv.bufs[B_PSI][:] = pv.bufs[B_PSI64]
    arena = pv.bufs[B_PSI]
    offs = tree.offsets()
    seg = pv.tables[20]
    kin, kout = int(pv.tables[21][0]), int(pv.tables[21][1])

    def get(a):
        n = tree.nodes[a]
        return arena[offs[a]:offs[a + 1]].reshape(n.shape, order="F").copy()

    def put(a, x):
        arena[offs[a]:offs[a + 1]] = x.ravel(order="F")

    def H(x, a):
        K = pv.bufs[B_KRY]
        n = x.size
        K[kin:kin + n] = x.ravel(order="F")
        pv.exec(range(seg[a][4], seg[a][5]))
        return K[kout:kout + n].reshape(x.shape, order="F").copy()

    for n in tree.nodes:
        if n.parent >= 0:
            pv.exec(range(seg[n.address][0], seg[n.address][1]))
    order = sweep_order(tree)
    energies = []
    for it in range(n_iter):
        for i, a in enumerate(order):
            n = tree.nodes[a]
            size = min(n_krylov, int(np.prod(n.shape)))
            x = get(a)
            x = x / np.sqrt(np.vdot(x, x).real)
            space = [x]
            alpha, betas = [], []
            hx = H(x, a)
            alpha.append(np.vdot(x, hx).real)
            w = hx - alpha[-1] * x
            for l in range(1, size):
                nrm = np.sqrt(np.vdot(w, w).real)
                betas.append(nrm)
                v = w / nrm
                space.append(v)
                hx = H(v, a)
                alpha.append(np.vdot(v, hx).real)
                w = hx - alpha[-1] * space[l] - betas[-1] * space[l - 1]
            T = np.diag(alpha)
            for l in range(size - 1):
                T[l + 1, l] = T[l, l + 1] = betas[l]
            E, U = np.linalg.eigh(T)
            energies.append(E[0])
            if it < n_itp:
                c = np.zeros(size, complex)
                for l in range(size):
                    c[l] += U[l, 0] * U[0, 0]
                    for k in range(size):
                        c[l] += U[l, k] * np.exp(-beta * (E[k] - E[0])) * U[0, k]
                y = sum(c[l] * space[l] for l in range(size))
                y = y / np.sqrt(np.vdot(y, y).real)
            else:
                y = sum(U[l, 0] * space[l] for l in range(size))
            nxt = order[i + 1] if i + 1 < len(order) else None
            out_idx = (n.children.index(nxt) if nxt is not None and nxt in n.children
                       else len(n.shape) - 1)
            q = chol_qr(y, out_idx)
            put(a, q)
            if nxt is None:
                break
            r = _hole(q, y, out_idx)
            m = tree.nodes[nxt]
            in_idx = m.children.index(a) if a in m.children else len(m.shape) - 1
            put(nxt, _mp(r, get(nxt), in_idx))
            up = n.parent == nxt
            if up:
                pv.exec(range(seg[a][0], seg[a][1]))
            else:
                pv.exec(range(seg[nxt][2], seg[nxt][3]))
    psi_out = arena[:offs[-1]].copy()
    return np.array(energies), psi_out
