"""ctypes front end of the CPU FP64 oracle (qt_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py's CPU-baseline leg.  The product path never
imports this module.

The oracle restates QuTree's Derivative() sweep; see qt_oracle.cpp for the
reference file:line of every routine.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LOOPS, BLAS = 0, 1

_P = np.ctypeslib.ndpointer
_i32 = _P(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = _P(dtype=np.int64, flags="C_CONTIGUOUS")


def _dptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def build(fast: bool = True, quiet: bool = True) -> str:
    """Compile the oracle with g++ into oracle/_build/.  ``fast`` uses the
    reference's release flags (-O3 -ffast-math -fopenmp-simd,
    CMakeLists.txt:163-165); otherwise -O2 without fast-math."""
    os.makedirs(BUILD, exist_ok=True)
    name = "liboracle_fast.so" if fast else "liboracle.so"
    out = os.path.join(BUILD, name)
    src = os.path.join(HERE, "qt_oracle.cpp")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    flags = ["-O3", "-ffast-math", "-fopenmp-simd"] if fast else ["-O2"]
    cmd = ["g++", "-std=c++17", "-shared", "-fPIC", *flags, "-o", out + ".tmp", src]
    subprocess.check_call(cmd, stdout=subprocess.DEVNULL if quiet else None)
    os.replace(out + ".tmp", out)
    return out


_libs = {}


def lib(fast: bool = False):
    if fast in _libs:
        return _libs[fast]
    path = build(fast)
    L = ctypes.CDLL(path)
    L.orc_mode_product.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                   ctypes.c_int]
    L.orc_hole_product.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
    L.orc_herm_eig.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.orc_inverse.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.orc_sparse_size.restype = ctypes.c_int64
    L.orc_sparse_size.argtypes = [ctypes.c_int, _i32, _i32, _i32, _i32, _i32, ctypes.c_int, _i32, _i32]
    L.orc_derivative.restype = ctypes.c_int
    L.orc_derivative.argtypes = [
        ctypes.c_int, ctypes.c_int, _i32, _i32, _i32, _i32, _i32,
        ctypes.c_int, _i32, _i32, _i64, ctypes.c_void_p,
        ctypes.c_int, ctypes.c_void_p, _i32, _i32, _i32,
        ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p]
    L.orc_set_zgemm.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.orc_cmf.restype = ctypes.c_int
    L.orc_cmf.argtypes = [
        ctypes.c_int, ctypes.c_int, _i32, _i32, _i32, _i32, _i32,
        ctypes.c_int, _i32, _i32, _i64, ctypes.c_void_p,
        ctypes.c_int, ctypes.c_void_p, _i32, _i32, _i32,
        ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_int, ctypes.c_int]
    L.orc_scf.restype = ctypes.c_int
    L.orc_scf.argtypes = [
        ctypes.c_int, ctypes.c_int, _i32, _i32, _i32, _i32, _i32,
        ctypes.c_int, _i32, _i32, _i64, ctypes.c_void_p,
        ctypes.c_int, ctypes.c_void_p, _i32, _i32, _i32,
        ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
        ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    L.orc_frozen_new.restype = ctypes.c_void_p
    L.orc_frozen_new.argtypes = [
        ctypes.c_int, ctypes.c_int, _i32, _i32, _i32, _i32, _i32,
        ctypes.c_int, _i32, _i32, _i64, ctypes.c_void_p,
        ctypes.c_int, ctypes.c_void_p, _i32, _i32, _i32, ctypes.c_double]
    L.orc_frozen_build.restype = ctypes.c_int
    L.orc_frozen_build.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.orc_frozen_deriv.restype = ctypes.c_int
    L.orc_frozen_deriv.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_void_p]
    L.orc_frozen_deriv_node.restype = ctypes.c_int
    L.orc_frozen_deriv_node.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_void_p]
    L.orc_frozen_rho.restype = ctypes.c_int
    L.orc_frozen_rho.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.orc_frozen_free.restype = None
    L.orc_frozen_free.argtypes = [ctypes.c_void_p]
    _libs[fast] = L
    return L


def attach_openblas(fast: bool = True) -> str | None:
    """Point the oracle's BLAS back end at scipy's bundled OpenBLAS
    (``scipy_cblas_zgemm``), the BLAS the reference links.  Returns the
    library path, or None when none is found (naive zgemm is then used)."""
    try:
        import scipy
    except ImportError:
        return None
    cands = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__) + ".libs",
                                          "libscipy_openblas*.so")))
    for c in cands:
        try:
            ob = ctypes.CDLL(c)
        except OSError:
            continue
        for sym, ilp in (("scipy_cblas_zgemm", 0), ("scipy_cblas_zgemm64_", 1),
                         ("cblas_zgemm", 0)):
            try:
                fn = getattr(ob, sym)
            except AttributeError:
                continue
            lib(fast).orc_set_zgemm(ctypes.cast(fn, ctypes.c_void_p), ilp)
            _libs.setdefault("_keep", []).append(ob)
            return c
    return None


def set_blas_threads(n: int) -> bool:
    """Thread count of the attached OpenBLAS (all cores by default); False
    when no OpenBLAS is attached or it has no such control."""
    for ob in _libs.get("_keep", []):
        for sym in ("scipy_openblas_set_num_threads", "scipy_openblas_set_num_threads64_",
                    "openblas_set_num_threads"):
            fn = getattr(ob, sym, None)
            if fn is not None:
                fn(int(n))
                return True
    return False


def detach_blas(fast: bool = True):
    lib(fast).orc_set_zgemm(None, 0)


# --------------------------------------------------------------------------
# primitives
# --------------------------------------------------------------------------
def mode_product(h, B, before, activeB, activeC, after, C=None, add=False, backend=LOOPS,
                 fast=False):
    h = np.ascontiguousarray(h, dtype=np.complex128).ravel(order="K")
    B = np.ascontiguousarray(B, dtype=np.complex128)
    if C is None:
        C = np.zeros(before * activeC * after, dtype=np.complex128)
    lib(fast).orc_mode_product(backend, C.ctypes.data, h.ctypes.data, B.ctypes.data,
                               before, activeB, activeC, after, int(add))
    return C


def hole_product(A, B, before, activeA, activeB, after, backend=LOOPS, fast=False):
    A = np.ascontiguousarray(A, dtype=np.complex128)
    B = np.ascontiguousarray(B, dtype=np.complex128)
    S = np.zeros(activeA * activeB, dtype=np.complex128)
    lib(fast).orc_hole_product(backend, S.ctypes.data, A.ctypes.data, B.ctypes.data,
                               before, activeA, activeB, after)
    return S


def herm_eig(A):
    A = np.asfortranarray(A, dtype=np.complex128)
    n = A.shape[0]
    U = np.zeros((n, n), dtype=np.complex128, order="F")
    w = np.zeros(n)
    lib().orc_herm_eig(n, A.ctypes.data, U.ctypes.data, w.ctypes.data)
    return w, U


def inverse(A):
    A = np.asfortranarray(A, dtype=np.complex128)
    n = A.shape[0]
    X = np.zeros((n, n), dtype=np.complex128, order="F")
    lib().orc_inverse(n, A.ctypes.data, X.ctypes.data)
    return X


# --------------------------------------------------------------------------
# full sweep
# --------------------------------------------------------------------------
class SweepResult:
    def __init__(self, **kw):
        self.__dict__.update(kw)

    @property
    def energy(self) -> float:
        """E = Re(h00) / Re(S00) (CMFIntegrator's energy output)."""
        return self.h00.real / self.s00.real


def sparse_size(tree, sop) -> int:
    order, dims, parent, child_idx, leaf_mode = tree.descriptor()
    coeff, ptr, modes, opids = sop.descriptor()
    return int(lib().orc_sparse_size(tree.n_nodes, order, dims, parent, child_idx, leaf_mode,
                                     len(sop), ptr, modes))


def derivative(tree, sop, psi, eps=1e-10, phase=1.0, backend=LOOPS, fast=False,
               want_mats=True) -> SweepResult:
    """One Derivative() sweep of the oracle on flat complex128 ``psi``."""
    order, dims, parent, child_idx, leaf_mode = tree.descriptor()
    kind, odim, ooff, odata = sop.ops.descriptor()
    coeff, ptr, modes, opids = sop.descriptor()
    psi = np.ascontiguousarray(psi, dtype=np.complex128)
    assert psi.size == int(tree.offsets()[-1])
    dpsi = np.zeros_like(psi)
    nrho = sum(n.d_up * n.d_up for n in tree.nodes)
    rho = np.zeros(nrho, np.complex128) if want_mats else None
    rhoinv = np.zeros(nrho, np.complex128) if want_mats else None
    ns = sparse_size(tree, sop) if want_mats else 0
    hmat = np.zeros(ns, np.complex128) if want_mats else None
    hcon = np.zeros(ns, np.complex128) if want_mats else None
    energy = np.zeros(4)
    odata = np.ascontiguousarray(odata)
    coeff = np.ascontiguousarray(coeff)
    rc = lib(fast).orc_derivative(
        backend, tree.n_nodes, order, dims, parent, child_idx, leaf_mode,
        len(kind), kind, odim, ooff, odata.ctypes.data,
        len(sop), coeff.ctypes.data, ptr, modes, opids,
        psi.ctypes.data, eps, complex(phase).real, complex(phase).imag,
        dpsi.ctypes.data,
        rho.ctypes.data if rho is not None else None,
        rhoinv.ctypes.data if rhoinv is not None else None,
        hmat.ctypes.data if hmat is not None else None,
        hcon.ctypes.data if hcon is not None else None,
        energy.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle derivative failed: {rc}")
    return SweepResult(dpsi=dpsi, rho=rho, rhoinv=rhoinv, hmat=hmat, hcon=hcon,
                       h00=complex(energy[0], energy[1]), s00=complex(energy[2], energy[3]))


def cmf(tree, sop, psi, dt, n_steps, n_sub=1, phase=1.0, eps=1e-10, backend=LOOPS, fast=False):
    """Fixed-step constant-mean-field propagation (see qt_oracle.cpp orc_cmf);
    returns the propagated flat wavefunction."""
    order, dims, parent, child_idx, leaf_mode = tree.descriptor()
    kind, odim, ooff, odata = sop.ops.descriptor()
    coeff, ptr, modes, opids = sop.descriptor()
    y = np.array(psi, dtype=np.complex128, copy=True)
    odata = np.ascontiguousarray(odata)
    coeff = np.ascontiguousarray(coeff)
    rc = lib(fast).orc_cmf(backend, tree.n_nodes, order, dims, parent, child_idx, leaf_mode,
                           len(kind), kind, odim, ooff, odata.ctypes.data, len(sop),
                           coeff.ctypes.data, ptr, modes, opids, y.ctypes.data, eps,
                           complex(phase).real, complex(phase).imag, dt, n_steps, n_sub)
    if rc != 0:
        raise RuntimeError(f"oracle cmf failed: {rc}")
    return y


def scf(tree, sop, psi, n_iter=1, n_krylov=5, n_itp=0, beta=1.0, breakdown=None, backend=LOOPS,
        fast=False):
    """The SCF sweep in compiled code (orc_scf, the twin of oracle/scf.py):
    returns (lowest Ritz value of every Krylov solve, final flat psi)."""
    order, dims, parent, child_idx, leaf_mode = tree.descriptor()
    kind, odim, ooff, odata = sop.ops.descriptor()
    coeff, ptr, modes, opids = sop.descriptor()
    y = np.array(psi, dtype=np.complex128, copy=True)
    odata = np.ascontiguousarray(odata)
    coeff = np.ascontiguousarray(coeff)
    cap = n_iter * (2 * tree.n_nodes - 1)
    E = np.zeros(max(cap, 1))
    cnt = ctypes.c_int64(0)
    rc = lib(fast).orc_scf(backend, tree.n_nodes, order, dims, parent, child_idx, leaf_mode,
                           len(kind), kind, odim, ooff, odata.ctypes.data, len(sop),
                           coeff.ctypes.data, ptr, modes, opids, y.ctypes.data, n_iter, n_krylov, n_itp,
                           beta, -1.0 if breakdown is None else breakdown, E.ctypes.data, cap,
                           ctypes.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"oracle scf failed: {rc}")
    return E[:cnt.value].copy(), y


class Frozen:
    """Frozen-matrix session: build(psi) = HamiltonianRepresentation::build,
    deriv(psi) = LayerDerivative of every node with those matrices, rho() =
    the build's density matrices (per node d_up x d_up, column-major, in
    node order)."""

    def __init__(self, tree, sop, eps=1e-10, phase=1.0, backend=LOOPS, fast=False):
        self.tree, self.phase = tree, complex(phase)
        self._desc = tree.descriptor()
        kind, odim, ooff, odata = sop.ops.descriptor()
        coeff, ptr, modes, opids = sop.descriptor()
        self._keep = (kind, odim, ooff, np.ascontiguousarray(odata), np.ascontiguousarray(coeff), ptr,
                      modes, opids)
        k = self._keep
        self.n = int(tree.offsets()[-1])
        self.nrho = sum(n.d_up * n.d_up for n in tree.nodes)
        self.L = lib(fast)
        order, dims, parent, child_idx, leaf_mode = self._desc
        self.h = self.L.orc_frozen_new(backend, tree.n_nodes, order, dims, parent, child_idx, leaf_mode,
                                       len(k[0]), k[0], k[1], k[2], k[3].ctypes.data, len(sop),
                                       k[4].ctypes.data, k[5], k[6], k[7], eps)

    def build(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        self.L.orc_frozen_build(self.h, psi.ctypes.data)

    def deriv(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        out = np.zeros(self.n, np.complex128)
        self.L.orc_frozen_deriv(self.h, psi.ctypes.data, self.phase.real, self.phase.imag, out.ctypes.data)
        return out

    def deriv_node(self, n, phi):
        """LayerDerivative of node n at node tensor phi (other nodes untouched)."""
        phi = np.ascontiguousarray(phi, dtype=np.complex128)
        out = np.zeros(phi.size, np.complex128)
        if self.L.orc_frozen_deriv_node(self.h, n, phi.ctypes.data, self.phase.real, self.phase.imag,
                                        out.ctypes.data) != 0:
            raise ValueError("node index out of range")
        return out

    def rho(self):
        out = np.zeros(self.nrho, np.complex128)
        self.L.orc_frozen_rho(self.h, out.ctypes.data)
        return out

    def close(self):
        if self.h:
            self.L.orc_frozen_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sparse_offsets(tree, sop):
    """{(term, node): offset} of the sparse matrix tree layout."""
    out = {}
    acc = 0
    for l, t in enumerate(sop.terms):
        act = set()
        for m in t.target_leaves():
            act |= set(tree.path_to_root(m))
        for n in tree.nodes:
            if n.address in act:
                out[(l, n.address)] = acc
                acc += n.d_up * n.d_up
    return out


if __name__ == "__main__":
    print(build(fast=False), build(fast=True), file=sys.stderr)
