"""ctypes binding of libqtgpu.so and a host mirror of QuTree's sweep API.

The GPU library is the only compute path: if libqtgpu.so cannot be loaded or
no CUDA device is present, the calls raise; nothing falls back to the CPU.

QuTree names mirrored here (reference file:line):
  HamiltonianRepresentation(H, tree)  include/TreeClasses/HamiltonianRepresentation.h:17-45
  .build(H, Psi, tree, time)          include/TreeClasses/HamiltonianRepresentation.h:62-87
  Derivative(dPsi, hRep, t, Psi, H, tree, phase)
                                      src/TreeClasses/HamiltonianRepresentation.cpp:74-81
  Expectation(hRep, Psi, H, tree)     src/TreeClasses/HamiltonianRepresentation.cpp:45-51
  matrixTensor / contraction / multStateAB on device pointers
                                      include/Core/Tensor.h:231-329
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from .model import SOP, Tree, TensorTree

QT_OK = 0
QT_PLAN_REFERENCE = 0
QT_PLAN_GROUPED = 1
QT_PLAN_COMPRESSED = 2
QT_PREC_F64 = 0x000
QT_PREC_DF64 = 0x100
QT_PREC_DF64_TC = 0x200
QT_PREC_C32 = 0x400
QT_PREC_TF32X3 = 0x800
QT_PLAN_GRADIENT = 0x1000
QT_PLAN_SCF = 0x2000
QT_PLAN_CDVR = 0x4000
QT_MAT_RHO, QT_MAT_RHOINV, QT_MAT_HMAT, QT_MAT_HCON, QT_MAT_CDVR = 0, 1, 2, 3, 4
QT_CDVR_ALIGNED_HOLE_GRIDS = 1
ERRORS = {1: "QT_ERR_ARG", 2: "QT_ERR_SHAPE", 3: "QT_ERR_ALLOC", 4: "QT_ERR_CUDA",
          5: "QT_ERR_STATE", 6: "QT_ERR_NUMERIC", 7: "QT_ERR_TIMEOUT"}

_lib = None
_P = np.ctypeslib.ndpointer
_i32 = _P(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = _P(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p


class QtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libqtgpu.so (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build._stale(path)):
        _build.build()
    L = ctypes.CDLL(path)
    sig = {
        "qt_ctx_create": ([ctypes.POINTER(_vp), ctypes.c_int], ctypes.c_int),
        "qt_ctx_destroy": ([_vp], None),
        "qt_last_error": ([_vp], ctypes.c_char_p),
        "qt_sync": ([_vp], ctypes.c_int),
        "qt_get_stream": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
        "qt_tree_upload": ([_vp, ctypes.c_int, _i32, _i32, _i32, _i32, _i32], ctypes.c_int),
        "qt_sop_upload": ([_vp, ctypes.c_int, _i32, _i32, _i64, _vp, ctypes.c_int, _vp, _i32, _i32,
                           _i32], ctypes.c_int),
        "qt_set_regularization": ([_vp, ctypes.c_double], ctypes.c_int),
        "qt_prepare": ([_vp, ctypes.c_int], ctypes.c_int),
        "qt_psi_upload": ([_vp, _vp], ctypes.c_int),
        "qt_psi_upload_device": ([_vp, _vp], ctypes.c_int),
        "qt_psi_download": ([_vp, _vp], ctypes.c_int),
        "qt_psi_size": ([_vp], ctypes.c_int64),
        "qt_derivative": ([_vp, ctypes.c_double, ctypes.c_double], ctypes.c_int),
        "qt_dpsi_download": ([_vp, _vp], ctypes.c_int),
        "qt_dpsi_device": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
        "qt_energy": ([_vp, _vp], ctypes.c_int),
        "qt_matrices_size": ([_vp, ctypes.c_int], ctypes.c_int64),
        "qt_matrices_download": ([_vp, ctypes.c_int, _vp], ctypes.c_int),
        "qt_plan_stats": ([_vp, _vp], ctypes.c_int),
        "qt_mode_product": ([_vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                             ctypes.c_int64, ctypes.c_int], ctypes.c_int),
        "qt_hole_product": ([_vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                             ctypes.c_int64], ctypes.c_int),
        "qt_last_mode_product": ([_vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int],
                                 ctypes.c_int),
        "qt_dev_alloc": ([_vp, ctypes.c_int64, ctypes.POINTER(_vp)], ctypes.c_int),
        "qt_dev_free": ([_vp, _vp], ctypes.c_int),
        "qt_memcpy_h2d": ([_vp, _vp, _vp, ctypes.c_int64], ctypes.c_int),
        "qt_memcpy_d2h": ([_vp, _vp, _vp, ctypes.c_int64], ctypes.c_int),
        "qt_launch_count": ([_vp], ctypes.c_int64),
        "qt_stage_count": ([_vp], ctypes.c_int),
        "qt_stage_info": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "qt_stage_launch": ([_vp, ctypes.c_int], ctypes.c_int),
        "qt_probe_fp64_peak": ([_vp, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "qt_probe_df64_peak": ([_vp, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "qt_qr_orthogonal": ([_vp], ctypes.c_int),
        "qt_set_tc_thresholds": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "qt_rho_inverse_noalloc": ([_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_double],
                                   ctypes.c_int),
        "qt_tree_count": ([_vp], ctypes.c_int),
        "qt_gradient_download": ([_vp, _vp], ctypes.c_int),
        "qt_psi_save": ([_vp, ctypes.c_char_p], ctypes.c_int),
        "qt_build": ([_vp], ctypes.c_int),
        "qt_layer_derivatives": ([_vp, ctypes.c_double, ctypes.c_double], ctypes.c_int),
        "qt_cmf_propagate": ([_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                              ctypes.c_double], ctypes.c_int),
        "qt_psi_load": ([_vp, ctypes.c_char_p], ctypes.c_int),
        "qt_energies": ([_vp, _vp, ctypes.c_int], ctypes.c_int),
        "qt_scf": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, _vp, ctypes.c_int64,
                    ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "qt_cdvr_upload": ([_vp, ctypes.c_int, _i32, _vp, ctypes.c_int, _vp, _i32, _i32, _i32,
                            ctypes.c_int], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def exported_symbols():
    """Names declared in include/qtgpu.h (the C ABI surface)."""
    return [
        "qt_ctx_create", "qt_ctx_destroy", "qt_last_error", "qt_sync", "qt_get_stream",
        "qt_tree_upload", "qt_sop_upload", "qt_set_regularization", "qt_prepare",
        "qt_psi_upload", "qt_psi_upload_device", "qt_psi_download", "qt_psi_size",
        "qt_derivative", "qt_dpsi_download", "qt_dpsi_device", "qt_energy",
        "qt_matrices_size", "qt_matrices_download", "qt_plan_stats", "qt_mode_product",
        "qt_hole_product", "qt_last_mode_product", "qt_dev_alloc", "qt_dev_free",
        "qt_memcpy_h2d", "qt_memcpy_d2h", "qt_launch_count", "qt_stage_count",
        "qt_stage_info", "qt_stage_launch", "qt_probe_fp64_peak", "qt_rho_inverse_noalloc",
        "qt_tree_count", "qt_energies", "qt_gradient_download", "qt_psi_save", "qt_psi_load",
        "qt_build", "qt_layer_derivatives", "qt_cmf_propagate", "qt_scf", "qt_probe_df64_peak",
        "qt_cdvr_upload", "qt_qr_orthogonal", "qt_set_tc_thresholds",
    ]


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class Context:
    """One libqtgpu context (one device, one stream, one device arena)."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = _vp()
        rc = self.L.qt_ctx_create(ctypes.byref(h), device)
        if rc != QT_OK:
            raise QtError(rc, self.L.qt_last_error(None).decode())
        self.h = h

    def check(self, rc):
        if rc != QT_OK:
            raise QtError(rc, self.L.qt_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.qt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- device memory helpers -------------------------------------------
    def alloc(self, nbytes: int) -> int:
        p = _vp()
        self.check(self.L.qt_dev_alloc(self.h, int(nbytes), ctypes.byref(p)))
        return p.value

    def free(self, p: int):
        self.check(self.L.qt_dev_free(self.h, _vp(p)))

    def to_device(self, a: np.ndarray) -> int:
        a = np.ascontiguousarray(a)
        p = self.alloc(max(a.nbytes, 16))
        self.check(self.L.qt_memcpy_h2d(self.h, _vp(p), _ptr(a), a.nbytes))
        return p

    def from_device(self, p: int, shape, dtype=np.complex128) -> np.ndarray:
        out = np.zeros(shape, dtype=dtype)
        self.check(self.L.qt_memcpy_d2h(self.h, _ptr(out), _vp(p), out.nbytes))
        return out

    def sync(self):
        self.check(self.L.qt_sync(self.h))

    def launch_count(self) -> int:
        return int(self.L.qt_launch_count(self.h))

    def fp64_peak(self) -> float:
        v = ctypes.c_double()
        self.check(self.L.qt_probe_fp64_peak(self.h, ctypes.byref(v)))
        return v.value

    def df64_peak(self) -> float:
        v = ctypes.c_double()
        self.check(self.L.qt_probe_df64_peak(self.h, ctypes.byref(v)))
        return v.value

    # -- primitives (device pointers) ------------------------------------
    def rho_inverse_noalloc(self, rhoinv, rho, n_mats, d, eps=1e-10):
        """Regularised inverses of n_mats Hermitian d x d device matrices; the
        library allocates nothing (its workspace is a static device array)."""
        self.check(self.L.qt_rho_inverse_noalloc(self.h, _vp(rhoinv), _vp(rho), n_mats, d, eps))

    def mode_product(self, C, h, B, before, activeB, activeC, after, add=False):
        self.check(self.L.qt_mode_product(self.h, _vp(C), _vp(h), _vp(B), before, activeB, activeC,
                                          after, int(add)))

    def hole_product(self, S, A, B, before, activeA, activeB, after):
        self.check(self.L.qt_hole_product(self.h, _vp(S), _vp(A), _vp(B), before, activeA, activeB,
                                          after))

    def last_mode_product(self, C, A, B, last_before, active, add=False):
        self.check(self.L.qt_last_mode_product(self.h, _vp(C), _vp(A), _vp(B), last_before, active,
                                               int(add)))


class HamiltonianRepresentation:
    """Device-resident sweep state of one tree and one SOP operator: the
    GPU counterpart of QuTree's HamiltonianRepresentation together with the
    wavefunction it acts on."""

    def __init__(self, H: SOP, tree: Tree, flavour: int = QT_PLAN_REFERENCE, eps: float = 1e-10,
                 device: int = 0, ctx: Context | None = None, potential=None, leaf_x=None,
                 aligned_hole_grids: bool = False, tc_thresholds=None):
        """potential (a PolyPotential) with leaf_x (mode -> DVR grid points):
        the Hamiltonian also has that potential, applied by CDVR.
        tc_thresholds: (mp, hp, acc) lower bounds of the shapes put on the
        tensor cores, or "auto" for the bounds the autotuner cached for this
        device (qutree_gb300.autotune; the built-in bounds when none is
        cached); None keeps the built-in bounds."""
        if potential is not None:
            flavour |= QT_PLAN_CDVR
        self.tree, self.H, self.flavour = tree, H, flavour
        self.ctx = ctx or Context(device)
        L, h = self.ctx.L, self.ctx.h
        order, dims, parent, child_idx, leaf_mode = tree.descriptor()
        self.ctx.check(L.qt_tree_upload(h, tree.n_nodes, order, dims, parent, child_idx, leaf_mode))
        kind, odim, ooff, odata = H.ops.descriptor()
        coeff, ptr, modes, opids = H.descriptor()
        self._keep = (odata, coeff)
        self.ctx.check(L.qt_sop_upload(h, len(kind), kind, odim, ooff, _ptr(odata), len(H),
                                       _ptr(coeff), ptr, modes, opids))
        self.ctx.check(L.qt_set_regularization(h, eps))
        if tc_thresholds == "auto":
            from . import autotune
            tc_thresholds = autotune.cached(device)
        if tc_thresholds is not None:
            self.ctx.check(L.qt_set_tc_thresholds(h, *(int(v) for v in tc_thresholds)))
        if potential is not None:
            f = tree.n_leaves
            ldim = np.array([len(leaf_x[m]) for m in range(f)], dtype=np.int32)
            lx = np.ascontiguousarray(np.concatenate([np.asarray(leaf_x[m], float) for m in range(f)]))
            pc, pp, pm, pw = potential.descriptor()
            pc = np.ascontiguousarray(pc)
            self._keep_pot = (lx, pc)
            self.ctx.check(L.qt_cdvr_upload(h, f, ldim, _ptr(lx), len(pc), _ptr(pc), pp, pm, pw,
                                            QT_CDVR_ALIGNED_HOLE_GRIDS if aligned_hole_grids else 0))
        self.ctx.check(L.qt_prepare(h, flavour))
        self.n_psi = int(L.qt_psi_size(h))

    # -- wavefunction ----------------------------------------------------
    def upload(self, psi):
        flat = psi.flat() if isinstance(psi, TensorTree) else np.ascontiguousarray(psi, np.complex128)
        assert flat.size == self.n_psi
        self.ctx.check(self.ctx.L.qt_psi_upload(self.ctx.h, _ptr(flat)))

    def save(self, path: str):
        """Write the device wavefunction as a QuTree TTre file."""
        self.ctx.check(self.ctx.L.qt_psi_save(self.ctx.h, path.encode()))

    def load(self, path: str):
        """Upload a QuTree TTre file (shapes checked against the tree)."""
        self.ctx.check(self.ctx.L.qt_psi_load(self.ctx.h, path.encode()))

    def upload_device(self, ptr: int):
        self.ctx.check(self.ctx.L.qt_psi_upload_device(self.ctx.h, _vp(ptr)))

    # -- sweep -------------------------------------------------------------
    def derivative(self, phase: complex = 1.0):
        self.ctx.check(self.ctx.L.qt_derivative(self.ctx.h, complex(phase).real, complex(phase).imag))

    def build(self):
        """HamiltonianRepresentation::build for the current Psi."""
        self.ctx.check(self.ctx.L.qt_build(self.ctx.h))

    def layer_derivatives(self, phase: complex = 1.0):
        """LayerDerivative at every node with the matrices of the last build frozen."""
        self.ctx.check(self.ctx.L.qt_layer_derivatives(self.ctx.h, complex(phase).real,
                                                       complex(phase).imag))

    def cmf(self, dt: float, n_steps: int, n_sub: int = 1, phase: complex = 1.0):
        """Fixed-step constant-mean-field propagation of the device wavefunction."""
        self.ctx.check(self.ctx.L.qt_cmf_propagate(self.ctx.h, dt, n_steps, n_sub,
                                                   complex(phase).real, complex(phase).imag))

    def scf(self, n_iter: int = 1, n_krylov: int = 5, n_itp: int = 0, beta: float = 1.0) -> np.ndarray:
        """QuTree's SCF / Krylov sweep on the device wavefunction (plans with
        QT_PLAN_COMPRESSED | QT_PLAN_SCF); returns the lowest Ritz value of every
        Krylov solve.  The optimised wavefunction stays on the device (psi())."""
        n_nodes = len(self.tree.nodes)
        cap = max(1, n_iter * (2 * n_nodes - 1))
        out = np.zeros(cap, dtype=np.float64)
        cnt = ctypes.c_int64(0)
        self.ctx.check(self.ctx.L.qt_scf(self.ctx.h, n_iter, n_krylov, n_itp, beta, _ptr(out), cap,
                                         ctypes.byref(cnt)))
        return out[:cnt.value].copy()

    def qr_orthogonal(self):
        """qrOrthogonal on the uploaded wavefunction, on the device (qt_qr_orthogonal)."""
        self.ctx.check(self.ctx.L.qt_qr_orthogonal(self.ctx.h))

    def psi(self) -> np.ndarray:
        out = np.zeros(self.n_psi, dtype=np.complex128)
        self.ctx.check(self.ctx.L.qt_psi_download(self.ctx.h, _ptr(out)))
        return out

    def dpsi(self) -> np.ndarray:
        out = np.zeros(self.n_psi, dtype=np.complex128)
        self.ctx.check(self.ctx.L.qt_dpsi_download(self.ctx.h, _ptr(out)))
        return out

    def gradient(self) -> np.ndarray:
        """dE/dPhi^* of the last sweep (plans with QT_PLAN_GRADIENT)."""
        out = np.zeros(self.n_psi, dtype=np.complex128)
        self.ctx.check(self.ctx.L.qt_gradient_download(self.ctx.h, _ptr(out)))
        return out

    def dpsi_into(self, out: np.ndarray):
        self.ctx.check(self.ctx.L.qt_dpsi_download(self.ctx.h, _ptr(out)))

    def dpsi_device(self) -> int:
        p = _vp()
        self.ctx.check(self.ctx.L.qt_dpsi_device(self.ctx.h, ctypes.byref(p)))
        return p.value

    def energy_parts(self):
        out = np.zeros(4)
        self.ctx.check(self.ctx.L.qt_energy(self.ctx.h, _ptr(out)))
        return complex(out[0], out[1]), complex(out[2], out[3])

    def energy(self) -> float:
        h00, s00 = self.energy_parts()
        return h00.real / s00.real

    def energies(self) -> np.ndarray:
        """Energy of every tree of a forest (roots in ascending address order)."""
        nt = int(self.ctx.L.qt_tree_count(self.ctx.h))
        out = np.zeros(4 * nt)
        self.ctx.check(self.ctx.L.qt_energies(self.ctx.h, _ptr(out), nt))
        o = out.reshape(nt, 4)
        return o[:, 0] / o[:, 2]

    def matrices(self, which: int) -> np.ndarray:
        n = int(self.ctx.L.qt_matrices_size(self.ctx.h, which))
        out = np.zeros(n, dtype=np.complex128)
        self.ctx.check(self.ctx.L.qt_matrices_download(self.ctx.h, which, _ptr(out)))
        return out

    def stats(self) -> dict:
        out = np.zeros(8)
        self.ctx.check(self.ctx.L.qt_plan_stats(self.ctx.h, _ptr(out)))
        keys = ["ref_flops", "exec_flops", "launches", "arena_bytes", "scratch_bytes",
                "rep_chains", "mf_chains", "app_chains"]
        return dict(zip(keys, out.tolist()))

    def sync(self):
        self.ctx.sync()

    def close(self):
        self.ctx.close()

    # -- profiling -----------------------------------------------------------
    def stages(self):
        """[(kind, tiles, flops, bytes)] of the prepared sweep's launches."""
        L, h = self.ctx.L, self.ctx.h
        out = []
        for i in range(int(L.qt_stage_count(h))):
            k, t, f, b = ctypes.c_int(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
            self.ctx.check(L.qt_stage_info(h, i, ctypes.byref(k), ctypes.byref(t), ctypes.byref(f),
                                           ctypes.byref(b)))
            out.append((k.value, t.value, f.value, b.value))
        return out

    def launch_stage(self, i: int):
        self.ctx.check(self.ctx.L.qt_stage_launch(self.ctx.h, i))

    def stream(self) -> int:
        p = _vp()
        self.ctx.check(self.ctx.L.qt_get_stream(self.ctx.h, ctypes.byref(p)))
        return p.value or 0


def Derivative(hrep: HamiltonianRepresentation, psi, phase: complex = 1.0) -> np.ndarray:
    """dPsi of one full sweep (build + LayerDerivative at every node)."""
    hrep.upload(psi)
    hrep.derivative(phase)
    return hrep.dpsi()


def Expectation(hrep: HamiltonianRepresentation) -> complex:
    """<Phi_top| H |Phi_top> of the last sweep (1x1 for a single state)."""
    h00, _ = hrep.energy_parts()
    return h00
