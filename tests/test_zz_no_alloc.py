"""The allocation-free density inverse (qt_rho_inverse_noalloc) against the
density inverses the sweep computes (qt_derivative, QT_MAT_RHOINV).

Some callers cannot allocate device memory (stream capture, latency-bound
loops, pooled allocators); this entry point serves them with a static device
workspace.  It must reproduce the sweep's inverses and, up to the largest
bond it admits, numpy's eigendecomposition, on two calls in a row (the
second call finds the previous call's workspace contents), through the C
ABI.  Collected last on purpose: it runs after every other GPU test and
also passes alone in a fresh process."""
import numpy as np
import pytest

from helpers import rel_err, rho_condition
from qutree_gb300 import qtgpu
from qutree_gb300.model import config_problem

pytestmark = pytest.mark.gpu


def _by_dim(tree, flat):
    """{d: (node addresses, stacked d x d matrices)} of a per-node matrix set."""
    groups, ro = {}, 0
    for n in tree.nodes:
        d = n.d_up
        groups.setdefault(d, ([], []))
        groups[d][0].append(n.address)
        groups[d][1].append(flat[ro:ro + d * d])
        ro += d * d
    return {d: (a, np.concatenate(m)) for d, (a, m) in groups.items()}


@pytest.mark.parametrize("cfg", [0, 4])
def test_noalloc_inverse_matches_sweep(cfg):
    tree, sop, psi = config_problem(cfg)
    hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_GROUPED)
    try:
        qtgpu.Derivative(hrep, psi.flat())
        rho = hrep.matrices(qtgpu.QT_MAT_RHO)
        rhoinv = hrep.matrices(qtgpu.QT_MAT_RHOINV)
        cond = rho_condition(tree, rho)
        ctx = hrep.ctx
        want = _by_dim(tree, rhoinv)
        for d, (addrs, mats) in _by_dim(tree, rho).items():
            n = len(addrs)
            d_rho = ctx.to_device(mats)
            d_out = ctx.to_device(np.zeros_like(mats))
            try:
                for call in range(2):
                    ctx.rho_inverse_noalloc(d_out, d_rho, n, d, 1e-10)
                    got = ctx.from_device(d_out, mats.shape)
                    err = rel_err(got, want[d][1])
                    assert err <= 1e-13 * max(cond, 10.0), (d, call, err)
            finally:
                ctx.free(d_rho)
                ctx.free(d_out)
    finally:
        hrep.close()


def test_noalloc_rejects_oversize():
    ctx = qtgpu.Context(0)
    try:
        p = ctx.alloc(256)
        with pytest.raises(qtgpu.QtError, match="exceeds the static scratch"):
            ctx.rho_inverse_noalloc(p, p + 128, 1 << 10, 64)  # 1024 * 64 * 64 > 524288
        with pytest.raises(qtgpu.QtError, match="QT_ERR_SHAPE"):
            ctx.rho_inverse_noalloc(p, p + 128, 1, 113)
        ctx.free(p)
    finally:
        ctx.close()


def _regularised_inverse(rho, eps):
    """U diag(1/(w + eps exp(-w/eps))) U^dagger from numpy's eigh: the
    reference's regularised inverse (include/Core/Vector_Implementation.h:266-280,
    src/TreeClasses/SpectralDecompositionTree.cpp:30-48), computed
    independently of the library's eigensolver."""
    w, U = np.linalg.eigh(rho)
    f = 1.0 / (w + eps * np.exp(-w / eps))
    return (U * f) @ U.conj().T


def _hermitian(rng, d, w):
    q, _ = np.linalg.qr(rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)))
    m = (q * w) @ q.conj().T
    return 0.5 * (m + m.conj().T)


@pytest.mark.parametrize("d", [64, 96, 112])
def test_noalloc_inverse_largest_bonds_against_eigh(d):
    """Bonds up to the largest the entry point admits, as many matrices as the
    static workspace holds, against numpy's eigh.  Well-conditioned positive
    matrices take the factorisation shortcut; the last matrix of the batch
    is rank-deficient (two zero eigenvalues, far below 50 eps), which forces
    the Jacobi eigensolver whose eigenvectors live in the static workspace."""
    rng = np.random.default_rng(1000 + d)
    eps = 1e-10
    n = 524288 // (d * d)
    mats, want, tol = [], [], []
    for b in range(n):
        if b == n - 1:
            w = np.concatenate([np.zeros(2), 10.0 ** rng.uniform(-3, 0, d - 2)])
        else:
            w = 10.0 ** rng.uniform(-3, 0, d)
        m = _hermitian(rng, d, w)
        mats.append(m.ravel(order="F"))
        want.append(_regularised_inverse(m, eps).ravel(order="F"))
    mats = np.concatenate(mats)
    ctx = qtgpu.Context(0)
    try:
        d_rho = ctx.to_device(mats)
        d_out = ctx.to_device(np.zeros_like(mats))
        for call in range(2):
            ctx.rho_inverse_noalloc(d_out, d_rho, n, d, eps)
            got = ctx.from_device(d_out, mats.shape)
            for b in range(n):
                g = got[b * d * d:(b + 1) * d * d]
                # relative to the largest entry: 1e3 for the positive
                # matrices (condition 1e3), 1/eps for the rank-deficient one
                err = rel_err(g, want[b])
                assert err <= 1e-13 * 1e3 * d / 32, (d, call, b, err)
        ctx.free(d_rho)
        ctx.free(d_out)
    finally:
        ctx.close()


def test_noalloc_rejects_overlapping_ranges():
    ctx = qtgpu.Context(0)
    try:
        p = ctx.alloc(16 * 2 * 64 * 64)
        with pytest.raises(qtgpu.QtError, match="overlap"):
            ctx.rho_inverse_noalloc(p + 16 * 100, p, 1, 64)  # rhoinv starts inside rho
        ctx.free(p)
    finally:
        ctx.close()
