"""Shared comparison helpers of the test suite."""
import numpy as np


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / (s if s > 0 else 1.0))


def rho_weighted(tree, dpsi, rho):
    """dPsi of every non-top node multiplied back by its density matrix
    (C[r, m] = sum_n rho(m, n) dPsi[r, n]), undoing the regularised inverse
    whose conditioning amplifies rounding noise; the top node unchanged.
    Returns the concatenation in node order."""
    off = tree.offsets()
    ro = 0
    out = []
    for n in tree.nodes:
        d = n.d_up
        R = rho[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
        x = dpsi[off[n.address]:off[n.address + 1]].reshape((-1, d), order="F")
        out.append((x if n.is_top else x @ R.T).ravel(order="F"))
    return np.concatenate(out)


def rho_condition(tree, rho):
    ro = 0
    worst = 1.0
    for n in tree.nodes:
        d = n.d_up
        R = rho[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
        if n.is_top:
            continue
        w = np.linalg.eigvalsh(0.5 * (R + R.conj().T))
        worst = max(worst, w.max() / max(w.min(), 1e-300))
    return worst


def deriv_errors(tree, dpsi, ref, rho):
    """Compare derivatives node by node after multiplying each non-top node
    back by its density matrix (C[r, m] = sum_n rho(m, n) dPsi[r, n]).

    Returns (err, noise): err is the largest difference over nodes whose
    derivative is not identically zero, relative to the largest reference
    value; noise is the largest magnitude, relative to the same scale, on
    nodes whose SPFs span their whole space (lastBefore == d_up): there the
    projector (1-P) is zero and both derivatives are rounding noise of a
    cancellation."""
    off = tree.offsets()
    ro = 0
    scale = 0.0
    parts = []
    for n in tree.nodes:
        d = n.d_up
        R = rho[ro:ro + d * d].reshape((d, d), order="F")
        ro += d * d
        a = dpsi[off[n.address]:off[n.address + 1]].reshape((-1, d), order="F")
        b = ref[off[n.address]:off[n.address + 1]].reshape((-1, d), order="F")
        if not n.is_top:
            a, b = a @ R.T, b @ R.T
        degenerate = (not n.is_top) and n.size == d * d
        parts.append((degenerate, a, b))
        if not degenerate:
            scale = max(scale, float(np.abs(b).max()))
    scale = scale if scale > 0 else 1.0
    err = max((float(np.abs(a - b).max()) for dg, a, b in parts if not dg), default=0.0) / scale
    noise = max((max(float(np.abs(a).max()), float(np.abs(b).max())) for dg, a, b in parts if dg),
                default=0.0) / scale
    return err, noise


def cdvr_device_wsd(tree, arena, xtab, rho_nodes, rtol=1e-10):
    """Hook for the CDVR oracle's several-matrix grid solve: run the oracle's
    (bit-fixed) solver on the device's own inputs -- its X matrices (from
    the CDVR arena, offsets of plan table 39) and its density matrices -- after
    checking they agree with the oracle's to ``rtol``.  The solver's accept /
    reject steps make its output discontinuous in its inputs, so parity past
    the grid step is only meaningful on identical inputs."""
    import cdvr as C
    offs = {(int(m), int(a)): (int(xm), int(xr), int(xh)) for m, a, xm, xr, xh in xtab}
    f = tree.n_leaves
    calls = []

    def wsd(kind, a, xs, W):
        d = tree.nodes[a].d_up
        if kind == "grid":
            modes = sorted(tree.subtree_modes(a))
            src = [offs[(m, a)][0] for m in modes]
        else:
            modes = [m for m in range(f) if tree.leaf_node[m] != a]
            src = [offs[(m, a)][2] for m in modes]
        dev = [arena[o:o + d * d].reshape((d, d), order="F") for o in src]
        for x, y in zip(dev, xs):
            assert np.abs(x - y).max() <= rtol * max(np.abs(y).max(), 1e-300)
        Wd = rho_nodes[a]
        assert np.abs(Wd - W).max() <= rtol * np.abs(W).max()
        calls.append((kind, a))
        return C.layer_grid_multi(dev, Wd)
    wsd.calls = calls
    return wsd


def node_matrices(tree, flat):
    """Split a dense per-node matrix download (QT_MAT_RHO layout) into d x d blocks."""
    out, off = [], 0
    for n in tree.nodes:
        d = n.d_up
        out.append(flat[off:off + d * d].reshape((d, d), order="F"))
        off += d * d
    return out


def tree_overlap(tree, psi_a, psi_b):
    """<Psi_a|Psi_b> of two flat tensor trees (QuTree's dotProduct, bottom
    up: S_node = Phi_a^H (Phi_b with the children's S applied), the top's
    (0, 0) element); independent of the gauge of either tree."""
    off = tree.offsets()
    S = {}
    for n in tree.nodes:
        a = n.address
        shape = list(n.shape)
        A = psi_a[off[a]:off[a + 1]].reshape(shape, order="F")
        Bt = psi_b[off[a]:off[a + 1]].reshape(shape, order="F")
        for k, c in enumerate(n.children):
            Bt = np.moveaxis(np.tensordot(S[c], Bt, axes=([1], [k])), 0, k)
        d = shape[-1]
        S[a] = A.reshape((-1, d), order="F").conj().T @ Bt.reshape((-1, d), order="F")
    return S[tree.top.address][0, 0]
