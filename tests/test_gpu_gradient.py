"""Energy gradient dE/dPhi^* through the C ABI (plans with QT_PLAN_GRADIENT),
on the 16-mode differentiation workload (p = 32, bond 32, 152 terms):
central finite differences (h = 1e-6) along random directions, consistency
with the sweep's own derivative at the top node, and a test-only
torch.autograd.Function around the library call."""
import numpy as np
import pytest

from qutree_gb300 import qtgpu
from qutree_gb300.model import config_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg4():
    return config_problem(4)


def _gradient(tree, sop, psi, prec, plan=qtgpu.QT_PLAN_GROUPED):
    h = qtgpu.HamiltonianRepresentation(sop, tree, flavour=plan | qtgpu.QT_PLAN_GRADIENT | prec)
    try:
        dpsi = qtgpu.Derivative(h, psi.flat())
        g = h.gradient()
        e = h.energy()
        h00, s00 = h.energy_parts()
        arena = h.stats()["arena_bytes"]
    finally:
        h.close()
    return g, dpsi, e, s00.real, arena


@pytest.mark.parametrize("plan,prec,n_dirs,tol", [
    (qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PREC_F64, 64, 1e-6), (qtgpu.QT_PLAN_GROUPED, qtgpu.QT_PREC_DF64, 16, 1e-6),
    (qtgpu.QT_PLAN_COMPRESSED, qtgpu.QT_PREC_F64, 32, 1e-6), (qtgpu.QT_PLAN_COMPRESSED, qtgpu.QT_PREC_DF64, 16, 1e-6),
    (qtgpu.QT_PLAN_COMPRESSED, qtgpu.QT_PREC_DF64_TC, 16, 1e-6)])
def test_gradient_matches_finite_differences(cfg4, plan, prec, n_dirs, tol):
    from tree_energy import energy, fd_directional
    tree, sop, psi = cfg4
    g, _, e, _, arena = _gradient(tree, sop, psi, prec, plan)
    assert abs(e - energy(tree, sop, psi.tensors)) <= 1e-11 * abs(e)
    assert arena < 2 << 30  # device arena of the gradient plan (bytes), stated in DESIGN
    rng = np.random.default_rng(1234)
    worst = 0.0
    for _ in range(n_dirs):
        dirs = [rng.standard_normal(n.shape) + 1j * rng.standard_normal(n.shape) for n in tree.nodes]
        flat = np.concatenate([d.ravel(order="F") for d in dirs])
        analytic = 2.0 * np.vdot(g, flat).real
        fd = fd_directional(tree, sop, psi, dirs, h=1e-6)
        worst = max(worst, abs(analytic - fd) / max(1.0, abs(fd)))
    assert worst <= tol, worst


def test_gradient_top_node_is_the_projected_apply(cfg4):
    # at the top, dE/dPhi^* * S00 = Apply(top) - E Phi_top = i dPsi_top - E Phi_top
    tree, sop, psi = cfg4
    g, dpsi, e, s00, _ = _gradient(tree, sop, psi, qtgpu.QT_PREC_F64)
    off = tree.offsets()
    t = tree.top.address
    seg = slice(off[t], off[t + 1])
    ref = 1j * dpsi[seg] - e * psi.flat()[seg]
    assert np.abs(g[seg] * s00 - ref).max() <= 1e-12 * np.abs(ref).max()


def test_autograd_function(cfg4):
    torch = pytest.importorskip("torch")
    tree, sop, psi = cfg4
    hrep = qtgpu.HamiltonianRepresentation(sop, tree, flavour=qtgpu.QT_PLAN_GROUPED | qtgpu.QT_PLAN_GRADIENT)

    class Energy(torch.autograd.Function):
        """E(Phi_1..Phi_n) by the library; backward returns the library's
        dE/dPhi^* in PyTorch's convention for a real loss (2 * dE/dz^*)."""

        @staticmethod
        def forward(ctx, *phis):
            flat = np.concatenate([p.detach().cpu().numpy().ravel(order="F") for p in phis])
            hrep.upload(flat)
            hrep.derivative()
            ctx.grad = hrep.gradient()
            ctx.shapes = [tuple(p.shape) for p in phis]
            return torch.tensor(hrep.energy(), dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            out, o = [], 0
            for shp in ctx.shapes:
                n = int(np.prod(shp))
                g = ctx.grad[o:o + n].reshape(shp, order="F")
                o += n
                out.append(torch.from_numpy(2.0 * g) * gout)
            return tuple(out)

    try:
        phis = [torch.from_numpy(np.asfortranarray(t)).requires_grad_(True) for t in psi.tensors]
        e = Energy.apply(*phis)
        e.backward()
        lib = hrep.gradient()
        got = np.concatenate([p.grad.numpy().ravel(order="F") for p in phis])
        assert np.allclose(got, 2.0 * lib, rtol=0, atol=1e-14 * np.abs(lib).max())
    finally:
        hrep.close()


def test_gradient_compressed_equals_grouped(cfg4):
    tree, sop, psi = cfg4
    g1 = _gradient(tree, sop, psi, qtgpu.QT_PREC_F64)[0]
    g2 = _gradient(tree, sop, psi, qtgpu.QT_PREC_F64, qtgpu.QT_PLAN_COMPRESSED)[0]
    assert np.abs(g2 - g1).max() <= 1e-12 * np.abs(g1).max()
